"""Host-side lattice tables and equilibria (numpy).

D3Q27 ordering: the reference's linking/modules/linkwise.f95:25-32 (cx_27 ... opp_27),
0-based here.  The equilibrium is the D3Q27 entropic equilibrium (a product of
D1Q3 factors, Ansumali, Karlin, Oettinger 2003) at T0 = 1/3; the reference computes its
boundary equilibria once on the host (boundary_conditions/basic_calcs/
freestream_basis_calcs.f90:33-71), and so does this module for D3Q27.
"""
from __future__ import annotations

import numpy as np

Q27 = 27
CX = np.array([0, 1, 0, 0, -1, 0, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, 1, 1, -1, -1, -1, -1], np.int64)
CY = np.array([0, 0, 1, 0, 0, -1, 0, 1, 1, 1, 1, 0, 0, 0, 0, -1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1], np.int64)
CZ = np.array([0, 0, 0, 1, 0, 0, -1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, -1, 1, -1, 1, -1, 1, -1], np.int64)
OPP = np.array([0, 4, 5, 6, 1, 2, 3, 17, 18, 15, 16, 13, 14, 11, 12, 9, 10, 7, 8, 26, 25, 24, 23, 22, 21, 20, 19],
               np.int64)
C = np.stack([CX, CY, CZ], axis=1)
T0 = 1.0 / 3.0


def _w1(c):
    return np.where(c == 0, 2.0 / 3.0, 1.0 / 6.0)


W = _w1(CX) * _w1(CY) * _w1(CZ)


def equilibrium27(rho, u):
    """D3Q27 entropic equilibrium.  rho: (...), u: (..., 3) -> (27, ...).

    The minimiser of H = sum f ln(f/w) at fixed rho and j (Ansumali, Karlin,
    Oettinger 2003), a product over the axes of the D1Q3 solution:
    f_i = rho * prod_a w1(c_ia) psi(u_a) zeta(u_a)^c_ia,
    psi(u) = 2 - sqrt(1 + 3u^2), zeta(u) = (2u + sqrt(1 + 3u^2)) / (1 - u).
    """
    rho = np.asarray(rho, np.float64)
    u = np.asarray(u, np.float64)
    g = []
    for a in range(3):
        ua = u[..., a]
        s = np.sqrt(1.0 + 3.0 * ua * ua)
        psi = 2.0 - s
        zeta = (2.0 * ua + s) / (1.0 - ua)
        g.append({-1: psi / zeta / 6.0, 0: psi * 2.0 / 3.0, 1: psi * zeta / 6.0})
    shape = np.broadcast_shapes(rho.shape, u.shape[:-1])
    out = np.empty((Q27,) + shape, np.float64)
    for i in range(Q27):
        out[i] = rho * g[0][int(CX[i])] * g[1][int(CY[i])] * g[2][int(CZ[i])]
    return out


def moments27(f):
    """rho, u of populations f with shape (27, ...)."""
    rho = f.sum(axis=0)
    u = np.stack([np.tensordot(CX.astype(np.float64), f, axes=(0, 0)),
                  np.tensordot(CY.astype(np.float64), f, axes=(0, 0)),
                  np.tensordot(CZ.astype(np.float64), f, axes=(0, 0))], axis=-1) / rho[..., None]
    return rho, u


def beta_from_nu(nu: float) -> float:
    """beta = 1/(2 tau), tau = nu/T0 + 1/2 (dt = 1)."""
    return 1.0 / (2.0 * nu / T0 + 1.0)
