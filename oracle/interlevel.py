"""FP64 numpy restatement of the D3Q27 coarse-fine transfer (test
infrastructure: the checker of the library's explosion and coalescence).

explosion (interlevel_interpolation.f95:161-257, amrex_interp_node_bilinear,
ratio 2): a fine node at fine coordinates X takes the mean of the coarse nodes
floor(X/2) .. floor(X/2) + (X odd) on every axis (1, 2, 4 or 8 nodes, summed
z-, y-, x-major in that order); a negative or NaN population sends the node to
the entropic equilibrium of the interpolated density and velocity.
coalescence (fine_to_coarse.f95:30-64, amrex_average_down_nodes): a coarse
node at C takes the populations of the fine node at 2C.
"""
from __future__ import annotations

import numpy as np

from .oracle import equilibrium  # entropic D3Q27 equilibrium (rho, u) -> f

# D3Q27 velocities in the reference's order (linking/modules/linkwise.f95:25-32)
CX = np.array([0, 1, 0, 0, -1, 0, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, 1, 1, -1, -1, -1, -1])
CY = np.array([0, 0, 1, 0, 0, -1, 0, 1, 1, 1, 1, 0, 0, 0, 0, -1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1])
CZ = np.array([0, 0, 0, 1, 0, 0, -1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, -1, 1, -1, 1, -1, 1, -1])


def _coarse_nodes(X):
    lo = X // 2
    return [lo, lo + 1] if X % 2 else [lo]


def explode(coarse_f, coarse_lo, fine_f, fine_lo, ghost_mask):
    """coarse_f, fine_f: (27, nz, ny, nx) box arrays (fine_f is updated in place
    at the ghost nodes); *_lo: global (x, y, z) of the boxes' first node."""
    repaired = 0
    cx0, cy0, cz0 = coarse_lo
    for z, y, x in zip(*np.nonzero(ghost_mask)):
        X, Y, Z = fine_lo[0] + x, fine_lo[1] + y, fine_lo[2] + z
        acc = np.zeros(27)
        k = 0
        for cz in _coarse_nodes(Z):
            for cy in _coarse_nodes(Y):
                for cx in _coarse_nodes(X):
                    acc = acc + coarse_f[:, cz - cz0, cy - cy0, cx - cx0]
                    k += 1
        f = acc * (1.0 / k)
        if not np.all(f >= 0.0):
            rho = f.sum()
            u = np.array([(CX * f).sum(), (CY * f).sum(), (CZ * f).sum()]) / rho
            f = equilibrium(rho, u)
            repaired += 1
        fine_f[:, z, y, x] = f
    return repaired


def average_down(fine_f, fine_lo, fine_valid, coarse_f, coarse_lo, coarse_fluid):
    """Coarse nodes C with a valid fine node at 2C take its populations (in place)."""
    fx0, fy0, fz0 = fine_lo
    _, nz, ny, nx = fine_f.shape
    for z, y, x in zip(*np.nonzero(coarse_fluid)):
        X, Y, Z = 2 * (coarse_lo[0] + x) - fx0, 2 * (coarse_lo[1] + y) - fy0, 2 * (coarse_lo[2] + z) - fz0
        if 0 <= X < nx and 0 <= Y < ny and 0 <= Z < nz and fine_valid[Z, Y, X]:
            coarse_f[:, z, y, x] = fine_f[:, Z, Y, X]
