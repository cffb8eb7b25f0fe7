"""FP64 numpy restatement of the coarse-fine transfer (test infrastructure:
the checker of the library's explosion and coalescence).

D3Q27:
explosion (interlevel_interpolation.f95:161-257, amrex_interp_node_bilinear,
ratio 2): a fine node at fine coordinates X takes the mean of the coarse nodes
floor(X/2) .. floor(X/2) + (X odd) on every axis (1, 2, 4 or 8 nodes, summed
z-, y-, x-major in that order); a negative or NaN population sends the node to
the entropic equilibrium of the interpolated density and velocity.
coalescence (fine_to_coarse.f95:30-64, amrex_average_down_nodes): a coarse
node at C takes the populations of the fine node at 2C.

D3Q39 (explode39 / average_down39): the same nodal means of f, g, the 13
multipliers, rho and T, then per node interlevel_interpolation.f95:364-440
(the C oracle's o39_explode_node); coalescence injects f, g, multipliers, w,
alpha and the five fields (fine_to_coarse.f95:13-45).
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


def _mean(arr, X, Y, Z, lo):
    """Nodal mean of arr[..., z, y, x] over the coarse nodes around fine (X, Y, Z),
    summed z-, y-, x-major, then times 1/k."""
    acc = None
    k = 0
    for cz in _coarse_nodes(Z):
        for cy in _coarse_nodes(Y):
            for cx in _coarse_nodes(X):
                v = arr[..., cz - lo[2], cy - lo[1], cx - lo[0]]
                acc = v.copy() if acc is None else acc + v
                k += 1
    return acc * (1.0 / k)


def explode39(k, step, coarse, coarse_lo, fine, fine_lo, ghost_mask):
    """coarse, fine: dicts of box arrays f, g (39, nz, ny, nx), lm (13, ...),
    w (nz, ny, nx), alpha (nz, ny, nx), macro (5, ...); fine is updated in place
    at its ghost nodes.  Returns (ghost nodes with a replaced population,
    capped multiplier solves)."""
    from . import oracle39 as o39
    repaired = capped = 0
    for z, y, x in zip(*np.nonzero(ghost_mask)):
        X, Y, Z = fine_lo[0] + x, fine_lo[1] + y, fine_lo[2] + z
        f = _mean(coarse["f"], X, Y, Z, coarse_lo)
        g = _mean(coarse["g"], X, Y, Z, coarse_lo)
        lm = _mean(coarse["lm"], X, Y, Z, coarse_lo)
        mc = _mean(coarse["macro"], X, Y, Z, coarse_lo)
        f, g, lm, m5, a, flags = o39.explode_node(k, step, f, g, lm, mc[0], mc[4])
        fine["f"][:, z, y, x] = f
        fine["g"][:, z, y, x] = g
        fine["lm"][:, z, y, x] = lm
        fine["w"][z, y, x] = m5[3]
        fine["alpha"][z, y, x] = a
        fine["macro"][:, z, y, x] = m5
        repaired += flags & 1
        capped += (flags >> 1) & 1
    return repaired, capped


def average_down39(fine, fine_lo, fine_valid, coarse, coarse_lo, coarse_fluid):
    """Coarse nodes C with a valid fine node at 2C take every per-node array of it (in place)."""
    fx0, fy0, fz0 = fine_lo
    nz, ny, nx = fine["w"].shape
    for z, y, x in zip(*np.nonzero(coarse_fluid)):
        X, Y, Z = 2 * (coarse_lo[0] + x) - fx0, 2 * (coarse_lo[1] + y) - fy0, 2 * (coarse_lo[2] + z) - fz0
        if 0 <= X < nx and 0 <= Y < ny and 0 <= Z < nz and fine_valid[Z, Y, X]:
            for key in ("f", "g", "lm", "w", "alpha", "macro"):
                coarse[key][..., z, y, x] = fine[key][..., Z, Y, X]
