"""FP64 numpy restatement of the negative-population repair for D3Q27
(damp_it.f95:64-177, unshifted lattice; test infrastructure).  Neighbours are
read from the unrepaired field.  Link codes: state[i][x] >= 0 means the link
from x along c_i joins two fluid nodes."""
from __future__ import annotations

import numpy as np

from .interlevel import CX, CY, CZ

OPP = [int(np.where((CX == -CX[i]) & (CY == -CY[i]) & (CZ == -CZ[i]))[0][0]) for i in range(27)]


def _fluid(s0):
    return s0 >= 0 and not (1000 <= s0 < 51000) and not (200 <= s0 < 299)


def damp(state, f):
    """Return (repaired copy of f, number of populations changed); state, f: (27, nz, ny, nx)."""
    out = f.copy()
    count = 0
    for i, z, y, x in zip(*np.nonzero(f < 0.0)):
        if not _fluid(state[0, z, y, x]):
            continue
        count += 1
        v = f[i, z, y, x]
        av = abs(v)
        plus = state[i, z, y, x] >= 0
        minus = state[OPP[i], z, y, x] >= 0
        fp = f[i, z + CZ[i], y + CY[i], x + CX[i]] if plus else None
        fm = f[i, z - CZ[i], y - CY[i], x - CX[i]] if minus else None
        r = av
        if plus and minus:
            if fp > 0.0 and fm > 0.0:
                r = (fp + fm) / 2.0
            elif fp > 0.0 and fm < 0.0:
                r = (fp + av) / 2.0
            elif fp < 0.0 and fm > 0.0:
                r = (fm + av) / 2.0
        elif plus:
            if fp > 0.0:
                r = (fp + av) / 2.0
        elif minus:
            if fm > 0.0:
                r = (fm + av) / 2.0
        out[i, z, y, x] = r
    return out, count
