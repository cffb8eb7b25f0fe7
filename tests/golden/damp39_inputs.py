"""Seeded inputs of the D3Q39 negative-population repair cases (damp_it.f95),
shared by the golden generator and the test: 12 x 11 x 11 boxes (one at lo =
(0, 12, 3), where the shifted band test's comparison of the x index with
lo(2) matters, one at the origin), positive populations with 3% or 15%
negative ones, and link codes drawn from interior, boundary and wall codes on
both sides of the -500 threshold.  The legacy RandomState stream is
frozen across numpy versions, so the inputs are the same wherever they are
rebuilt."""
import numpy as np

NX, NY, NZ = 12, 11, 11
# name: (shifted lattice, the box's lo, fraction of negative populations, seed, region);
# the "shifted_core" box sits at the origin, where the band test leaves the corner
# x < 5, y < 4, z < 4 to the neighbour rules, and only that corner holds negative
# populations (30% of them, to cover every branch of those rules)
CASES = {"shifted": (True, (0, 12, 3), 0.03, 7321, None), "unshifted": (False, (0, 12, 3), 0.03, 7322, None),
         "shifted_core": (True, (0, 0, 0), 0.3, 7323, (5, 4, 4))}


def bounds(name):
    lo = CASES[name][1]
    return lo, (lo[0] + NX - 1, lo[1] + NY - 1, lo[2] + NZ - 1)
# interior (>= 0), coarse-fine and outflow node codes, boundary codes above and
# below -500 (bounce-back -10, inviscid -11, inlet -101, outlet -201, shifted
# inlet -301, null -666, freestream -1000) and packed wall links
CODES = np.array([0, 0, 0, 0, 1, 2, 1500, 250, -10, -11, -101, -201, -301, -666, -1000, -1001 - 250000000,
                  -1001 - 730000000], np.int64)


def _pops(rs, frac, region):
    fs = 0.02 + 0.08 * rs.random_sample(39)
    pop = 0.01 + 0.1 * rs.random_sample((39, NZ, NY, NX))
    neg = rs.random_sample((39, NZ, NY, NX)) < frac
    if region is not None:
        inside = np.zeros((NZ, NY, NX), bool)
        inside[:region[2], :region[1], :region[0]] = True
        neg &= inside[None]
    pop[neg] = -0.05 * rs.random_sample(int(neg.sum()))
    return pop, fs


def case(name: str):
    """(fout, gout, state, fs_f, fs_g): populations (39, nz, ny, nx), link codes, and
    the freestream equilibria that stand outside the box."""
    _, _, frac, seed, region = CASES[name]
    rs = np.random.RandomState(seed)
    fout, fs_f = _pops(rs, frac, region)
    gout, fs_g = _pops(rs, frac, region)
    state = CODES[rs.randint(0, len(CODES), size=(39, NZ, NY, NX))].astype(np.int32)
    return fout, gout, state, fs_f, fs_g
