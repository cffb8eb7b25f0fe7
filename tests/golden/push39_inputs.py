"""Seeded inputs of the D3Q39 push-loop cases (streaming.f95 with boundary
links, no interpolated wall links), shared by the golden generator and the
test: a 14 x 6 x 7 box with an inlet (-101) at x-, an outlet (-201, of the
case's type) at x+, a bounce-back floor (-10), a freestream top (-1000), and
either a periodic span or inviscid side walls (-11); two solid nodes whose
fluid neighbours bounce back towards them (-10) and one null link (-666).
Populations, the previous step's post-streaming values and the boundary
equilibria are seeded positive numbers: the push loop only moves, swaps and
copies them.  The legacy RandomState stream is frozen across numpy versions."""
import numpy as np

NX, NY, NZ = 14, 6, 7
# name: (shifted lattice, outlet type, side-face code (0: periodic span), seed).  A
# shifted box with a periodic span is left out: there the reference's pushes across
# the periodic face come from ghost images swept before the face's first layer, so an
# outlet link at the face writes its slot after them, while the library's single array
# lets the wrapped node push later in the sweep (a documented difference at the
# corners where an outlet face meets a periodic one).
CASES = {"unshifted_outflow": (0, 6, 0, 11), "unshifted_rho_v": (0, 1, 0, 12), "unshifted_inviscid": (0, 6, -11, 15),
         "shifted_inviscid": (1, 1, -11, 16), "shifted_inviscid_press_temp": (1, 2, -11, 17)}


def case(name: str, s39):
    """dict of the case: state (39, nz, ny, nx), fout, gout, prev_f, prev_g, the
    equilibrium tables ff, gf (freestream), fi, gi (inlets), fo, go (outlets),
    inlet and outlet types, periodic flags, shifted.  s39: the package's
    d3q39_setup (box_state39, lattice39)."""
    shifted, outlet_type, side, seed = CASES[name]
    periodic = 2 if side == 0 else 0
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": side, "y+": side}
    prio = ("x-", "x+", "z-", "z+", "y-", "y+") if side == 0 else ("y-", "y+", "x-", "x+", "z-", "z+")
    st = s39.box_state39(NX, NY, NZ, faces, shifted, 1, periodic=periodic, priority=prio)
    st[0, 3, 2:4, 5:7] = -1
    cx, cy, cz, _ = s39.lattice39(shifted, 1)
    for i in range(1, 39):
        for z in range(NZ):
            for y in range(NY):
                for x in range(NX):
                    if st[0, z, y, x] < 0:
                        continue
                    tx, ty, tz = x + cx[i], (y + cy[i]) % NY, z + cz[i]
                    if 0 <= tx < NX and 0 <= tz < NZ and st[0, tz, ty, tx] < 0:
                        st[i, z, y, x] = -10
    st[5, 1, 1, 1] = -666
    rs = np.random.RandomState(seed)
    pops = [0.01 + 0.1 * rs.random_sample((39, NZ, NY, NX)) for _ in range(4)]
    tabs = [0.01 + 0.1 * rs.random_sample(39) for _ in range(6)]
    return {"state": st, "fout": pops[0], "gout": pops[1], "prev_f": pops[2], "prev_g": pops[3],
            "ff": tabs[0], "gf": tabs[1], "fi": tabs[2], "gi": tabs[3], "fo": tabs[4], "go": tabs[5],
            "inlet_type": [1] * 8, "outlet_type": [outlet_type] + [1] * 7, "periodic": periodic,
            "shifted": shifted}


def digest(a: np.ndarray) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


# wall cases: the shifted lattice's double-ramp wedge between inviscid side walls (inlet,
# outlet of type 6, bounce-back floor, freestream top, the ramp's interpolated wall links),
# at the start (timestep 0: the start-up multipliers seed the target solves) and past the
# start-up (the node's own multipliers seed them)
WALL_CASES = {"wedge_start": (0, 21), "wedge_late": (150, 22)}
# side faces of the wall cases: bounce-back, so that no inviscid link meets a wall link (where
# the reference's inviscid_edge assigns no direction and the push writes into the slot of a
# stale direction variable, which the library does not reproduce)
WALL_FACES = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": -10, "y+": -10}
WNX, WNY, WNZ = 20, 6, 10


def unshifted_wall_case(s39, seed=23, step=150):
    """An unshifted box (Mach 0.5) with an inlet, an outlet of type 6, bounce-back floor
    and side faces, a freestream top and a solid block whose fluid neighbours carry
    interpolated wall links of seeded fractions; fields near the freestream, every
    node's multipliers at the freestream solution."""
    import math

    c = s39.wedge_case_consts(v_inf_ms=0.5 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=False)
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": -10, "y+": -10}
    st = s39.box_state39(WNX, WNY, WNZ, faces, 0, 1, periodic=0)
    solid = np.zeros((WNZ, WNY, WNX), bool)
    solid[0:3, 2:4, 8:11] = True
    rs = np.random.RandomState(seed)
    s39.wall_links39(st, solid, rs.uniform(0.05, 0.95, (39, WNZ, WNY, WNX)), 0, 1, periodic=0)
    shape = (39, WNZ, WNY, WNX)
    pops = [0.01 + 0.1 * rs.random_sample(shape) for _ in range(4)]
    tabs = [0.01 + 0.1 * rs.random_sample(39) for _ in range(6)]
    n3 = (WNZ, WNY, WNX)
    fields = [1.0 + 0.02 * rs.uniform(-1, 1, n3), c.mach * (1 + 0.05 * rs.uniform(-1, 1, n3)),
              0.02 * c.mach * rs.uniform(-1, 1, n3), 0.02 * c.mach * rs.uniform(-1, 1, n3),
              c.temperature * (1 + 0.03 * rs.uniform(-1, 1, n3))]
    lm0 = np.asarray(s39.freestream_start_lm(c), np.float64)
    lm = np.broadcast_to(lm0[:, None, None, None], (13,) + n3).copy()
    return c, {"state": st, "fout": pops[0], "gout": pops[1], "prev_f": pops[2], "prev_g": pops[3],
               "ff": tabs[0], "gf": tabs[1], "fi": tabs[2], "gi": tabs[3], "fo": tabs[4], "go": tabs[5],
               "inlet_type": [1] * 8, "outlet_type": [6] + [1] * 7, "periodic": 0, "shifted": 0,
               "fields": fields, "lm": lm, "su_lm": list(c.su_lm), "fs_uvwT": (c.mach, 0.0, 0.0, c.temperature),
               "step": step}


def wall_case(name: str, s39):
    """The push-loop case dict (see case) plus the fields rho, u, v, w, T near the
    freestream, every node's multipliers at the freestream solution, the start-up
    multipliers, the freestream (u, v, w, T) and the step."""
    step, seed = WALL_CASES[name]
    c = s39.wedge_case_consts()
    st = s39.wedge_state39(WNX, WNY, WNZ, 5.0, 12.0, 20.0, WALL_FACES, periodic=0, priority=s39.WEDGE_PRIORITY)
    rs = np.random.RandomState(seed)
    shape = (39, WNZ, WNY, WNX)
    pops = [0.01 + 0.1 * rs.random_sample(shape) for _ in range(4)]
    tabs = [0.01 + 0.1 * rs.random_sample(39) for _ in range(6)]
    n3 = (WNZ, WNY, WNX)
    fields = [1.0 + 0.02 * rs.uniform(-1, 1, n3), c.mach * (1 + 0.05 * rs.uniform(-1, 1, n3)),
              0.02 * c.mach * rs.uniform(-1, 1, n3), 0.02 * c.mach * rs.uniform(-1, 1, n3),
              c.temperature * (1 + 0.03 * rs.uniform(-1, 1, n3))]
    lm0 = np.asarray(s39.freestream_start_lm(c), np.float64)
    lm = np.broadcast_to(lm0[:, None, None, None], (13,) + n3).copy()
    return {"state": st, "fout": pops[0], "gout": pops[1], "prev_f": pops[2], "prev_g": pops[3],
            "ff": tabs[0], "gf": tabs[1], "fi": tabs[2], "gi": tabs[3], "fo": tabs[4], "go": tabs[5],
            "inlet_type": [1] * 8, "outlet_type": [6] + [1] * 7, "periodic": 0, "shifted": 1,
            "fields": fields, "lm": lm, "su_lm": list(c.su_lm), "fs_uvwT": (c.mach, 0.0, 0.0, c.temperature),
            "step": step}
