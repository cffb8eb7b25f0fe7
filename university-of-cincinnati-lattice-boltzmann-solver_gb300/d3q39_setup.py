"""Host-side set-up of the D3Q39 compressible path: reference scales, relaxation
ramps and the start-up multipliers, computed from the physical inputs exactly
as the reference's background calculations do (before any time step):

  basic_fluid_calcs     general/background_calcs/basic_fluids_calcs.f95:17-86
  viscosity_and_timing  utilities/viscosity_and_timing.f95:35-68
  timing_calcs          general/background_calcs/timing_calcs.f95:23-35 (dt = dx/c, eps = dt)
  start-up multipliers  boundary_conditions/basic_calcs/freestream_basis_calcs.f90:127-150

Several of the reference's constants are default-real (single precision)
literals assigned to double variables (e.g. sutherlands_const = 110.4,
visc_ref = 1.716E-5, temp_ref = 273.15, molec_mass_air = 28.97); they are
reproduced through float32 rounding below.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def _f32(x: float) -> float:
    return float(np.float32(x))


GAS_CONST_R = 287.052874
MOLEC_MASS_AIR = _f32(28.97)   # general/modules/constants.f95:9 (default real)
AVOCADOS_NUMBER = 6.022e23


@dataclass
class D3Q39Consts:
    shifted: int
    primary_flow_dir: int
    turbulent: int
    lvl: int
    startup_timesteps: int
    max_lm_iters: int
    gama: float
    t_ref: float
    rho_ref: float
    p_ref: float
    mu_ref: float
    kappa_ref: float
    gas_const_R: float
    const_vol: float
    const_press: float
    molec_weight: float
    dt: float
    elbm_epsilon: float
    init_beta_1: float
    init_beta_2: float
    beta_1_scaling: float
    beta_2_scaling: float
    su_lm: list = field(default_factory=lambda: [0.0] * 13)
    # lattice-unit freestream
    temperature: float = 0.0
    mach: float = 0.0


def _therm_cond_startup(rho, T_lattice, t_ref, gama, rho_ref):
    """quick_therm_cond with startup present (kappa_bottom = 1), T <= 500 K branch."""
    unit_temp = T_lattice * t_ref * gama
    if unit_temp > 500.0:
        raise ValueError("start-up conductivity outside the <= 500 K branch")
    return 418.1 * (5.9776e-6 * unit_temp ** 1.5 / (unit_temp + _f32(194.4))) / 1.0


def reference_consts(temperature_K: float, pressure_Pa: float, v_inf_ms: float, dx_m: float, gama: float = 1.4,
                     primary_flow_dir: int = 1, use_shifted: bool = False, turbulent: bool = True,
                     startup_timesteps: int = 100, lvl: int = 0, max_lm_iters: int = 200) -> D3Q39Consts:
    # basic_fluid_calcs
    R = GAS_CONST_R
    rho_ref = pressure_Pa / (R * temperature_K)
    t_ref = temperature_K
    p_ref = pressure_Pa
    const_vol = 1.0 / (gama - 1.0)
    const_press = gama / (gama - 1.0)
    temperature = 1.0 / gama
    rho_inf = 1.0
    speed_of_sound = math.sqrt(gama * R * t_ref)
    u_ref = speed_of_sound
    mach = v_inf_ms / u_ref
    molec_weight = MOLEC_MASS_AIR / (AVOCADOS_NUMBER * 1000)
    shifted = bool(mach >= 1.2 or use_shifted)
    # viscosity_and_timing
    sutherlands_const = _f32(110.4)
    visc_ref = _f32(1.716e-5)
    temp_ref = _f32(273.15)
    viscosity = visc_ref * ((t_ref / temp_ref) ** 1.5) * ((temp_ref + sutherlands_const) / (t_ref + sutherlands_const))
    mu_ref = rho_ref * u_ref * mach * 1
    kappa_base = _therm_cond_startup(rho_inf, temperature, t_ref, gama, rho_ref)
    kappa_ref = rho_inf * speed_of_sound ** 3 / temperature
    init_beta_1 = 0.5001
    init_beta_2 = 0.5001
    beta_1 = 1.0 / ((2.0 * viscosity) / (rho_inf * temperature) + 1.0)
    beta_2 = 1.0 / ((2.0 * kappa_base / kappa_ref) / (rho_inf * const_press * temperature) + 1.0)
    beta_1_scaling = (beta_1 - init_beta_1) / float(startup_timesteps)
    beta_2_scaling = (beta_2 - init_beta_2) / float(startup_timesteps)
    # timing_calcs: dt = dx / c, eps = dt, per level dx / 2^lvl
    dt = (dx_m / 2 ** lvl) / speed_of_sound
    # start-up multipliers (freestream_basis_calcs.f90:127-150), refined by the LM solve of su_* moments
    if mach > 1.0:
        su_lm = [-2.2, 0.4, 0.0, 0.0, -0.45, -0.45, -0.45, 0.0, 0.0, 0.0, 0.015, 0.0, 0.0]
    else:
        su_lm = [-2.0, 0.0, 0.0, 0.0, -0.4, -0.4, -0.4, 0.0, 0.0, 0.0, 0.002, 0.0, 0.0]
    return D3Q39Consts(shifted=int(shifted), primary_flow_dir=primary_flow_dir, turbulent=int(turbulent), lvl=lvl,
                       startup_timesteps=startup_timesteps, max_lm_iters=max_lm_iters, gama=gama, t_ref=t_ref,
                       rho_ref=rho_ref, p_ref=p_ref, mu_ref=mu_ref, kappa_ref=kappa_ref, gas_const_R=R,
                       const_vol=const_vol, const_press=const_press, molec_weight=molec_weight, dt=dt,
                       elbm_epsilon=dt, init_beta_1=init_beta_1, init_beta_2=init_beta_2,
                       beta_1_scaling=beta_1_scaling, beta_2_scaling=beta_2_scaling, su_lm=su_lm,
                       temperature=temperature, mach=mach)


def freestream_start_lm(c: D3Q39Consts):
    """Initial multiplier guess of the freestream solve (freestream_basis_calcs.f90:24-90)."""
    if not c.shifted:
        return [-2.4, 0.0, 0.0, 0.0, -0.4, -0.4, -0.4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    lm = [-3.0, 0.0, 0.0, 0.0, -0.4, -0.4, -0.4, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    axis = (c.primary_flow_dir - 1) % 3
    sign = 1.0 if c.primary_flow_dir <= 3 else -1.0
    lm[1 + axis] = sign * c.mach
    lm[10 + axis] = -sign * c.mach / 50.0
    return lm


def wedge_case_consts(nu_lattice=None, **kw) -> D3Q39Consts:
    """The Mach 1.5 wedge case in reference units: gamma = 1.4, air at 288.15 K and
    101325 Pa, v_inf = 1.5 c (so the Galilean-shifted lattice is on), dx = 1e-4 m.
    nu_lattice: the freestream's lattice kinematic viscosity mu / rho instead (the
    relaxation 1 / (2 mu / (rho T) + 1) of amr_processes.f95:1751-1787).  The
    reference scales viscosity by mu_ref = rho_ref c Ma x 1 m (viscosity_and_timing),
    so the lattice viscosity goes as 1 / pressure: the pressure is set to give it
    (14.6 Pa for 2e-4; at 101325 Pa it is 2.9e-8)."""
    T, p, gama = 288.15, 101325.0, 1.4
    c = math.sqrt(gama * GAS_CONST_R * T)
    if nu_lattice is not None:
        # the step's Sutherland law at the freestream temperature (quick_calcs.f95:24-64)
        const_s, temp_ref = _f32(110.15), _f32(273.15)
        unit_mu = 1.716e-5 * (T / temp_ref) ** 1.5 * ((temp_ref + const_s) / (T + const_s))
        p = unit_mu * GAS_CONST_R * T / (nu_lattice * c * 1.5)
    args = dict(temperature_K=T, pressure_Pa=p, v_inf_ms=1.5 * c, dx_m=1e-4, gama=gama, primary_flow_dir=1)
    args.update(kw)
    return reference_consts(**args)


# D3Q39 velocities in the reference's order and its opposites (1-based in the
# reference, general/background_calcs/directions_and_weights.f95:463-499).
CX39 = [0, 1, 0, 0, -1, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 2, 0, 0, -2, 0,
        0, 2, 2, 0, -2, -2, 2, 2, -2, -2, 0, 0, 0, 3, 0, 0, -3, 0, 0]
CY39 = [0, 0, 1, 0, 0, -1, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 2, 0, 0, -2,
        0, 2, 0, 2, 2, -2, -2, 0, 0, 0, 2, -2, -2, 0, 3, 0, 0, -3, 0]
CZ39 = [0, 0, 0, 1, 0, 0, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 2, 0, 0,
        -2, 0, 2, 2, 0, 0, 0, -2, -2, 2, -2, -2, 2, 0, 0, 3, 0, 0, -3]
OPP39 = [1, 5, 6, 7, 2, 3, 4, 14, 15, 12, 13, 10, 11, 8, 9, 19, 20, 21, 16, 17,
         18, 26, 29, 32, 27, 22, 25, 30, 23, 28, 33, 24, 31, 37, 38, 39, 34, 35, 36]


def lattice39(shifted: int, primary_flow_dir: int = 1):
    """Streaming velocities (cx, cy, cz) and opposites (0-based) of the D3Q39
    set; the shifted set adds one unit along the primary flow direction and
    maps every direction to itself as its opposite (directions_and_weights.f95:477-499)."""
    cx, cy, cz = (np.array(v, np.int64) for v in (CX39, CY39, CZ39))
    if shifted:
        axis, sign = (primary_flow_dir - 1) % 3, (1 if primary_flow_dir <= 3 else -1)
        (cx, cy, cz)[axis][:] += sign
        opp = np.arange(39)
    else:
        opp = np.array(OPP39) - 1
    return cx, cy, cz, opp


def box_state39(nx: int, ny: int, nz: int, faces: dict, shifted: int, primary_flow_dir: int = 1, periodic: int = 0,
                priority=("x-", "x+", "z-", "z+", "y-", "y+")) -> np.ndarray:
    """int32 state (39, nz, ny, nx) of a box: a link that leaves the box across a
    non-periodic face carries that face's code (faces: 'x-', 'x+', 'y-', 'y+',
    'z-', 'z+'); links crossing two faces take the code of the first in
    `priority`; component 0 (node type) is 0."""
    cx, cy, cz, _ = lattice39(shifted, primary_flow_dir)
    st = np.zeros((39, nz, ny, nx), np.int32)
    x = np.arange(nx)[None, None, :]
    y = np.arange(ny)[None, :, None]
    z = np.arange(nz)[:, None, None]
    shape = (nz, ny, nx)
    for i in range(1, 39):
        comp = np.zeros(shape, np.int32)
        crossed = {
            "x-": np.broadcast_to((x + cx[i] < 0) & (not periodic & 1), shape),
            "x+": np.broadcast_to((x + cx[i] >= nx) & (not periodic & 1), shape),
            "y-": np.broadcast_to((y + cy[i] < 0) & (not periodic & 2), shape),
            "y+": np.broadcast_to((y + cy[i] >= ny) & (not periodic & 2), shape),
            "z-": np.broadcast_to((z + cz[i] < 0) & (not periodic & 4), shape),
            "z+": np.broadcast_to((z + cz[i] >= nz) & (not periodic & 4), shape),
        }
        for face in reversed(priority):
            comp[crossed[face]] = faces[face]
        st[i] = comp
    return st


def wall_links39(state: np.ndarray, solid: np.ndarray, q, shifted: int = 1, primary_flow_dir: int = 1,
                 periodic: int = 0) -> np.ndarray:
    """Mark solid nodes and interpolated wall links in a D3Q39 state array
    (39, nz, ny, nx), in place: a solid node gets node type -1001 and -666 on
    every link; on the shifted lattice (lbgrid/shifted_state_directions.f95:
    54-68) a fluid node x whose upstream node x - c_i is solid gets, on link i,
    the code -1001 - floor(q 1e9) (linking/modules/linkwise.f95:45-57), q being
    the wall distance along the link as a fraction of its length; on the
    unshifted lattice (lbgrid/state_directions.f95:696) the link i whose
    downstream node x + c_i is solid gets it.  q: array (39, nz, ny, nx) or a
    number."""
    cx, cy, cz, _ = lattice39(shifted, primary_flow_dir)
    if not shifted:
        cx, cy, cz = -np.asarray(cx), -np.asarray(cy), -np.asarray(cz)
    nz, ny, nx = solid.shape
    state[0][solid] = -1001
    state[1:, solid] = -666
    qa = np.broadcast_to(np.asarray(q, np.float64), (39, nz, ny, nx))
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    for i in range(1, 39):
        sx, sy, sz = x - cx[i], y - cy[i], z - cz[i]
        inside = np.ones(solid.shape, bool)
        for s, n, bit in ((sx, nx, 1), (sy, ny, 2), (sz, nz, 4)):
            if periodic & bit:
                s %= n
            else:
                inside &= (s >= 0) & (s < n)
        up_solid = np.zeros(solid.shape, bool)
        up_solid[inside] = solid[sz[inside], sy[inside], sx[inside]]
        mark = up_solid & ~solid
        state[i][mark] = (-1001 - np.floor(qa[i][mark] * 1e9)).astype(np.int32)
    return state


def wedge_state39(nx: int, ny: int, nz: int, x0: float, x1: float, angle_deg: float, faces: dict,
                  primary_flow_dir: int = 1, periodic: int = 2,
                  priority=("x-", "x+", "z-", "z+", "y-", "y+"), x_apex=None) -> np.ndarray:
    """State array (39, nz, ny, nx) of the shifted-lattice wedge case: box faces as in
    box_state39 and a wedge across the whole span, its ramp rising at the given angle from
    the floor at x = x0 to a vertical back face at x = x1 (nodes with x0 <= x <= x1 and
    z <= tan(angle) (x - x0) are solid); with x_apex, the ramp rises to x_apex and a
    second ramp at the same angle falls back to the floor at x = x1 (no back face).
    Every fluid node x whose upstream node x - c_i is solid gets the wall code of the
    first crossing of the segment from x to x - c_i with the wedge surface, at the
    fraction q of the segment (lbgrid/inter_bb_setup.f95: ray from the node towards
    x - c_i on the shifted lattice; linking/modules/linkwise.f95:45-57)."""
    st = box_state39(nx, ny, nz, faces, 1, primary_flow_dir, periodic=periodic, priority=priority)
    cx, cy, cz, _ = lattice39(1, primary_flow_dir)
    t = math.tan(math.radians(angle_deg))
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    xa = x1 if x_apex is None else x_apex
    solid = (z <= t * (x - x0)) & (x >= x0) & (x <= xa)
    if x_apex is not None:
        solid |= (z <= t * (x1 - x)) & (x >= xa) & (x <= x1)
    q = np.full((39, nz, ny, nx), 0.5)
    for i in range(1, 39):
        best = np.full(solid.shape, np.inf)
        with np.errstate(divide="ignore", invalid="ignore"):
            # front ramp z = t (x - x0), between x0 and the apex (or the back face)
            dh = cz[i] - t * cx[i]
            lam = (z - t * (x - x0)) / dh
            X = x - lam * cx[i]
            ok = (dh != 0.0) & (lam >= 0.0) & (lam <= 1.0) & (X >= x0) & (X <= xa)
            best = np.where(ok, np.minimum(best, lam), best)
            if x_apex is None:
                # back face x = x1, below the ramp's top
                lam = (x - x1) / cx[i] if cx[i] != 0 else np.full(solid.shape, np.inf)
                Z = z - lam * cz[i]
                ok = (lam >= 0.0) & (lam <= 1.0) & (Z <= t * (x1 - x0))
            else:
                # rear ramp z = t (x1 - x), between the apex and x1
                dh = cz[i] + t * cx[i]
                lam = (z - t * (x1 - x)) / dh
                X = x - lam * cx[i]
                ok = (dh != 0.0) & (lam >= 0.0) & (lam <= 1.0) & (X >= xa) & (X <= x1)
            best = np.where(ok, np.minimum(best, lam), best)
        q[i] = np.where(np.isfinite(best), np.clip(best, 0.0, 1.0 - 1e-9), 0.5)
    return wall_links39(st, solid, q, 1, primary_flow_dir, periodic=periodic)


# Faces of the 10-degree wedge case: inlet 1 at x = 0, outlet 1 at x = nx - 1,
# bounce-back floor (the wedge's base plane) at z = 0, freestream top,
# inviscid side walls at y = 0 and y = ny - 1.  Links that cross two faces
# take the floor's code first, then the side walls': with the side walls
# first, the floor's corner lines went non-finite within 250 steps (FP64, the
# repair on), with the floor first the run stays finite.
WEDGE_FACES = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": -11, "y+": -11}
WEDGE_PRIORITY = ("z-", "y-", "y+", "x-", "x+", "z+")


def wedge_case_state(nx: int = 384, ny: int = 48, nz: int = 192) -> np.ndarray:
    """State array (39, nz, ny, nx) of the Mach 1.5 wedge case: x streamwise, y the
    48-node span between inviscid side walls, z the height; the wedge's leading
    edge on the floor at x = nx / 4 (96 at the full size), its ramp rising at 10
    degrees to x = 9 nx / 16 (216, 21 nodes high), then falling at 10 degrees back
    to the floor at x = 7 nx / 8 (336).  The rear ramp stands in for a back face:
    behind a vertical face the flow separates into a base region that this
    explicit scheme does not keep finite."""
    return wedge_state39(nx, ny, nz, nx / 4, nx * 7 / 8, 10.0, WEDGE_FACES, periodic=0, priority=WEDGE_PRIORITY,
                         x_apex=nx * 9 / 16)


def wedge_triangles(x0: float, x_apex: float, x1: float, angle_deg: float, ny: int) -> np.ndarray:
    """The double-ramp wedge of wedge_state39 (x_apex given) as a closed
    triangulated prism (8 triangles, (8, 3, 3)): its cross-section in the x-z
    plane is the triangle under the two ramps, continued below the floor to
    z = -1, extruded over y from -2 to ny + 1 (beyond the box, so that its end
    caps meet no link)."""
    t = math.tan(math.radians(angle_deg))
    a = (x0 - 1.0 / t, -1.0)
    b = (x_apex, t * (x_apex - x0))
    c = (x1 + 1.0 / t, -1.0)
    y0, y1 = -2.0, ny + 1.0
    P = lambda q, y: (q[0], y, q[1])
    tris = [(P(a, y0), P(b, y0), P(c, y0)), (P(a, y1), P(c, y1), P(b, y1))]
    for p, q in ((a, b), (b, c), (c, a)):
        tris.append((P(p, y0), P(q, y0), P(q, y1)))
        tris.append((P(p, y0), P(q, y1), P(p, y1)))
    return np.asarray(tris, np.float64)
