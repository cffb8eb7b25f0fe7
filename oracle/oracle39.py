"""ctypes binding of the D3Q39 CPU oracle (test infrastructure only)."""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import oracle as _o27

Q39 = 39
NLM = 13


class O39Consts(ct.Structure):
    _fields_ = [
        ("shifted", ct.c_int),
        ("primary_flow_dir", ct.c_int),
        ("turbulent", ct.c_int),
        ("lvl", ct.c_int),
        ("startup_timesteps", ct.c_int),
        ("max_lm_iters", ct.c_int),
        ("gama", ct.c_double),
        ("t_ref", ct.c_double),
        ("rho_ref", ct.c_double),
        ("p_ref", ct.c_double),
        ("mu_ref", ct.c_double),
        ("kappa_ref", ct.c_double),
        ("gas_const_R", ct.c_double),
        ("const_vol", ct.c_double),
        ("const_press", ct.c_double),
        ("molec_weight", ct.c_double),
        ("dt", ct.c_double),
        ("elbm_epsilon", ct.c_double),
        ("init_beta_1", ct.c_double),
        ("init_beta_2", ct.c_double),
        ("beta_1_scaling", ct.c_double),
        ("beta_2_scaling", ct.c_double),
        ("su_lm", ct.c_double * NLM),
    ]


class O39Stats(ct.Structure):
    _fields_ = [(n, ct.c_int64) for n in ("nodes", "lm_iters", "lm_capped", "alpha_not2", "damped", "errors")]


class O39Level(ct.Structure):
    _fields_ = [("nx", ct.c_int), ("ny", ct.c_int), ("nz", ct.c_int)] + [
        (n, ct.c_void_p) for n in ("fout", "gout", "lm", "w_vel", "alpha", "rho", "u", "v", "temp")]


def lib():
    L = _o27.lib()
    vp = ct.c_void_p
    if not getattr(L, "_o39_ready", False):
        L.o39_step_periodic.restype = ct.c_int
        L.o39_step_periodic.argtypes = [ct.POINTER(O39Consts), ct.POINTER(O39Level), ct.c_int, ct.POINTER(O39Stats)]
        L.o39_init_node.restype = ct.c_int
        L.o39_init_node.argtypes = [ct.POINTER(O39Consts)] + [ct.c_double] * 5 + [vp, vp, vp]
        L.o39_lagrange_api.restype = ct.c_int
        L.o39_lagrange_api.argtypes = [ct.POINTER(O39Consts)] + [ct.c_double] * 5 + [vp, vp, vp]
        L.o39_alpha.restype = ct.c_double
        L.o39_alpha.argtypes = [ct.POINTER(O39Consts), vp, vp, ct.c_double, ct.c_int]
        L.o39_tables.restype = None
        L.o39_tables.argtypes = [ct.c_int, ct.c_int, vp, vp, vp, vp]
        L._o39_ready = True
    return L


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def consts(c) -> O39Consts:
    """O39Consts from a D3Q39Consts dataclass (same field names)."""
    k = O39Consts()
    for name, _ in O39Consts._fields_:
        if name == "su_lm":
            for i, v in enumerate(c.su_lm):
                k.su_lm[i] = v
        else:
            setattr(k, name, getattr(c, name))
    return k


def tables(shifted, pfd=1):
    cx, cy, cz, opp = (np.zeros(Q39, np.int32) for _ in range(4))
    lib().o39_tables(shifted, pfd, _p(cx), _p(cy), _p(cz), _p(opp))
    return cx, cy, cz, opp


def lagrange(k: O39Consts, rho, u, v, w, T, P, lm0):
    P = np.ascontiguousarray(P, np.float64)
    lm = np.ascontiguousarray(lm0, np.float64).copy()
    fe = np.zeros(Q39)
    it = lib().o39_lagrange_api(ct.byref(k), rho, u, v, w, T, _p(P), _p(lm), _p(fe))
    return lm, fe, it


def init_node(k: O39Consts, rho, u, v, w, T, lm0):
    lm = np.ascontiguousarray(lm0, np.float64).copy()
    f = np.zeros(Q39)
    g = np.zeros(Q39)
    it = lib().o39_init_node(ct.byref(k), rho, u, v, w, T, _p(lm), _p(f), _p(g))
    return lm, f, g, it


def explode_node(k: O39Consts, step, f, g, lm, rho_c, temp_c):
    """One fine ghost node of the D3Q39 explosion from its coarse interpolants:
    returns (f, g, lm, macro5, alpha, flags) (flags bit 0: a population was
    replaced by the coarse equilibrium, bit 1: the multiplier Newton hit the cap)."""
    L = lib()
    if not getattr(L, "_o39_explode_ready", False):
        L.o39_explode_node.restype = ct.c_int
        L.o39_explode_node.argtypes = [ct.POINTER(O39Consts), ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                       ct.c_double, ct.c_double, ct.c_void_p, ct.POINTER(ct.c_double)]
        L._o39_explode_ready = True
    f = np.ascontiguousarray(f, np.float64).copy()
    g = np.ascontiguousarray(g, np.float64).copy()
    lm = np.ascontiguousarray(lm, np.float64).copy()
    m5 = np.zeros(5)
    a = ct.c_double(0.0)
    flags = L.o39_explode_node(ct.byref(k), step, _p(f), _p(g), _p(lm), rho_c, temp_c, _p(m5), ct.byref(a))
    return f, g, lm, m5, a.value, flags


def alpha(k: O39Consts, f, fd, T, step):
    return lib().o39_alpha(ct.byref(k), _p(np.ascontiguousarray(f, np.float64)),
                           _p(np.ascontiguousarray(fd, np.float64)), T, step)


class Level39:
    """Level state for the periodic-box oracle (component-major, x fastest)."""

    def __init__(self, nx, ny, nz):
        self.shape = (nz, ny, nx)
        N = nx * ny * nz
        self.fout = np.zeros((Q39,) + self.shape)
        self.gout = np.zeros((Q39,) + self.shape)
        self.lm = np.zeros((NLM,) + self.shape)
        self.w_vel = np.zeros(self.shape)
        self.alpha = np.zeros(self.shape)
        self.rho = np.zeros(self.shape)
        self.u = np.zeros(self.shape)
        self.v = np.zeros(self.shape)
        self.temp = np.zeros(self.shape)
        self.nx, self.ny, self.nz, self.N = nx, ny, nz, N

    def c(self):
        s = O39Level()
        s.nx, s.ny, s.nz = self.nx, self.ny, self.nz
        for n in ("fout", "gout", "lm", "w_vel", "alpha", "rho", "u", "v", "temp"):
            setattr(s, n, getattr(self, n).ctypes.data)
        return s


def step_periodic(k: O39Consts, lev: Level39, step: int):
    st = O39Stats()
    s = lev.c()
    rc = lib().o39_step_periodic(ct.byref(k), ct.byref(s), step, ct.byref(st))
    if rc != 0:
        raise RuntimeError(f"o39 step failed {rc}")
    return {n: getattr(st, n) for n, _ in st._fields_}


class O39Bc(ct.Structure):
    _fields_ = [("inlet_type", ct.c_int * 8), ("outlet_type", ct.c_int * 8),
                ("fs_fieq", ct.c_double * Q39), ("fs_gieq", ct.c_double * Q39),
                ("inl_fieq", (ct.c_double * Q39) * 8), ("inl_gieq", (ct.c_double * Q39) * 8),
                ("outl_fieq", (ct.c_double * Q39) * 8), ("outl_gieq", (ct.c_double * Q39) * 8),
                ("fs_u", ct.c_double), ("fs_v", ct.c_double), ("fs_w", ct.c_double), ("fs_temp", ct.c_double)]


def bc(inlet_type, outlet_type, fs_f, fs_g, inl_f, inl_g, outl_f, outl_g, fs_uvwT=(0.0, 0.0, 0.0, 0.0)) -> O39Bc:
    b = O39Bc()
    b.fs_u, b.fs_v, b.fs_w, b.fs_temp = (float(x) for x in fs_uvwT)
    for k in range(8):
        b.inlet_type[k] = int(inlet_type[k])
        b.outlet_type[k] = int(outlet_type[k])
        for i in range(Q39):
            b.inl_fieq[k][i], b.inl_gieq[k][i] = inl_f[k][i], inl_g[k][i]
            b.outl_fieq[k][i], b.outl_gieq[k][i] = outl_f[k][i], outl_g[k][i]
    for i in range(Q39):
        b.fs_fieq[i], b.fs_gieq[i] = fs_f[i], fs_g[i]
    return b


def step_links(k: O39Consts, lev: Level39, step: int, state: np.ndarray, periodic: int, b: O39Bc,
               fi_prev: np.ndarray, gi_prev: np.ndarray):
    """One step with the reference's link codes (state: (39, nz, ny, nx) int32); fi_prev and gi_prev
    hold the post-streaming populations of the previous step and are updated in place.  Wall links
    (codes -1001 - q*1e9) read the previous step's macroscopic fields lev.rho, u, v, w_vel, temp."""
    L = lib()
    if not getattr(L, "_o39_links_ready", False):
        L.o39_step_links.restype = ct.c_int
        L.o39_step_links.argtypes = [ct.POINTER(O39Consts), ct.POINTER(O39Level), ct.c_int, ct.POINTER(O39Stats),
                                     ct.c_void_p, ct.c_int, ct.POINTER(O39Bc), ct.c_void_p, ct.c_void_p]
        L._o39_links_ready = True
    st = O39Stats()
    s = lev.c()
    stc = np.ascontiguousarray(state, np.int32)
    assert fi_prev.flags.c_contiguous and gi_prev.flags.c_contiguous
    rc = L.o39_step_links(ct.byref(k), ct.byref(s), step, ct.byref(st), _p(stc), periodic, ct.byref(b),
                          _p(fi_prev), _p(gi_prev))
    if rc != 0:
        raise RuntimeError(f"o39 link step failed {rc}")
    return {n: getattr(st, n) for n, _ in st._fields_}


def ibb_wall_axis(i, axis):
    """(wall form?, up-wind?) of the oracle's derivative rule for direction i (0-based), axis 0..2."""
    L = lib()
    if not getattr(L, "_o39_axis_ready", False):
        L.o39_ibb_wall_axis.restype = ct.c_int
        L.o39_ibb_wall_axis.argtypes = [ct.c_int, ct.c_int, ct.POINTER(ct.c_int)]
        L._o39_axis_ready = True
    up = ct.c_int(0)
    wall = L.o39_ibb_wall_axis(i, axis, ct.byref(up))
    return bool(wall), bool(up.value)


def inviscid(i, codes):
    """(found, j, d) of the oracle's specular rule for an inviscid link of direction i (0-based),
    given the node's 39 state components."""
    L = lib()
    if not getattr(L, "_o39_inv_ready", False):
        L.o39_inviscid.restype = ct.c_int
        L.o39_inviscid.argtypes = [ct.c_int, ct.c_void_p, ct.POINTER(ct.c_int), ct.c_void_p]
        L._o39_inv_ready = True
    c = np.ascontiguousarray(codes, np.int32)
    j = ct.c_int(0)
    d = np.zeros(3, np.int32)
    ok = L.o39_inviscid(i, _p(c), ct.byref(j), _p(d))
    return bool(ok), j.value, tuple(int(x) for x in d)


def step_links_damp(k: O39Consts, lev: Level39, step: int, state: np.ndarray, periodic: int, b: O39Bc,
                    fi_prev: np.ndarray, gi_prev: np.ndarray, lo, hi):
    """step_links, then the fout and gout parts of damp_it on the box (lo, hi: its index-space corners)."""
    L = lib()
    if not getattr(L, "_o39_damp_ready", False):
        L.o39_step_links_damp.restype = ct.c_int
        L.o39_step_links_damp.argtypes = [ct.POINTER(O39Consts), ct.POINTER(O39Level), ct.c_int,
                                          ct.POINTER(O39Stats), ct.c_void_p, ct.c_int, ct.POINTER(O39Bc),
                                          ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]
        L._o39_damp_ready = True
    st = O39Stats()
    s = lev.c()
    stc = np.ascontiguousarray(state, np.int32)
    lo_a = np.ascontiguousarray(lo, np.int32)
    hi_a = np.ascontiguousarray(hi, np.int32)
    rc = L.o39_step_links_damp(ct.byref(k), ct.byref(s), step, ct.byref(st), _p(stc), periodic, ct.byref(b),
                               _p(fi_prev), _p(gi_prev), _p(lo_a), _p(hi_a))
    if rc != 0:
        raise RuntimeError(f"o39 link step failed {rc}")
    return {n: getattr(st, n) for n, _ in st._fields_}


# ---- pieces of the step, for the golden fixtures run from the reference's statements ----
def _pieces():
    L = lib()
    if not getattr(L, "_o39_pieces", False):
        vp, d, i = ct.c_void_p, ct.c_double, ct.c_int
        L.o39_fieq_api.restype = None
        L.o39_fieq_api.argtypes = [i, i, d, vp, vp]
        L.o39_jacobian_api.restype = None
        L.o39_jacobian_api.argtypes = [i, i, vp, vp]
        L.o39_lu_api.restype = d
        L.o39_lu_api.argtypes = [vp, vp, vp]
        L.o39_q_bar_api.restype = None
        L.o39_q_bar_api.argtypes = [ct.POINTER(O39Consts), vp, d, d, d, d, i, vp]
        L.o39_little_q_bar_api.restype = None
        L.o39_little_q_bar_api.argtypes = [ct.POINTER(O39Consts), vp, d, d, d, d, i, vp]
        L.o39_collide_node_api.restype = None
        L.o39_collide_node_api.argtypes = [ct.POINTER(O39Consts), vp, vp, vp, d, d, d, d, d, d, i, vp, vp]
        L.o39_flow_vars_api.restype = None
        L.o39_flow_vars_api.argtypes = [ct.POINTER(O39Consts), vp, vp, d, vp]
        L.o39_shifted_ibb_api.restype = None
        L.o39_shifted_ibb_api.argtypes = [ct.POINTER(O39Consts), i, i, d, d, d, vp, vp, vp, vp, vp, vp, vp]
        L.o39_target_finder_api.restype = None
        L.o39_target_finder_api.argtypes = [ct.POINTER(O39Consts), vp, vp, vp, vp, vp, vp, d, vp]
        L.o39_damp_api.restype = ct.c_int64
        L.o39_damp_api.argtypes = [ct.POINTER(O39Consts), vp, vp, i, i, i, vp, vp, vp]
        L._o39_pieces = True
    return L


def _a(x):
    return np.ascontiguousarray(x, np.float64)


def shifted_ibb(k: O39Consts, i, step, fieq, gieq, rho, tgt, u, v, w, T, sp):
    """(fout, gout) of shifted_ibb.f95 for wall link i (0-based): the closure direction's
    equilibria, rho, the (u, v, w, T) targets, the seven-point stencil's fields and node
    types (rest, +x, +y, +z, -x, -y, -z)."""
    out = np.zeros(2)
    spa = np.ascontiguousarray(sp, np.int32)
    _pieces().o39_shifted_ibb_api(ct.byref(k), int(i), int(step), float(fieq), float(gieq), float(rho),
                                  _p(_a(tgt)), _p(_a(u)), _p(_a(v)), _p(_a(w)), _p(_a(T)), _p(spa), _p(out))
    return out


def target_finder(k: O39Consts, code, u, v, w, T, fi, fs_temp):
    """rho, u, v, w, T targets of a wall node (target_finder.f95): its 39 link codes, the
    fields at x + c_j, its post-streaming slots and the freestream temperature."""
    out = np.zeros(5)
    cd = np.ascontiguousarray(code, np.int32)
    _pieces().o39_target_finder_api(ct.byref(k), _p(cd), _p(_a(u)), _p(_a(v)), _p(_a(w)), _p(_a(T)), _p(_a(fi)),
                                    float(fs_temp), _p(out))
    return out


def damp(k: O39Consts, fout, state, lo, hi, fs_fieq):
    """The fout repair of a box without periodic axes (damp_it.f95:64-177): fout and
    state (39, nz, ny, nx); lo, hi the box in the level's index space; outside the box
    fout is fs_fieq and the node type -666.  Returns (repaired fout, count)."""
    f = _a(fout).copy()
    st = np.ascontiguousarray(state, np.int32)
    nz, ny, nx = f.shape[1:]
    lo_a, hi_a = np.asarray(lo, np.int32), np.asarray(hi, np.int32)
    n = _pieces().o39_damp_api(ct.byref(k), _p(f), _p(st), nx, ny, nz, _p(lo_a), _p(hi_a), _p(_a(fs_fieq)))
    return f, int(n)


def flow_vars(k: O39Consts, f, g, w_old):
    """rho, u, v, w, T, P_xx, P_yy, P_zz, P_xy, P_xz, P_yz, press of one node from
    f and g (calculate_flow_variables.f95:192-228; P_zz reads the stored w_old)."""
    out = np.zeros(12)
    _pieces().o39_flow_vars_api(ct.byref(k), _p(_a(f)), _p(_a(g)), float(w_old), _p(out))
    return out


def fieq(shifted, pfd, rho, lm):
    out = np.zeros(Q39)
    _pieces().o39_fieq_api(shifted, pfd, rho, _p(_a(lm)), _p(out))
    return out


def jacobian(shifted, pfd, expo):
    J = np.zeros(NLM * NLM)
    _pieces().o39_jacobian_api(shifted, pfd, _p(_a(expo)), _p(J))
    return J.reshape(NLM, NLM)


def lu_update(J, target, lm):
    lm = _a(lm).copy()
    md = _pieces().o39_lu_api(_p(_a(J)), _p(_a(target)), _p(lm))
    return lm, md


def q_bar(k: O39Consts, fd, u, v, w, T, step):
    out = np.zeros(Q39)
    _pieces().o39_q_bar_api(ct.byref(k), _p(_a(fd)), u, v, w, T, step, _p(out))
    return out


def little_q_bar(k: O39Consts, gd, u, v, w, T, step):
    out = np.zeros(Q39)
    _pieces().o39_little_q_bar_api(ct.byref(k), _p(_a(gd)), u, v, w, T, step, _p(out))
    return out


def collide_node(k: O39Consts, f, g, lm, rho, u, v, w, T, alpha, step):
    fo, go = np.zeros(Q39), np.zeros(Q39)
    _pieces().o39_collide_node_api(ct.byref(k), _p(_a(f)), _p(_a(g)), _p(_a(lm)), rho, u, v, w, T, alpha, step,
                                   _p(fo), _p(go))
    return fo, go
