"""ctypes binding of the C ABI declared in include/elbm_gb300.h.

This is the Python face of the same entry points the Fortran driver binds
through ISO_C_BINDING (fortran/elbm_gb300_iface.f90).  There is no fallback:
if libelbm_gb300.so is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes as ct
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libelbm_gb300.so"

ELBM_OK = 0
ELBM_E_ARG = -1
ELBM_E_CUDA = -2
ELBM_E_UNSUPPORTED = -3
ELBM_E_STATE = -4
ELBM_E_NUMERIC = -5
ELBM_KERNEL_VARIANTS = 10  # FP32 D3Q27 step-kernel variants (elbm_autotune's timing array)

ELBM_ST_NAN = 0x1
ELBM_ST_NEWTON_FALLBACK = 0x2
ELBM_ST_NEG_POP = 0x4
ELBM_ST_DH_TOL = 0x8

ELBM_D3Q27 = 27
ELBM_D3Q39 = 39
ELBM_STORE_FP64 = 0
ELBM_STORE_FP32_DEV = 1
ELBM_ALPHA_FIXED2 = 0
ELBM_ALPHA_NEWTON = 1
ELBM_ALPHA_LEARNED = 2

# every function the header declares, with its ctypes signature
_c_int, _c_double, _vp = ct.c_int, ct.c_double, ct.c_void_p


class D3Q27Params(ct.Structure):
    _fields_ = [
        ("nu", ct.c_double),
        ("tol_alpha", ct.c_double),
        ("tol_dH", ct.c_double),
        ("max_newton", ct.c_int32),
        ("alpha_mode", ct.c_int32),
        ("check_dH", ct.c_int32),
        ("record_alpha", ct.c_int32),
        ("outlet_type", ct.c_int32 * 8),
        ("fs_feq", ct.c_double * 27),
        ("inl_feq", (ct.c_double * 27) * 8),
        ("outl_feq", (ct.c_double * 27) * 8),
        ("damp", ct.c_int32),
        ("pad_damp", ct.c_int32),
    ]


class D3Q39Params(ct.Structure):
    _fields_ = [(n, ct.c_int32) for n in ("shifted", "primary_flow_dir", "turbulent", "lvl", "startup_timesteps",
                                         "max_lm_iters", "periodic", "timestep", "damp", "pad")] + [
        (n, ct.c_double) for n in ("gama", "t_ref", "rho_ref", "p_ref", "mu_ref", "kappa_ref", "gas_const_R",
                                   "const_vol", "const_press", "molec_weight", "dt", "elbm_epsilon", "init_beta_1",
                                   "init_beta_2", "beta_1_scaling", "beta_2_scaling")] + [
        ("su_lm", ct.c_double * 13)]


def make_d3q39_params(consts, timestep=0, periodic=7, damp=1) -> D3Q39Params:
    """D3Q39Params from a d3q39_setup.D3Q39Consts."""
    p = D3Q39Params()
    for name, _ in D3Q39Params._fields_:
        if name == "periodic":
            p.periodic = periodic
        elif name == "timestep":
            p.timestep = timestep
        elif name == "damp":
            p.damp = damp
        elif name == "pad":
            p.pad = 0
        elif name == "su_lm":
            for r, v in enumerate(consts.su_lm):
                p.su_lm[r] = v
        else:
            setattr(p, name, getattr(consts, name))
    return p


class D3Q39Bc(ct.Structure):
    _fields_ = [("inlet_type", ct.c_int32 * 8), ("outlet_type", ct.c_int32 * 8),
                ("fs_fieq", ct.c_double * 39), ("fs_gieq", ct.c_double * 39),
                ("inl_fieq", (ct.c_double * 39) * 8), ("inl_gieq", (ct.c_double * 39) * 8),
                ("outl_fieq", (ct.c_double * 39) * 8), ("outl_gieq", (ct.c_double * 39) * 8),
                ("fs_u", ct.c_double), ("fs_v", ct.c_double), ("fs_w", ct.c_double), ("fs_temp", ct.c_double)]


def mlp_init_weights(seed: int = 0) -> np.ndarray:
    """Initial weights of the 27-64-64-1 alpha network in the library's packed order
    (W1 27x64 row-major, b1, W2 64x64, b2, w3, b3): normal draws scaled by 1/sqrt(fan-in),
    zero biases."""
    rng = np.random.default_rng(seed)
    ni, nh = 27, 64
    w1 = rng.normal(0, 1 / np.sqrt(ni), (ni, nh))
    w2 = rng.normal(0, 1 / np.sqrt(nh), (nh, nh))
    w3 = rng.normal(0, 1 / np.sqrt(nh), nh)
    return np.concatenate([w1.ravel(), np.zeros(nh), w2.ravel(), np.zeros(nh), w3, np.zeros(1)]).astype(np.float32)


def make_d3q39_bc(inlet_type, outlet_type, fs_f, fs_g, inl_f, inl_g, outl_f, outl_g,
                  fs_uvwT=(0.0, 0.0, 0.0, 0.0)) -> D3Q39Bc:
    """Boundary equilibria (f and g), inlet/outlet types and the freestream velocity and
    temperature of a D3Q39 level with link codes."""
    b = D3Q39Bc()
    b.fs_u, b.fs_v, b.fs_w, b.fs_temp = (float(x) for x in fs_uvwT)
    for k in range(8):
        b.inlet_type[k] = int(inlet_type[k])
        b.outlet_type[k] = int(outlet_type[k])
        for i in range(39):
            b.inl_fieq[k][i], b.inl_gieq[k][i] = inl_f[k][i], inl_g[k][i]
            b.outl_fieq[k][i], b.outl_gieq[k][i] = outl_f[k][i], outl_g[k][i]
    for i in range(39):
        b.fs_fieq[i], b.fs_gieq[i] = fs_f[i], fs_g[i]
    return b


class Plot3DHeader(ct.Structure):
    _fields_ = [(n, ct.c_double) for n in ("mach", "reynolds", "time", "gama", "t_ref", "stag_temperature",
                                           "const_vol", "const_press", "non_dim_R")]


class Stats(ct.Structure):
    _fields_ = [
        ("node_updates", ct.c_int64),
        ("newton_iters", ct.c_int64),
        ("exact_path_nodes", ct.c_int64),
        ("fallbacks", ct.c_int64),
        ("status", ct.c_uint32),
        ("pad", ct.c_uint32),
        ("max_abs_dH", ct.c_double),
        ("dh_over_tol", ct.c_int64),
        ("guess_misses", ct.c_int64),
        ("kernel_ms", ct.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


SIGNATURES = {
    "elbm_create": (_c_int, [_c_int, ct.POINTER(_vp)]),
    "elbm_destroy": (None, [_vp]),
    "elbm_last_error_string": (ct.c_char_p, [_vp]),
    "elbm_level_register": (_c_int, [_vp, _c_int, _c_int, _c_int, _c_int, _vp, _c_int]),
    "elbm_set_d3q27_params": (_c_int, [_vp, _c_int, ct.POINTER(D3Q27Params)]),
    "elbm_set_links": (_c_int, [_vp, _c_int, _c_int, _vp, _c_int]),
    "elbm_upload_level": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "elbm_download_level": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "elbm_download_alpha": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "elbm_level_step": (_c_int, [_vp, _c_int, _c_int, ct.POINTER(Stats)]),
    "elbm_sync": (_c_int, [_vp]),
    "elbm_set_d3q39_params": (_c_int, [_vp, _c_int, ct.POINTER(D3Q39Params)]),
    "elbm_upload_level39": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp, _vp]),
    "elbm_download_level39": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "elbm_upload_macro39": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "elbm_init_level39": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp]),
    "elbm_ggm_tags": (_c_int, [_vp, _c_int, _c_int, _c_int, _c_int, _c_double, _vp, _vp, _vp]),
    "elbm_ggm_tags_pgs": (_c_int, [_vp, _c_int, _c_int, _c_int, _c_int, _c_double, _c_double, _c_int, _vp, _vp, _vp]),
    "elbm_write_plot3d": (_c_int, [_vp, _c_int, ct.c_char_p, ct.c_char_p, _vp, _c_double, _vp]),
    "elbm_mic_sample": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _vp, _vp]),
    "elbm_checkpoint_write": (_c_int, [_vp, _c_int, ct.c_char_p]),
    "elbm_checkpoint_read": (_c_int, [_vp, _c_int, ct.c_char_p]),
    "elbm_d3q39_equilibrium": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "elbm_upload_level_noalloc": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "elbm_autotune": (_c_int, [_vp, _c_int, _c_int, _vp, _vp]),
    "elbm_set_kernel_variant": (_c_int, [_vp, _c_int, _c_int]),
    "elbm_interlevel_setup": (_c_int, [_vp, _c_int]),
    "elbm_fill_fine_ghosts": (_c_int, [_vp, _c_int, _vp]),
    "elbm_average_down": (_c_int, [_vp, _c_int]),
    "elbm_amr_run": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "elbm_damp_level": (_c_int, [_vp, _c_int, _vp]),
    "elbm_set_links39": (_c_int, [_vp, _c_int, _c_int, _vp, _c_int, _vp]),
    "elbm_links39_tables": (_c_int, [_c_int, _c_int, _c_int, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp,
                                     _vp, _vp, ct.c_int64, _vp]),
    "elbm_mark_triangles": (_c_int, [_c_int, _c_int, _c_int, _vp, _c_double, _c_int, _vp, _vp]),
    "elbm_mark_triangles_gpu": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _c_double, _c_int, _vp, _vp]),
    "elbm_mark_triangles39": (_c_int, [_c_int, _c_int, _c_int, _vp, _c_double, _c_int, _vp, _c_int, _c_int, _c_int,
                                       _vp]),
    "elbm_mark_triangles39_gpu": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _c_double, _c_int, _vp, _c_int, _c_int,
                                           _c_int, _vp]),
    "elbm_alpha_harvest": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, ct.c_int64, _vp]),
    "elbm_alpha_mlp_infer": (_c_int, [_vp, _vp, _vp, ct.c_int64, _vp, _vp]),
    "elbm_alpha_mlp_grad": (_c_int, [_vp, _vp, _vp, ct.c_int64, _vp, _vp]),
    "elbm_alpha_mlp_train": (_c_int, [_vp, _vp, ct.c_int64, _c_int, _c_int, ct.c_float, ct.c_uint64, _vp, _vp]),
    "elbm_set_alpha_mlp": (_c_int, [_vp, _c_int, _vp]),
}
MLP_PARAMS = 6017
MLP_RECORD = 29

_lib = None


def load(path: pathlib.Path | str | None = None) -> ct.CDLL:
    """Load libelbm_gb300.so (built in-tree by build.py).  Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p.name} is not built; run the package build (nvcc for sm_103a) first")
    lib = ct.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class ElbmError(RuntimeError):
    def __init__(self, rc: int, msg: str):
        super().__init__(f"elbm error {rc}: {msg}")
        self.rc = rc


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_vp)


def _at_least(a: np.ndarray, need: int, name: str) -> np.ndarray:
    """a, if it holds at least need values: the library reads (or writes) exactly need
    values through the pointer, so a shorter array would be overrun."""
    if a.size < need:
        raise ValueError(f"{name}: {a.size} values given, the call reads or writes {need}")
    return a


def make_d3q27_params(nu, tol_alpha=1e-12, tol_dH=1e-10, max_newton=30, alpha_mode=ELBM_ALPHA_NEWTON, check_dH=0,
                      record_alpha=0, outlet_type=(1,) * 8, fs_feq=None, inl_feq=None, outl_feq=None,
                      damp=0) -> D3Q27Params:
    p = D3Q27Params()
    p.damp = damp
    p.nu = nu
    p.tol_alpha = tol_alpha
    p.tol_dH = tol_dH
    p.max_newton = max_newton
    p.alpha_mode = alpha_mode
    p.check_dH = check_dH
    p.record_alpha = record_alpha
    for k in range(8):
        p.outlet_type[k] = int(list(outlet_type)[k])
    z = np.zeros(27)
    fs = np.asarray(fs_feq if fs_feq is not None else z, np.float64)
    inl = np.asarray(inl_feq if inl_feq is not None else np.zeros((8, 27)), np.float64)
    outl = np.asarray(outl_feq if outl_feq is not None else np.zeros((8, 27)), np.float64)
    for j in range(27):
        p.fs_feq[j] = fs[j]
        for k in range(8):
            p.inl_feq[k][j] = inl[k, j]
            p.outl_feq[k][j] = outl[k, j]
    return p


def links39_tables(state: np.ndarray, periodic: int, shifted: int, primary_flow_dir: int, inlet_type, outlet_type,
                   ngrow_state: int = 0):
    """Host-side D3Q39 link tables of a box state (39, nz, ny, nx): (ntype, record nodes, words (nrec, 39))."""
    st = np.ascontiguousarray(state, np.int32)
    g = ngrow_state
    nz, ny, nx = (st.shape[1] - 2 * g, st.shape[2] - 2 * g, st.shape[3] - 2 * g)
    it = np.ascontiguousarray(inlet_type, np.int32)
    ot = np.ascontiguousarray(outlet_type, np.int32)
    ntype = np.zeros(nx * ny * nz, np.uint8)
    cap = nx * ny * nz
    rec = np.zeros(cap, np.int32)
    words = np.zeros((cap, 39), np.uint32)
    nrec = ct.c_int64(0)
    rc = load().elbm_links39_tables(nx, ny, nz, _ptr(st), g, periodic, shifted, primary_flow_dir, _ptr(it), _ptr(ot),
                                    _ptr(ntype), _ptr(rec), _ptr(words), cap, ct.byref(nrec))
    if rc != ELBM_OK:
        raise ElbmError(rc, "elbm_links39_tables failed")
    return ntype.reshape(nz, ny, nx), rec[:nrec.value], words[:nrec.value]


def mark_triangles(state: np.ndarray, origin, dx: float, tri: np.ndarray) -> None:
    """Mark solid nodes and wall-link fractions of a closed triangulated surface
    in a state array (27, nz, ny, nx), in place (host code, no GPU needed)."""
    lib = load()
    assert state.dtype == np.int32 and state.flags.c_contiguous and state.shape[0] == 27
    _, nz, ny, nx = state.shape
    o = np.ascontiguousarray(origin, np.float64)
    t = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    rc = lib.elbm_mark_triangles(nx, ny, nz, _ptr(o), dx, t.shape[0], _ptr(t), _ptr(state))
    if rc != ELBM_OK:
        raise ElbmError(rc, "elbm_mark_triangles failed")


def mark_triangles39(state: np.ndarray, origin, dx: float, tri: np.ndarray, shifted: int = 1,
                     primary_flow_dir: int = 1, periodic: int = 0) -> None:
    """D3Q39 solid nodes and wall links of a closed triangulated surface in a state
    array (39, nz, ny, nx), in place (host code, no GPU needed)."""
    lib = load()
    assert state.dtype == np.int32 and state.flags.c_contiguous and state.shape[0] == 39
    _, nz, ny, nx = state.shape
    o = np.ascontiguousarray(origin, np.float64)
    t = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    rc = lib.elbm_mark_triangles39(nx, ny, nz, _ptr(o), dx, t.shape[0], _ptr(t), shifted, primary_flow_dir, periodic,
                                   _ptr(state))
    if rc != ELBM_OK:
        raise ElbmError(rc, "elbm_mark_triangles39 failed")


class Context:
    """One elbm_ctx (one CUDA device, one stream)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _vp()
        rc = self.lib.elbm_create(device, ct.byref(h))
        if rc != ELBM_OK:
            raise ElbmError(rc, "elbm_create failed (no usable CUDA device?)")
        self.h = h
        self._boxes = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.elbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != ELBM_OK:
            raise ElbmError(rc, self.lib.elbm_last_error_string(self.h).decode())

    def level_register(self, lvl, lattice, storage, boxes, ngrow=0):
        lo_hi = np.ascontiguousarray(np.asarray(boxes, np.int32).reshape(-1, 6))
        self._check(self.lib.elbm_level_register(self.h, lvl, lattice, storage, lo_hi.shape[0], _ptr(lo_hi), ngrow))
        self._boxes[lvl] = (lo_hi.copy(), ngrow, lattice)

    def _fab_values(self, lvl, box, ncomp, ngrow=None):
        """Values of an ncomp-component FAB of a registered box (ghost width ngrow,
        default the level's), or None when the level or box is unknown here (the
        library reports that)."""
        if lvl not in self._boxes or not (0 <= box < self._boxes[lvl][0].shape[0]):
            return None
        lo_hi, g0, _ = self._boxes[lvl]
        g = g0 if ngrow is None else ngrow
        n = lo_hi[box, 3:] - lo_hi[box, :3] + 1 + 2 * g
        return int(ncomp) * int(n[0]) * int(n[1]) * int(n[2])

    def _fab(self, lvl, box, ncomp, arr, name, dtype=np.float64, ngrow=None):
        a = np.ascontiguousarray(arr, dtype)
        need = self._fab_values(lvl, box, ncomp, ngrow)
        return a if need is None else _at_least(a, need, name)

    def box_shape(self, lvl, box=0, ghosts=True):
        lo_hi, ngrow, _ = self._boxes[lvl]
        g = ngrow if ghosts else 0
        lo, hi = lo_hi[box, :3], lo_hi[box, 3:]
        n = hi - lo + 1 + 2 * g
        return int(n[2]), int(n[1]), int(n[0])

    def set_d3q27_params(self, lvl, params: D3Q27Params):
        self._check(self.lib.elbm_set_d3q27_params(self.h, lvl, ct.byref(params)))

    def set_links(self, lvl, box, state: np.ndarray, ngrow_state=0):
        st = self._fab(lvl, box, 27, state, "state", np.int32, ngrow_state)
        self._check(self.lib.elbm_set_links(self.h, lvl, box, _ptr(st), ngrow_state))

    def upload(self, lvl, box, f: np.ndarray):
        fa = self._fab(lvl, box, 27, f, "fout")
        self._check(self.lib.elbm_upload_level(self.h, lvl, box, _ptr(fa)))

    def download(self, lvl, box=0, out: np.ndarray | None = None) -> np.ndarray:
        q = self._boxes[lvl][2]
        if out is None:
            out = np.zeros((q,) + self.box_shape(lvl, box), np.float64)
        elif out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out: a C-contiguous float64 array is written in place")
        else:
            need = self._fab_values(lvl, box, q)
            if need is not None:
                _at_least(out, need, "out")
        self._check(self.lib.elbm_download_level(self.h, lvl, box, _ptr(out)))
        return out

    def download_alpha(self, lvl, box=0) -> np.ndarray:
        out = np.zeros(self.box_shape(lvl, box, ghosts=False), np.float64)
        self._check(self.lib.elbm_download_alpha(self.h, lvl, box, _ptr(out)))
        return out

    def step(self, lvl, nsteps=1, want_stats=True) -> dict | None:
        if want_stats:
            st = Stats()
            self._check(self.lib.elbm_level_step(self.h, lvl, nsteps, ct.byref(st)))
            return st.as_dict()
        self._check(self.lib.elbm_level_step(self.h, lvl, nsteps, None))
        return None

    def set_d3q39_params(self, lvl, params: D3Q39Params):
        self._check(self.lib.elbm_set_d3q39_params(self.h, lvl, ct.byref(params)))

    def set_links39(self, lvl, box, state: np.ndarray, bc: D3Q39Bc, ngrow_state=0):
        st = self._fab(lvl, box, 39, state, "state", np.int32, ngrow_state)
        self._check(self.lib.elbm_set_links39(self.h, lvl, box, _ptr(st), ngrow_state, ct.byref(bc)))

    def upload39(self, lvl, box, fout, gout, lm, w_vel):
        arrs = [self._fab(lvl, box, q, a, nm) for q, a, nm in ((39, fout, "fout"), (39, gout, "gout"), (13, lm, "lm"),
                                                                (1, w_vel, "w_vel"))]
        self._check(self.lib.elbm_upload_level39(self.h, lvl, box, *map(_ptr, arrs)))

    def ggm_tags(self, lvl, box, variable, scheme, limit, pgs_sensitivity=None, pgs_reach=-1):
        """(tags, ggm, ntagged) of a D3Q39 box, arrays (nz, ny, nx); with pgs_sensitivity
        and pgs_reach >= 0 the predictive splitting tags are added."""
        shp = self.box_shape(lvl, box, ghosts=False)
        tags = np.zeros(shp, np.uint8)
        ggm = np.zeros(shp)
        n = ct.c_int64(0)
        if pgs_sensitivity is None:
            self._check(self.lib.elbm_ggm_tags(self.h, lvl, box, variable, scheme, limit, _ptr(tags), _ptr(ggm),
                                               ct.byref(n)))
        else:
            self._check(self.lib.elbm_ggm_tags_pgs(self.h, lvl, box, variable, scheme, limit, pgs_sensitivity,
                                                   pgs_reach, _ptr(tags), _ptr(ggm), ct.byref(n)))
        return tags, ggm, n.value

    def write_plot3d(self, lvl, grid_path, data_path, origin, dx, header: Plot3DHeader):
        o = np.ascontiguousarray(origin, np.float64)
        self._check(self.lib.elbm_write_plot3d(self.h, lvl, str(grid_path).encode(), str(data_path).encode(), _ptr(o),
                                               dx, ct.byref(header)))

    def mic_sample(self, lvl, box, nodes, weights):
        """nodes, weights: (nmic, 8); returns (nmic, 6): pressure, T, rho, u, v, w."""
        nd = np.ascontiguousarray(nodes, np.int32)
        wt = np.ascontiguousarray(weights, np.float64)
        out = np.zeros((nd.shape[0], 6))
        self._check(self.lib.elbm_mic_sample(self.h, lvl, box, nd.shape[0], _ptr(nd), _ptr(wt), _ptr(out)))
        return out

    def mark_triangles(self, state: np.ndarray, origin, dx: float, tri: np.ndarray) -> None:
        """elbm_mark_triangles on this context's device (state (27, nz, ny, nx) int32, updated in place)."""
        assert state.dtype == np.int32 and state.flags.c_contiguous
        nz, ny, nx = state.shape[1:]
        o = np.ascontiguousarray(origin, np.float64)
        t = np.ascontiguousarray(tri, np.float64)
        self._check(self.lib.elbm_mark_triangles_gpu(self.h, nx, ny, nz, _ptr(o), dx, t.shape[0], _ptr(t),
                                                     _ptr(state)))

    def mark_triangles39(self, state: np.ndarray, origin, dx: float, tri: np.ndarray, shifted: int = 1,
                         primary_flow_dir: int = 1, periodic: int = 0) -> None:
        """elbm_mark_triangles39 on this context's device (state (39, nz, ny, nx) int32, updated in place)."""
        assert state.dtype == np.int32 and state.flags.c_contiguous and state.shape[0] == 39
        nz, ny, nx = state.shape[1:]
        o = np.ascontiguousarray(origin, np.float64)
        t = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
        self._check(self.lib.elbm_mark_triangles39_gpu(self.h, nx, ny, nz, _ptr(o), dx, t.shape[0], _ptr(t), shifted,
                                                       primary_flow_dir, periodic, _ptr(state)))

    def checkpoint_write(self, lvl, path):
        self._check(self.lib.elbm_checkpoint_write(self.h, lvl, str(path).encode()))

    def checkpoint_read(self, lvl, path):
        self._check(self.lib.elbm_checkpoint_read(self.h, lvl, str(path).encode()))

    def init_level39(self, lvl, box, macro, lm_start):
        """Equilibrium initial state of a D3Q39 box from rho, u, v, w, T (5, nz, ny, nx) on the
        device; returns the number of nodes whose multiplier Newton hit the cap."""
        m = self._fab(lvl, box, 5, macro, "macro")
        l0 = _at_least(np.ascontiguousarray(lm_start, np.float64), 13, "lm_start")
        capped = ct.c_int64(0)
        self._check(self.lib.elbm_init_level39(self.h, lvl, box, _ptr(m), _ptr(l0), ct.byref(capped)))
        return capped.value

    def d3q39_equilibrium(self, params, rho, u, v, w, T, lm_start):
        """(lm, fieq, gieq) of one state: the multiplier Newton from lm_start."""
        m = np.array([rho, u, v, w, T], np.float64)
        lm = _at_least(np.ascontiguousarray(lm_start, np.float64).copy(), 13, "lm_start")
        f = np.zeros(39)
        g = np.zeros(39)
        self._check(self.lib.elbm_d3q39_equilibrium(self.h, ct.byref(params), _ptr(m), _ptr(lm), _ptr(f), _ptr(g)))
        return lm, f, g

    def upload_macro39(self, lvl, box, macro):
        """rho, u, v, w, T (5, nz, ny, nx) the next step starts from (after upload39)."""
        m = self._fab(lvl, box, 5, macro, "macro")
        self._check(self.lib.elbm_upload_macro39(self.h, lvl, box, _ptr(m)))

    def download39(self, lvl, box=0):
        """Returns dict with fout, gout, lm, w_vel, alpha, macro (FAB layouts)."""
        shp = self.box_shape(lvl, box)
        out = {"fout": np.zeros((39,) + shp), "gout": np.zeros((39,) + shp), "lm": np.zeros((13,) + shp),
               "w_vel": np.zeros(shp), "alpha": np.zeros(shp), "macro": np.zeros((5,) + shp)}
        self._check(self.lib.elbm_download_level39(self.h, lvl, box, *(_ptr(out[k]) for k in
                                                                      ("fout", "gout", "lm", "w_vel", "alpha",
                                                                       "macro"))))
        return out

    def autotune(self, lvl, reps=3):
        """Pick the fastest step-kernel variant for the level; returns (index, ms per variant)."""
        chosen = ct.c_int(0)
        ms = np.zeros(ELBM_KERNEL_VARIANTS)
        self._check(self.lib.elbm_autotune(self.h, lvl, reps, ct.byref(chosen), _ptr(ms)))
        return chosen.value, ms

    def interlevel_setup(self, lvl):
        self._check(self.lib.elbm_interlevel_setup(self.h, lvl))

    def fill_fine_ghosts(self, lvl):
        """Explosion into level lvl from lvl - 1; returns the number of nodes set to equilibrium."""
        r = ct.c_int64(0)
        self._check(self.lib.elbm_fill_fine_ghosts(self.h, lvl, ct.byref(r)))
        return r.value

    def average_down(self, lvl):
        self._check(self.lib.elbm_average_down(self.h, lvl))

    def damp_level(self, lvl):
        """Repair negative populations of the level's current state; returns how many changed."""
        r = ct.c_int64(0)
        self._check(self.lib.elbm_damp_level(self.h, lvl, ct.byref(r)))
        return r.value

    def amr_run(self, nlev, ncycles):
        """ncycles coarse steps of levels 0 .. nlev-1 with 2:1 sub-cycling (CUDA graph); returns stats."""
        st = Stats()
        self._check(self.lib.elbm_amr_run(self.h, nlev, ncycles, ct.byref(st)))
        return st.as_dict()

    def set_kernel_variant(self, lvl, variant):
        self._check(self.lib.elbm_set_kernel_variant(self.h, lvl, variant))

    def alpha_harvest(self, lvl, nsteps, stride, capacity):
        rec = np.zeros((capacity, MLP_RECORD), np.float32)
        cnt = ct.c_int64(0)
        self._check(self.lib.elbm_alpha_harvest(self.h, lvl, nsteps, stride, _ptr(rec), capacity, ct.byref(cnt)))
        return rec[:cnt.value]

    def alpha_mlp_infer(self, weights, x):
        """Tensor-core network outputs for feature rows x (n, 27); returns (out, status)."""
        w = _at_least(np.ascontiguousarray(weights, np.float32), MLP_PARAMS, "weights")
        xs = np.ascontiguousarray(x, np.float32).reshape(-1, 27)
        out = np.zeros(xs.shape[0], np.float32)
        st = ct.c_uint32(0)
        self._check(self.lib.elbm_alpha_mlp_infer(self.h, _ptr(w), _ptr(xs), xs.shape[0], _ptr(out), ct.byref(st)))
        return out, st.value

    def alpha_mlp_grad(self, weights, records):
        w = _at_least(np.ascontiguousarray(weights, np.float32), MLP_PARAMS, "weights")
        r = np.ascontiguousarray(records, np.float32).reshape(-1, MLP_RECORD)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = ct.c_double(0)
        self._check(self.lib.elbm_alpha_mlp_grad(self.h, _ptr(w), _ptr(r), r.shape[0], _ptr(g), ct.byref(loss)))
        return g, loss.value

    def alpha_mlp_train(self, records, weights, epochs=4, batch=4096, lr=1e-3, seed=0):
        w = _at_least(np.ascontiguousarray(weights, np.float32).copy(), MLP_PARAMS, "weights")
        r = np.ascontiguousarray(records, np.float32).reshape(-1, MLP_RECORD)
        hist = np.zeros(epochs)
        self._check(self.lib.elbm_alpha_mlp_train(self.h, _ptr(r), r.shape[0], epochs, batch, lr, seed, _ptr(w),
                                                  _ptr(hist)))
        return w, hist

    def set_alpha_mlp(self, lvl, weights):
        w = _at_least(np.ascontiguousarray(weights, np.float32), MLP_PARAMS, "weights")
        self._check(self.lib.elbm_set_alpha_mlp(self.h, lvl, _ptr(w)))

    def sync(self):
        self._check(self.lib.elbm_sync(self.h))
