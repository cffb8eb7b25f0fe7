"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use this
module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as ct
import pathlib

import numpy as np

from . import build as _build

_lib = None


class O27Params(ct.Structure):
    _fields_ = [
        ("nu", ct.c_double),
        ("tol_alpha", ct.c_double),
        ("max_newton", ct.c_int),
        ("alpha_mode", ct.c_int),
        ("fs_feq", ct.c_double * 27),
        ("inl_feq", (ct.c_double * 27) * 8),
        ("outl_feq", (ct.c_double * 27) * 8),
        ("outlet_type", ct.c_int * 8),
    ]


class O27Stats(ct.Structure):
    _fields_ = [
        ("fluid_nodes", ct.c_int64),
        ("newton_iters", ct.c_int64),
        ("fallbacks", ct.c_int64),
        ("errors", ct.c_int64),
        ("max_abs_dH", ct.c_double),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ct.CDLL(str(path))
        vp = ct.c_void_p
        _lib.o27_step.restype = ct.c_int
        _lib.o27_step.argtypes = [ct.c_int, ct.c_int, ct.c_int, vp, vp, vp, ct.POINTER(O27Params), vp, vp,
                                  ct.POINTER(O27Stats)]
        _lib.o27_alpha_newton.restype = ct.c_double
        _lib.o27_alpha_newton.argtypes = [vp, vp, ct.c_double, ct.c_int, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int)]
        _lib.o27_entropy_diff.restype = ct.c_double
        _lib.o27_entropy_diff.argtypes = [vp, vp, ct.c_double]
        _lib.o27_mark_triangles.restype = ct.c_int
        _lib.o27_mark_triangles.argtypes = [ct.c_int, ct.c_int, ct.c_int, vp, ct.c_double, ct.c_int, vp, vp]
        _lib.o27_equilibrium.restype = None
        _lib.o27_equilibrium.argtypes = [ct.c_double, vp, vp]
    return _lib


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def params(nu, fs_feq, inl_feq, outl_feq, outlet_type=(1,) * 8, alpha_mode=1, tol_alpha=1e-12, max_newton=30):
    p = O27Params()
    p.nu = nu
    p.tol_alpha = tol_alpha
    p.max_newton = max_newton
    p.alpha_mode = alpha_mode
    fs = np.asarray(fs_feq, np.float64)
    inl = np.asarray(inl_feq, np.float64)
    outl = np.asarray(outl_feq, np.float64)
    for j in range(27):
        p.fs_feq[j] = fs[j]
        for k in range(8):
            p.inl_feq[k][j] = inl[k, j]
            p.outl_feq[k][j] = outl[k, j]
    for k in range(8):
        p.outlet_type[k] = int(list(outlet_type)[k])
    return p


def step27(state: np.ndarray, fo: np.ndarray, p: O27Params):
    """One oracle time step.  state (27,nz,ny,nx) int32, fo (27,nz,ny,nx) f64.
    Returns (fo_next, alpha, iters, stats dict)."""
    q, nz, ny, nx = fo.shape
    st = np.ascontiguousarray(state, np.int32)
    fin = np.ascontiguousarray(fo, np.float64)
    fout = np.empty_like(fin)
    alpha = np.zeros((nz, ny, nx), np.float64)
    iters = np.zeros((nz, ny, nx), np.int32)
    s = O27Stats()
    rc = lib().o27_step(nx, ny, nz, _p(st), _p(fin), _p(fout), ct.byref(p), _p(alpha), _p(iters), ct.byref(s))
    if rc != 0:
        raise RuntimeError(f"oracle step failed: {rc}")
    return fout, alpha, iters, {k: getattr(s, k) for k, _ in s._fields_}


def alpha_newton(f, d, tol=1e-12, max_it=30):
    f = np.ascontiguousarray(f, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    it = ct.c_int()
    fb = ct.c_int()
    a = lib().o27_alpha_newton(_p(f), _p(d), tol, max_it, ct.byref(it), ct.byref(fb))
    return a, it.value, fb.value


def entropy_diff(f, d, alpha):
    f = np.ascontiguousarray(f, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    return lib().o27_entropy_diff(_p(f), _p(d), alpha)


def equilibrium(rho, u):
    u = np.ascontiguousarray(u, np.float64)
    out = np.zeros(27)
    lib().o27_equilibrium(rho, _p(u), _p(out))
    return out


def mark_triangles(state, origin, dx, tri):
    """Brute-force solid marking and wall fractions (every triangle for every link)."""
    _, nz, ny, nx = state.shape
    o = np.ascontiguousarray(origin, np.float64)
    t = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    rc = lib().o27_mark_triangles(nx, ny, nz, _p(o), dx, t.shape[0], _p(t), _p(state))
    if rc != 0:
        raise RuntimeError("oracle marking failed")
