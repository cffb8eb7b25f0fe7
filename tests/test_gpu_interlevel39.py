"""Coarse-fine transfer between two D3Q39 levels on the GPU against the CPU
restatement: the explosion into the fine level's ghost nodes
(interlevel_interpolation.f95:364-440: nodal means of f, g, multipliers, rho and
T; populations with f < 0, g < 0 or NaN from the coarse equilibrium; the
node's moments, multiplier solve and alpha), the coalescence onto the coarse
level (fine_to_coarse.f95:13-45), and a two-level run in the reference's
sub-cycle order.  Tolerance 1e-12 relative in f and g after one transfer (the
multiplier Newton of each ghost node), exact for the coalescence copies."""
import math

import numpy as np
import pytest

from oracle import interlevel as il

pytestmark = pytest.mark.gpu

GHOST = 10000000
COARSE = ((0, 0, 0), (15, 11, 11))        # coarse index space, periodic on every axis
FINE_VALID = ((8, 6, 6), (23, 17, 17))    # fine index space (coarse 4..11.5, 3..8.5, 3..8.5)
SHELL = 3                                 # ghost layers: the D3Q39 stencil reaches 3 nodes


@pytest.fixture(scope="module")
def o39():
    from oracle import oracle39

    oracle39.lib()
    return oracle39


def _fine_box():
    (x0, y0, z0), (x1, y1, z1) = FINE_VALID
    return (x0 - SHELL, y0 - SHELL, z0 - SHELL), (x1 + SHELL, y1 + SHELL, z1 + SHELL)


def _dims(lo, hi):
    return tuple(hi[a] - lo[a] + 1 for a in range(3))


def _init_level(o39, k, c, lm0, shape, seed):
    """Oracle level at equilibrium of smoothly varying fields with a little noise."""
    nz, ny, nx = shape
    lev = o39.Level39(nx, ny, nz)
    rng = np.random.default_rng(seed)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                rho = 1.0 + 0.02 * math.sin(0.4 * x + 0.3 * y) + 0.005 * rng.uniform(-1, 1)
                u = c.mach * (1 + 0.02 * math.cos(0.3 * z) + 0.005 * rng.uniform(-1, 1))
                v, w = 0.01 * rng.uniform(-1, 1, 2)
                T = c.temperature * (1 + 0.01 * math.sin(0.2 * y + 0.5 * z))
                lm, f, g, _ = o39.init_node(k, rho, u, v, w, T, lm0)
                lev.fout[:, z, y, x], lev.gout[:, z, y, x], lev.lm[:, z, y, x] = f, g, lm
                lev.rho[z, y, x], lev.u[z, y, x], lev.v[z, y, x], lev.w_vel[z, y, x] = rho, u, v, w
                lev.temp[z, y, x] = T
    return lev


def _macro(lev):
    return np.stack([lev.rho, lev.u, lev.v, lev.w_vel, lev.temp])


def _case(pkg, o39, shifted):
    s39, cap = pkg.d3q39_setup, pkg.capi
    kw = dict(v_inf_ms=0.8 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=bool(shifted))
    cc, cf = s39.wedge_case_consts(**kw), s39.wedge_case_consts(lvl=1, **kw)
    kc, kf = o39.consts(cc), o39.consts(cf)
    lm0 = s39.freestream_start_lm(cc)
    zero = {f: 0 for f in ("x-", "x+", "y-", "y+", "z-", "z+")}
    nc, nf = _dims(*COARSE), _dims(*_fine_box())
    stc = s39.box_state39(*nc, zero, shifted, periodic=7)
    stf = s39.box_state39(*nf, zero, shifted, periodic=0)
    ghost = np.ones(nf[::-1], bool)
    ghost[SHELL:-SHELL, SHELL:-SHELL, SHELL:-SHELL] = False
    stf[0][ghost] = GHOST
    levc = _init_level(o39, kc, cc, lm0, nc[::-1], 21)
    levf = _init_level(o39, kf, cf, lm0, nf[::-1], 22)
    _, f, g, _ = o39.init_node(kc, 1.0, cc.mach, 0.0, 0.0, cc.temperature, lm0)
    bc_args = ([1] * 8, [1] * 8, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8, (cc.mach, 0.0, 0.0, cc.temperature))
    ctx = cap.Context(0)
    lof = _fine_box()
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [list(COARSE[0]) + list(COARSE[1])])
    ctx.level_register(1, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [list(lof[0]) + list(lof[1])])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(cc, timestep=0, periodic=7, damp=0))
    ctx.set_d3q39_params(1, cap.make_d3q39_params(cf, timestep=0, periodic=0, damp=0))
    ctx.set_links39(0, 0, stc, cap.make_d3q39_bc(*bc_args))
    ctx.set_links39(1, 0, stf, cap.make_d3q39_bc(*bc_args))
    for lvl, lev in ((0, levc), (1, levf)):
        ctx.upload39(lvl, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
        ctx.upload_macro39(lvl, 0, _macro(lev))
    ctx.interlevel_setup(1)
    return dict(ctx=ctx, kc=kc, kf=kf, stc=stc, stf=stf, ghost=ghost, levc=levc, levf=levf,
                bc=o39.bc(*bc_args), bc_args=bc_args)


def _as_dict(out):
    return {"f": out["fout"].copy(), "g": out["gout"].copy(), "lm": out["lm"].copy(), "w": out["w_vel"].copy(),
            "alpha": out["alpha"].copy(), "macro": out["macro"].copy()}


@pytest.mark.parametrize("shifted", [1, 0])
def test_d3q39_explosion_and_coalescence_match_oracle(pkg, o39, built_lib, shifted):
    S = _case(pkg, o39, shifted)
    ctx, kf, ghost = S["ctx"], S["kf"], S["ghost"]
    ctx.step(0, 2, want_stats=False)  # a coarse state off equilibrium
    ctx.step(1, 1, want_stats=False)  # the fine level's odd step: its counter is now 1
    cd = ctx.download39(0)
    # plant populations the explosion must replace: a strongly negative f and a NaN g under the ghost shell
    cd["fout"][5, 4, 3, 3] = -0.5
    cd["gout"][17, 9, 9, 12] = np.nan
    ctx.upload39(0, 0, cd["fout"], cd["gout"], cd["lm"], cd["w_vel"])
    ctx.upload_macro39(0, 0, cd["macro"])
    coarse, fine0 = _as_dict(ctx.download39(0)), _as_dict(ctx.download39(1))
    step = 1
    rep = ctx.fill_fine_ghosts(1)
    got = _as_dict(ctx.download39(1))
    ref = {k: v.copy() for k, v in fine0.items()}
    rep_ref, capped = il.explode39(kf, step, coarse, COARSE[0], ref, _fine_box()[0], ghost)
    assert capped == 0 and rep == rep_ref > 0
    for name in ("f", "g"):
        rel = np.max(np.abs(got[name] - ref[name]) / np.abs(ref[name]))
        assert rel <= 1e-12, (name, rel)
    assert np.max(np.abs(got["lm"] - ref["lm"])) <= 1e-12 * np.max(np.abs(ref["lm"]))
    assert np.max(np.abs(got["macro"] - ref["macro"]) / np.maximum(np.abs(ref["macro"]), 1e-3)) <= 1e-12
    # alpha: the closed form divides by each population and takes the difference of a quadratic's
    # terms; at the ghost nodes next to the planted f = -0.5 it moves ~1e-11 for a 1e-15 change in f
    assert np.max(np.abs(got["alpha"] - ref["alpha"])) <= 1e-10
    assert np.max(np.abs(got["w"] - ref["w"])) <= 1e-14
    for name in ("f", "g", "lm", "w", "macro"):  # valid fine nodes untouched
        assert np.array_equal(got[name][..., ~ghost], fine0[name][..., ~ghost]), name
    ctx.average_down(1)
    gotc = _as_dict(ctx.download39(0))
    refc = {k: v.copy() for k, v in coarse.items()}
    il.average_down39(got, _fine_box()[0], ~ghost, refc, COARSE[0], np.ones(S["stc"].shape[1:], bool))
    for name in ("f", "g", "lm", "w", "alpha", "macro"):
        assert np.array_equal(gotc[name], refc[name], equal_nan=True), name
    assert not np.array_equal(gotc["f"], coarse["f"], equal_nan=True)  # some coarse nodes were overwritten
    ctx.close()


def test_d3q39_two_level_subcycle_matches_oracle(pkg, o39, built_lib):
    """Three coarse cycles: a coarse step, two fine steps with the explosion after the
    fine level's odd step, the coalescence after its even one (loop.f95:94-147)."""
    S = _case(pkg, o39, 1)
    ctx, kc, kf, levc, levf = S["ctx"], S["kc"], S["kf"], S["levc"], S["levf"]
    ghost = S["ghost"]
    pcf, pcg = levc.fout.copy(), levc.gout.copy()
    pff, pfg = levf.fout.copy(), levf.gout.copy()
    cycles = 3
    for cyc in range(cycles):
        ctx.step(0, 1, want_stats=False)
        o39.step_links(kc, levc, cyc, S["stc"], 7, S["bc"], pcf, pcg)
        for kk in range(2):
            ctx.step(1, 1, want_stats=False)
            o39.step_links(kf, levf, 2 * cyc + kk, S["stf"], 0, S["bc"], pff, pfg)
            if kk == 0:
                ctx.fill_fine_ghosts(1)
                cdict = {"f": levc.fout, "g": levc.gout, "lm": levc.lm, "macro": _macro(levc)}
                fdict = {"f": levf.fout, "g": levf.gout, "lm": levf.lm, "w": levf.w_vel, "alpha": levf.alpha,
                         "macro": _macro(levf)}
                il.explode39(kf, 2 * cyc + kk + 1, cdict, COARSE[0], fdict, _fine_box()[0], ghost)
                levf.rho[...], levf.u[...], levf.v[...], levf.temp[...] = (fdict["macro"][m] for m in (0, 1, 2, 4))
        ctx.average_down(1)
        cdict = {"f": levc.fout, "g": levc.gout, "lm": levc.lm, "w": levc.w_vel, "alpha": levc.alpha,
                 "macro": _macro(levc)}
        fdict = {"f": levf.fout, "g": levf.gout, "lm": levf.lm, "w": levf.w_vel, "alpha": levf.alpha,
                 "macro": _macro(levf)}
        il.average_down39(fdict, _fine_box()[0], ~ghost, cdict, COARSE[0], np.ones(S["stc"].shape[1:], bool))
        levc.rho[...], levc.u[...], levc.v[...], levc.temp[...] = (cdict["macro"][m] for m in (0, 1, 2, 4))
    for lvl, lev in ((0, levc), (1, levf)):
        out = ctx.download39(lvl)
        assert np.isfinite(out["fout"]).all()
        for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
            rel = np.max(np.abs(out[name] - ref) / np.abs(ref))
            assert rel <= 1e-11, (lvl, name, rel)
    ctx.close()
