"""Learned alpha end to end on the GPU: harvest (populations, alpha) records
from Newton solves, train the network with the library's kernels, and run the
step with the learned guess + at most two Newton steps (Newton from 2 as the
fallback).  The result must satisfy the same entropy condition and agree with
the Newton path; the test reports what the guess saves."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _level(pkg, alpha_mode, check=0, n=(64, 32, 32)):
    geo, cap = pkg.geometry, pkg.capi
    nx, ny, nz = n
    st = geo.box_state27(nx, ny, nz, geo.flat_plate_faces())
    f0 = geo.perturbed_equilibrium(nx, ny, nz, (0.06, 0, 0), 5e-3, seed=77)
    bp = geo.d3q27_boundary_params((0.06, 0, 0), 2e-5)
    bp.update(alpha_mode=alpha_mode, check_dH=check)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    return ctx, st, f0, bp


def test_learned_alpha_pipeline(pkg, built_lib):
    cap = pkg.capi
    # harvest from Newton solves
    ctx, st, f0, bp = _level(pkg, cap.ELBM_ALPHA_NEWTON)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f0)
    rec = ctx.alpha_harvest(0, nsteps=30, stride=3, capacity=1 << 20)
    assert rec.shape[0] > 100000 and np.isfinite(rec).all()
    w, hist = ctx.alpha_mlp_train(rec, mlp_ref.init(0).astype(np.float32), epochs=8, batch=4096, lr=2e-3, seed=3)
    assert hist[-1] < 0.5 * hist[0], hist
    f_mid = ctx.download(0)
    # Newton and learned steps from the same state
    res = {}
    for mode in (cap.ELBM_ALPHA_NEWTON, cap.ELBM_ALPHA_LEARNED):
        c2, st2, _, bp2 = _level(pkg, mode, check=1)
        if mode == cap.ELBM_ALPHA_LEARNED:
            c2.set_alpha_mlp(0, w)
        c2.set_d3q27_params(0, cap.make_d3q27_params(**bp2))
        c2.set_links(0, 0, st2)
        c2.upload(0, 0, f_mid)
        s = c2.step(0, 10)
        res[mode] = (s, c2.download(0))
        c2.close()
    sn, fn = res[cap.ELBM_ALPHA_NEWTON]
    sl, fl = res[cap.ELBM_ALPHA_LEARNED]
    assert sl["dh_over_tol"] == 0 and sl["max_abs_dH"] <= 1e-10, sl
    assert sl["fallbacks"] <= 1e-5 * sl["node_updates"]
    # both paths solve the same equation: the populations agree to FP32 level
    assert np.max(np.abs(fl - fn)) <= 1e-6
    it_newton = sn["newton_iters"] / sn["node_updates"]
    it_learned = sl["newton_iters"] / sl["node_updates"]
    print(f"Newton iterations per node: {it_newton:.3f} from alpha = 2, {it_learned:.3f} from the learned guess; "
          f"guesses needing the fallback: {sl['guess_misses'] / sl['node_updates']:.2e}")
    assert sl["guess_misses"] <= 0.01 * sl["node_updates"]
    assert it_learned < it_newton
    # outside check mode the learned step runs the tensor-core inference kernel
    c3, st3, _, bp3 = _level(pkg, cap.ELBM_ALPHA_LEARNED, check=0)
    c3.set_alpha_mlp(0, w)
    c3.set_d3q27_params(0, cap.make_d3q27_params(**bp3))
    c3.set_links(0, 0, st3)
    c3.upload(0, 0, f_mid)
    s3 = c3.step(0, 10)
    f3 = c3.download(0)
    c3.close()
    assert s3["status"] & 0x10 == 0 and s3["fallbacks"] <= 1e-5 * s3["node_updates"]
    assert np.max(np.abs(f3 - fn)) <= 1e-6
    it_tc = s3["newton_iters"] / s3["node_updates"]
    print(f"tensor-core guess: {it_tc:.3f} iterations per node, guesses needing the fallback: "
          f"{s3['guess_misses'] / s3['node_updates']:.2e}")
    assert s3["guess_misses"] <= 0.02 * s3["node_updates"]
    ctx.close()


def test_learned_alpha_budget(pkg, built_lib):
    """What the learned guess could save against what the network costs, measured
    on one state of the boundary layer (256x128x64): the step with alpha = 2 (no
    alpha solve), with Newton from alpha = 2 and with the learned guess on the
    tensor cores.  The whole alpha solve costs t_newton - t_fixed per node; a
    guess still needs the power sums and at least one certified Newton step, so
    it can save at most that.  The network (27-64-64-1, 11.8 kFLOP per node on the
    tensor cores, and per node 128 bias + GELU evaluations and a 64-term dot
    product on the FP32 pipe) costs more than the whole alpha solve: the learned
    step is slower than Newton by more than the alpha solve costs, and the guess
    saves almost no iterations (Newton converges in two from alpha = 2)."""
    cap = pkg.capi
    ctx, st, f0, bp = _level(pkg, cap.ELBM_ALPHA_NEWTON)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f0)
    rec = ctx.alpha_harvest(0, nsteps=30, stride=3, capacity=1 << 20)
    w, _ = ctx.alpha_mlp_train(rec, mlp_ref.init(0).astype(np.float32), epochs=8, batch=4096, lr=2e-3, seed=3)
    ctx.close()
    n = (256, 128, 64)
    c0, st0, f1, bp0 = _level(pkg, cap.ELBM_ALPHA_NEWTON, n=n)
    c0.set_d3q27_params(0, cap.make_d3q27_params(**bp0))
    c0.set_links(0, 0, st0)
    c0.upload(0, 0, f1)
    c0.step(0, 20, want_stats=False)  # develop the non-equilibrium parts
    f_mid = c0.download(0)
    c0.close()
    res = {}
    for mode in (cap.ELBM_ALPHA_FIXED2, cap.ELBM_ALPHA_NEWTON, cap.ELBM_ALPHA_LEARNED):
        c2, st2, _, bp2 = _level(pkg, mode, n=n)
        if mode == cap.ELBM_ALPHA_LEARNED:
            c2.set_alpha_mlp(0, w)
        c2.set_d3q27_params(0, cap.make_d3q27_params(**bp2))
        c2.set_links(0, 0, st2)
        best = None
        for _ in range(3):
            c2.upload(0, 0, f_mid)
            s = c2.step(0, 4)
            if best is None or s["kernel_ms"] < best["kernel_ms"]:
                best = s
        res[mode] = best
        c2.close()
    ns = {m: 1e6 * s["kernel_ms"] / s["node_updates"] for m, s in res.items()}
    it = {m: s["newton_iters"] / s["node_updates"] for m, s in res.items()}
    t_alpha = ns[cap.ELBM_ALPHA_NEWTON] - ns[cap.ELBM_ALPHA_FIXED2]
    t_net = ns[cap.ELBM_ALPHA_LEARNED] - ns[cap.ELBM_ALPHA_NEWTON]
    print(f"BUDGET ns/node: alpha=2 {ns[cap.ELBM_ALPHA_FIXED2]:.4f}, Newton {ns[cap.ELBM_ALPHA_NEWTON]:.4f} "
          f"({it[cap.ELBM_ALPHA_NEWTON]:.3f} iterations), learned {ns[cap.ELBM_ALPHA_LEARNED]:.4f} "
          f"({it[cap.ELBM_ALPHA_LEARNED]:.3f} iterations); whole alpha solve {t_alpha:.4f}, network net {t_net:.4f}")
    assert res[cap.ELBM_ALPHA_LEARNED]["fallbacks"] <= 1e-5 * res[cap.ELBM_ALPHA_LEARNED]["node_updates"]
    # the guess saves less than a tenth of an iteration per node
    assert it[cap.ELBM_ALPHA_NEWTON] - it[cap.ELBM_ALPHA_LEARNED] < 0.1
    # the network costs more than the whole alpha solve it could at best replace
    assert t_net > t_alpha
