"""Coarse-fine transfer between two D3Q27 levels on the GPU (explosion into
the fine level's ghost nodes, coalescence onto the coarse level) against the
numpy restatement, and a short two-level run with the reference's sub-cycle
order (loop.f95:94-147): the fine level steps twice per coarse step, ghosts
are refilled on the fine level's odd steps and the coarse level is averaged
down on its even ones."""
import numpy as np
import pytest

from oracle import interlevel as il

pytestmark = pytest.mark.gpu

GHOST = 10000000
COARSE = ((0, 0, 0), (23, 15, 15))          # coarse index space
FINE_VALID = ((16, 8, 8), (31, 23, 23))     # fine index space (coarse 8..15.5, 4..11.5, 4..11.5)
SHELL = 2


def _coarse_state(pkg):
    geo = pkg.geometry
    (x0, y0, z0), (x1, y1, z1) = COARSE
    faces = {k: -10 for k in ("x-", "x+", "y-", "y+", "z-", "z+")}  # closed box, bounce-back walls
    return geo.box_state27(x1 - x0 + 1, y1 - y0 + 1, z1 - z0 + 1, faces)


def _fine_box():
    (x0, y0, z0), (x1, y1, z1) = FINE_VALID
    return (x0 - SHELL, y0 - SHELL, z0 - SHELL), (x1 + SHELL, y1 + SHELL, z1 + SHELL)


def _fine_state():
    lo, hi = _fine_box()
    n = [hi[a] - lo[a] + 1 for a in range(3)]
    st = np.zeros((27, n[2], n[1], n[0]), np.int32)
    ghost = np.ones((n[2], n[1], n[0]), bool)
    ghost[SHELL:-SHELL, SHELL:-SHELL, SHELL:-SHELL] = False
    st[0][ghost] = GHOST
    return st, ghost


def _setup(pkg, storage):
    cap, geo = pkg.capi, pkg.geometry
    ctx = cap.Context(0)
    (cx0, cy0, cz0), (cx1, cy1, cz1) = COARSE
    flo, fhi = _fine_box()
    ctx.level_register(0, cap.ELBM_D3Q27, storage, [[cx0, cy0, cz0, cx1, cy1, cz1]])
    ctx.level_register(1, cap.ELBM_D3Q27, storage, [list(flo) + list(fhi)])
    bp = geo.d3q27_boundary_params((0.0, 0.0, 0.0), 1e-2)
    for lvl in (0, 1):
        ctx.set_d3q27_params(0 if lvl == 0 else 1, cap.make_d3q27_params(**bp))
    cst = _coarse_state(pkg)
    fst, ghost = _fine_state()
    ctx.set_links(0, 0, cst)
    ctx.set_links(1, 0, fst)
    nc = cst.shape[1:][::-1]
    nf = fst.shape[1:][::-1]
    fc = geo.perturbed_equilibrium(*nc, (0.03, 0.01, 0.0), 2e-2, seed=11)
    ff = geo.perturbed_equilibrium(*nf, (0.03, 0.01, 0.0), 2e-2, seed=12)
    ctx.upload(0, 0, fc)
    ctx.upload(1, 0, ff)
    ctx.interlevel_setup(1)
    return ctx, cst, fst, ghost, fc, ff


@pytest.mark.parametrize("storage", [0, 1])
def test_explosion_and_coalescence_match_oracle(pkg, built_lib, storage):
    ctx, cst, fst, ghost, fc, ff = _setup(pkg, storage)
    fc_dev, ff_dev = ctx.download(0), ctx.download(1)  # after the FP32 round trip, if any
    rep = ctx.fill_fine_ghosts(1)
    got = ctx.download(1)
    ref = ff_dev.copy()
    rep_ref = il.explode(fc_dev, COARSE[0], ref, _fine_box()[0], ghost)
    assert rep == rep_ref
    tol = 0.0 if storage == 0 else 2e-7
    assert np.max(np.abs(got - ref)) <= tol
    assert np.array_equal(got[:, ~ghost], ff_dev[:, ~ghost])  # valid fine nodes untouched
    ctx.average_down(1)
    gotc = ctx.download(0)
    refc = fc_dev.copy()
    il.average_down(got, _fine_box()[0], ~ghost, refc, COARSE[0], np.ones(cst.shape[1:], bool))
    assert np.max(np.abs(gotc - refc)) <= tol
    assert not np.array_equal(gotc, fc_dev)  # some coarse nodes were overwritten
    ctx.close()


def test_two_level_subcycle_runs_stably(pkg, built_lib):
    ctx, cst, fst, ghost, fc, ff = _setup(pkg, 0)
    m0 = ctx.download(0).sum()
    for _ in range(10):
        ctx.step(0, 1)                 # coarse step
        for k in range(2):             # two fine steps
            ctx.step(1, 1)
            if k == 0:
                ctx.fill_fine_ghosts(1)  # the fine level's odd step
        ctx.average_down(1)            # the fine level's even step
    fcn, ffn = ctx.download(0), ctx.download(1)
    assert np.isfinite(fcn).all() and np.isfinite(ffn).all()
    # closed box: the coarse mass changes only through the coalescence of fine data
    assert abs(fcn.sum() - m0) <= 1e-3 * m0
    ctx.close()


@pytest.mark.parametrize("storage", [0, 1])
def test_amr_run_graph_matches_host_sequence(pkg, built_lib, storage):
    """elbm_amr_run (two coarse cycles captured in a CUDA graph, replayed) gives
    the same populations as the same sequence issued call by call."""
    ctx, *_ = _setup(pkg, storage)
    ref, *_ = _setup(pkg, storage)
    s = ctx.amr_run(2, 5)  # two graph replays and one plain cycle
    for _ in range(5):
        ref.step(0, 1)
        for k in range(2):
            ref.step(1, 1)
            if k == 0:
                ref.fill_fine_ghosts(1)
        ref.average_down(1)
    for lvl in (0, 1):
        assert np.array_equal(ctx.download(lvl), ref.download(lvl))
    nc = np.prod(_coarse_state(pkg).shape[1:])
    nf = np.prod(_fine_state()[0].shape[1:])
    assert s["node_updates"] == 5 * (nc + 2 * nf)
    s2 = ctx.amr_run(2, 4)  # the captured graph is reused
    assert s2["node_updates"] == 4 * (nc + 2 * nf) and s2["status"] == 0
    ctx.close()
    ref.close()
