"""Negative-population repair of a D3Q27 level (damp_it.f95:64-177) on the GPU
against the numpy restatement, and the step's built-in repair (damp = 1)
against a step followed by the stand-alone repair."""
import numpy as np
import pytest

from oracle import damp27

pytestmark = pytest.mark.gpu


def _field(pkg, nx, ny, nz, seed):
    geo = pkg.geometry
    st = geo.box_state27(nx, ny, nz, geo.flat_plate_faces())
    f = geo.perturbed_equilibrium(nx, ny, nz, (0.06, 0.0, 0.0), 1e-2, seed=seed)
    rng = np.random.default_rng(seed)
    k = rng.choice(f.size, 300, replace=False)
    f.reshape(-1)[k] = -rng.uniform(1e-4, 1e-2, k.size)
    return st, f


def _ctx(pkg, st, f, storage, damp=0):
    cap, geo = pkg.capi, pkg.geometry
    _, nz, ny, nx = f.shape
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**dict(geo.d3q27_boundary_params((0.06, 0.0, 0.0), 1e-3), damp=damp)))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f)
    return ctx


@pytest.mark.parametrize("storage", [0, 1])
def test_damp_level_matches_oracle(pkg, built_lib, storage):
    st, f = _field(pkg, 32, 24, 20, seed=21)
    ctx = _ctx(pkg, st, f, storage)
    f_dev = ctx.download(0)  # the field as stored (FP32 deviations round it)
    n = ctx.damp_level(0)
    got = ctx.download(0)
    ref, nref = damp27.damp(st, f_dev)
    assert n == nref == 300
    tol = 0.0 if storage == 0 else 1e-7
    assert np.max(np.abs(got - ref)) <= tol
    assert (got >= 0.0).all()
    ctx.close()


@pytest.mark.parametrize("storage", [0, 1])
def test_step_with_repair_equals_step_then_repair(pkg, built_lib, storage):
    st, f = _field(pkg, 32, 24, 20, seed=22)
    a = _ctx(pkg, st, f, storage, damp=1)
    b = _ctx(pkg, st, f, storage, damp=0)
    for _ in range(3):
        a.step(0, 1)
        b.step(0, 1)
        b.damp_level(0)
    fa, fb = a.download(0), b.download(0)
    fluid = st[0] >= 0
    assert np.array_equal(fa[:, fluid], fb[:, fluid])
    a.close()
    b.close()
