"""Level checkpoints: N steps, write, M more steps; a fresh context registered,
parameterised and linked the same way reads the checkpoint and runs the same M
steps: the states agree bit for bit (D3Q27 FP32 and FP64, D3Q39 with link codes
and interpolated walls)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _d3q27(pkg, storage):
    geo, cap = pkg.geometry, pkg.capi
    nx, ny, nz = 32, 16, 12
    st = geo.box_state27(nx, ny, nz, geo.flat_plate_faces())
    f0 = geo.perturbed_equilibrium(nx, ny, nz, (0.05, 0.0, 0.0), 2e-3, seed=77)
    bp = geo.d3q27_boundary_params((0.05, 0.0, 0.0), 1e-3)

    def make():
        ctx = cap.Context(0)
        ctx.level_register(0, cap.ELBM_D3Q27, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
        ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
        ctx.set_links(0, 0, st)
        return ctx

    return make, f0


@pytest.mark.parametrize("storage", ["fp32", "fp64"])
def test_d3q27_checkpoint_restart_bitwise(pkg, built_lib, tmp_path, storage):
    cap = pkg.capi
    make, f0 = _d3q27(pkg, cap.ELBM_STORE_FP32_DEV if storage == "fp32" else cap.ELBM_STORE_FP64)
    a = make()
    a.upload(0, 0, f0)
    a.step(0, 7, want_stats=False)
    path = tmp_path / "level0.ckp"
    a.checkpoint_write(0, path)
    a.step(0, 5, want_stats=False)
    ref = a.download(0)
    a.close()
    b = make()
    b.checkpoint_read(0, path)
    b.step(0, 5, want_stats=False)
    got = b.download(0)
    b.close()
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_d3q39_checkpoint_restart_bitwise(pkg, built_lib, tmp_path, storage):
    """FP32 storage carries the per-direction reference of its deviations in the
    checkpoint."""
    s39, cap = pkg.d3q39_setup, pkg.capi
    store = cap.ELBM_STORE_FP32_DEV if storage == "fp32" else cap.ELBM_STORE_FP64
    c = s39.wedge_case_consts(v_inf_ms=0.8 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=True)
    nx, ny, nz, periodic = 24, 6, 12, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = s39.wedge_state39(nx, ny, nz, 6.0, 14.0, 20.0, faces, periodic=periodic)
    lm0 = s39.freestream_start_lm(c)
    params = cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=1)
    shape = (nz, ny, nx)
    rng = np.random.default_rng(3)
    macro = np.stack([1 + 0.01 * rng.uniform(-1, 1, shape), np.full(shape, c.mach), np.zeros(shape),
                      np.zeros(shape), np.full(shape, c.temperature)])

    def make():
        ctx = cap.Context(0)
        _, f, g = ctx.d3q39_equilibrium(params, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
        ctx.level_register(0, cap.ELBM_D3Q39, store, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
        ctx.set_d3q39_params(0, params)
        ctx.set_links39(0, 0, st, cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8,
                                                     [g] * 8, (c.mach, 0.0, 0.0, c.temperature)))
        return ctx

    a = make()
    a.init_level39(0, 0, macro, lm0)
    a.step(0, 6, want_stats=False)
    path = tmp_path / "level39.ckp"
    a.checkpoint_write(0, path)
    a.step(0, 4, want_stats=False)
    ref = a.download39(0)
    a.close()
    b = make()
    b.checkpoint_read(0, path)
    b.step(0, 4, want_stats=False)
    got = b.download39(0)
    b.close()
    assert np.isfinite(ref["fout"]).all()
    for name in ("fout", "gout", "lm", "w_vel", "macro"):
        assert np.array_equal(got[name], ref[name]), name


@pytest.mark.parametrize("storage", ["fp32", "fp64"])
def test_d3q27_checkpoint_solid_nodes_odd_steps(pkg, built_lib, tmp_path, storage):
    """A level with solid nodes (an icosphere), restarted and advanced an odd
    number of steps: the step never writes solid nodes, so after the restart
    both population buffers must hold the checkpoint's values there, and the
    download (which reads the buffer the last step wrote) matches the
    uninterrupted run everywhere, solid nodes included."""
    geo, cap = pkg.geometry, pkg.capi
    nx, ny, nz = 32, 20, 20
    st = geo.box_state27(nx, ny, nz, geo.sphere_faces())
    cap.mark_triangles(st, (0.0, 0.0, 0.0), 1.0, geo.icosphere(2, 5.0, (12.0, 10.0, 10.0)))
    assert (st[0] == -1001).sum() > 0  # there are solid nodes
    f0 = geo.perturbed_equilibrium(nx, ny, nz, (0.06, 0.0, 0.0), 1e-3, seed=91)
    bp = geo.d3q27_boundary_params((0.06, 0.0, 0.0), 1e-3)
    stor = cap.ELBM_STORE_FP32_DEV if storage == "fp32" else cap.ELBM_STORE_FP64

    def make():
        ctx = cap.Context(0)
        ctx.level_register(0, cap.ELBM_D3Q27, stor, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
        ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
        ctx.set_links(0, 0, st)
        return ctx

    a = make()
    a.upload(0, 0, f0)
    a.step(0, 4, want_stats=False)
    path = tmp_path / "solid.ckp"
    a.checkpoint_write(0, path)
    a.step(0, 3, want_stats=False)
    ref = a.download(0)
    a.close()
    b = make()
    b.checkpoint_read(0, path)
    b.step(0, 3, want_stats=False)
    got = b.download(0)
    b.close()
    assert np.isfinite(got).all()
    assert np.array_equal(got, ref)
