"""GPU parity of the D3Q39 compressible step (two populations, 13 multipliers,
closed-form alpha, heat-flux corrections) against the CPU restatement of the
reference routines.  Tolerance: 1e-12 relative in f, g and the multipliers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def o39():
    from oracle import oracle39

    oracle39.lib()
    return oracle39


def _init(o39, setup39, c, k, nx, ny, nz, noise, seed):
    lev = o39.Level39(nx, ny, nz)
    rng = np.random.default_rng(seed)
    lm0 = setup39.freestream_start_lm(c)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                rho = 1.0 + noise * rng.uniform(-1, 1)
                u = c.mach * (1 + noise * rng.uniform(-1, 1))
                v, w = noise * rng.uniform(-1, 1, 2)
                T = c.temperature * (1 + noise * rng.uniform(-1, 1))
                lm, f, g, _ = o39.init_node(k, rho, u, v, w, T, lm0)
                lev.fout[:, z, y, x] = f
                lev.gout[:, z, y, x] = g
                lev.lm[:, z, y, x] = lm
                lev.w_vel[z, y, x] = w
    return lev


@pytest.mark.parametrize("start_step,steps", [(0, 6), (140, 6)])
def test_d3q39_periodic_parity(pkg, o39, built_lib, start_step, steps):
    setup39, cap = pkg.d3q39_setup, pkg.capi
    c = setup39.wedge_case_consts()
    k = o39.consts(c)
    nx, ny, nz = 10, 6, 5
    lev = _init(o39, setup39, c, k, nx, ny, nz, noise=0.01, seed=11)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=start_step))
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    st = ctx.step(0, steps)
    out = ctx.download39(0)
    for s in range(steps):
        so = o39.step_periodic(k, lev, start_step + s)
    assert so["lm_capped"] == 0 and st["fallbacks"] == 0
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        rel = np.max(np.abs(out[name] - ref) / np.abs(ref))
        assert rel <= 1e-12, (name, rel)
    assert np.max(np.abs(out["lm"] - lev.lm)) <= 1e-12 * np.max(np.abs(lev.lm))
    assert np.max(np.abs(out["alpha"] - lev.alpha)) <= 1e-11  # closed-form alpha: sqrt and divisions
    assert st["node_updates"] == steps * nx * ny * nz
    ctx.close()
