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


@pytest.mark.parametrize("shifted,outlet_type", [(0, 6), (1, 6), (1, 2)])
def test_d3q39_link_codes_parity(pkg, o39, built_lib, shifted, outlet_type):
    """A D3Q39 box with an inlet, an outlet, a bounce-back wall, a freestream
    face, solid nodes and a periodic axis: the GPU step with the library's
    pull tables against the oracle's push loop, 1e-12 relative."""
    import math
    setup39, cap = pkg.d3q39_setup, pkg.capi
    if shifted:
        c = setup39.wedge_case_consts()
    else:
        c = setup39.wedge_case_consts(v_inf_ms=0.3 * math.sqrt(1.4 * 287.052874 * 288.15))
    c.shifted = shifted
    k = o39.consts(c)
    lm0 = setup39.freestream_start_lm(c)
    _, ff, gf, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    _, fi, gi, _ = o39.init_node(k, 1.02, c.mach, 0.0, 0.0, c.temperature, lm0)
    _, fo, go, _ = o39.init_node(k, 0.98, c.mach, 0.0, 0.0, c.temperature, lm0)
    nx, ny, nz, periodic = 16, 6, 7, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = setup39.box_state39(nx, ny, nz, faces, shifted, 1, periodic=periodic)
    st[0, 3, 2:4, 6:8] = -1
    cx, cy, cz, _ = setup39.lattice39(shifted, 1)
    for i in range(1, 39):
        for zz in range(nz):
            for yy in range(ny):
                for xx in range(nx):
                    tx, ty, tz = xx + cx[i], (yy + cy[i]) % ny, zz + cz[i]
                    if st[0, zz, yy, xx] >= 0 and 0 <= tx < nx and 0 <= tz < nz and st[0, tz, ty, tx] < 0:
                        st[i, zz, yy, xx] = -10
    inl_t, out_t = [1] * 8, [outlet_type] + [1] * 7
    lev = _init(o39, setup39, c, k, nx, ny, nz, noise=0.01, seed=12)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0))
    ctx.set_links39(0, 0, st, cap.make_d3q39_bc(inl_t, out_t, ff, gf, [fi] * 8, [gi] * 8, [fo] * 8, [go] * 8))
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    steps = 5
    s = ctx.step(0, steps)
    out = ctx.download39(0)
    b = o39.bc(inl_t, out_t, ff, gf, [fi] * 8, [gi] * 8, [fo] * 8, [go] * 8)
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    for step in range(steps):
        so = o39.step_links(k, lev, step, st, periodic, b, prev_f, prev_g)
    fluid = st[0] >= 0
    assert s["node_updates"] == steps * fluid.sum() and s["fallbacks"] == 0 and so["lm_capped"] == 0
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        rel = np.max(np.abs(out[name][:, fluid] - ref[:, fluid]) / np.abs(ref[:, fluid]))
        assert rel <= 1e-12, (name, rel)
    ctx.close()
