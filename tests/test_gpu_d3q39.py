"""GPU parity of the D3Q39 compressible step (two populations, 13 multipliers,
closed-form alpha, heat-flux corrections) against the CPU restatement of the
reference routines.  Tolerance: 1e-12 relative in f, g and the multipliers."""
import math

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


def test_d3q39_fp32_storage_periodic(pkg, o39, built_lib):
    """FP32 deviation storage of f and g (the multipliers, alpha and every operation
    stay FP64) against the oracle's FP64 step on the periodic box: each stored
    population is rounded once per step to a float deviation from the box's
    per-direction mean, so f and g stay within 1e-6 relative over 6 steps; the
    rounding error of the initial state alone is under 1e-7."""
    setup39, cap = pkg.d3q39_setup, pkg.capi
    c = setup39.wedge_case_consts()
    k = o39.consts(c)
    nx, ny, nz, steps = 10, 6, 5, 6
    lev = _init(o39, setup39, c, k, nx, ny, nz, noise=0.01, seed=11)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP32_DEV, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0))
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    start = ctx.download39(0)
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        assert np.max(np.abs(start[name] - ref) / np.abs(ref)) <= 1e-7, name
    st = ctx.step(0, steps)
    out = ctx.download39(0)
    ctx.close()
    for s in range(steps):
        o39.step_periodic(k, lev, s)
    assert st["fallbacks"] == 0 and st["node_updates"] == steps * nx * ny * nz
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        rel = np.max(np.abs(out[name] - ref) / np.abs(ref))
        print(f"FP32 storage {name}: {rel:.3e}")
        assert rel <= 1e-6, (name, rel)


@pytest.mark.parametrize("shifted,outlet_type,side", [(0, 6, 0), (1, 6, 0), (1, 2, 0), (0, 1, -11), (1, 6, -11)])
def test_d3q39_link_codes_parity(pkg, o39, built_lib, shifted, outlet_type, side):
    """A D3Q39 box with an inlet, an outlet, a bounce-back wall, a freestream
    face, solid nodes and either a periodic axis (side 0) or inviscid side
    walls (side -11, specular reflection of inviscid_edge.f95): the GPU step
    with the library's pull tables against the oracle's push loop, 1e-12
    relative."""
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
    nx, ny, nz, periodic = 16, 6, 7, (2 if side == 0 else 0)
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": side, "y+": side}
    prio = ("x-", "x+", "z-", "z+", "y-", "y+") if side == 0 else ("y-", "y+", "x-", "x+", "z-", "z+")
    st = setup39.box_state39(nx, ny, nz, faces, shifted, 1, periodic=periodic, priority=prio)
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


def _wall_case(pkg, o39, seed, outlet_type, nx=16, ny=6, nz=8, mach=1.5, wedge=False, shifted=True, sidewalls=False):
    """Shifted D3Q39 box (Mach 1.5 along +x): inlet at x-, outlet at x+, a
    bounce-back floor, a freestream top, periodic in y, and a solid block on
    the floor whose fluid neighbours carry interpolated wall links with random
    wall distances; one wall node also has a null link (target_finder's
    erp(i) = -666 branch).  Random rho, u, v, w, T per node."""
    s39 = pkg.d3q39_setup
    c = s39.wedge_case_consts(v_inf_ms=mach * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=shifted)
    sh = int(c.shifted)
    k = o39.consts(c)
    lm0 = s39.freestream_start_lm(c)
    eq = [o39.init_node(k, r, c.mach, 0.0, 0.0, c.temperature, lm0)[1:3] for r in (1.0, 1.02, 0.98)]
    (ff, gf), (fi, gi), (fo, go) = eq
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    periodic = 2
    rng = np.random.default_rng(seed)
    if wedge and sidewalls:
        # the wedge case's faces (inviscid side walls): behind the back face the side-wall nodes have
        # inviscid links whose axis links are wall links, which no branch of inviscid_edge.f95 covers
        faces, periodic = s39.WEDGE_FACES, 0
        st = s39.wedge_state39(nx, ny, nz, 5.0, 12.0, 20.0, faces, periodic=periodic, priority=s39.WEDGE_PRIORITY)
    elif wedge:
        # a 20-degree wedge across the span from x = 5 to x = 12, wall distances from the geometry
        st = s39.wedge_state39(nx, ny, nz, 5.0, 12.0, 20.0, faces, periodic=periodic)
    else:
        st = s39.box_state39(nx, ny, nz, faces, sh, 1, periodic=periodic)
        solid = np.zeros((nz, ny, nx), bool)
        solid[0:3, 1:4, 6:9] = True
        s39.wall_links39(st, solid, rng.uniform(0.05, 0.95, (39, nz, ny, nx)), sh, 1, periodic=periodic)
    cx, cy, cz, _ = s39.lattice39(sh, 1)
    erp = np.array(s39.OPP39) - 1
    for z, y, x, j in zip(*np.nonzero((st[0] >= 0)[None] & (st[1:15] <= -1001))[1:], np.nonzero(
            (st[0] >= 0)[None] & (st[1:15] <= -1001))[0] + 1):
        if 0 <= x + cx[j] < nx and 0 <= z + cz[j] < nz:  # target_finder reads node x + c_j
            st[erp[j], z, y, x] = -666
            break
    lev = o39.Level39(nx, ny, nz)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                rho = 1.0 + 0.01 * rng.uniform(-1, 1)
                u = c.mach * (1 + 0.01 * rng.uniform(-1, 1))
                v, w = 0.01 * rng.uniform(-1, 1, 2)
                T = c.temperature * (1 + 0.01 * rng.uniform(-1, 1))
                lm, f, g, _ = o39.init_node(k, rho, u, v, w, T, lm0)
                lev.fout[:, z, y, x], lev.gout[:, z, y, x], lev.lm[:, z, y, x] = f, g, lm
                lev.rho[z, y, x], lev.u[z, y, x], lev.v[z, y, x], lev.w_vel[z, y, x] = rho, u, v, w
                lev.temp[z, y, x] = T
    inl_t, out_t = [1] * 8, [outlet_type] + [1] * 7
    fs = (c.mach, 0.0, 0.0, c.temperature)
    args = (inl_t, out_t, ff, gf, [fi] * 8, [gi] * 8, [fo] * 8, [go] * 8, fs)
    return c, k, st, lev, periodic, o39.bc(*args), pkg.capi.make_d3q39_bc(*args)


@pytest.mark.parametrize("seed,outlet_type,mach,warm,steps,wedge,sidewalls",
                         [(3, 6, 1.5, 0, 5, False, False), (4, 1, 0.8, 0, 8, False, False),
                          (5, 6, 0.8, 97, 6, False, False), (6, 6, 1.5, 0, 5, True, False),
                          (9, 6, 1.5, 0, 6, True, True)])
def test_d3q39_wall_links_parity(pkg, o39, built_lib, seed, outlet_type, mach, warm, steps, wedge, sidewalls):
    """Interpolated wall links on the shifted lattice (target_finder, the target
    Newton solve, shifted_ibb) next to the other boundary codes: the GPU step
    against the oracle's push loop, 1e-12 relative.  Steps 0..4 (start-up
    multipliers), 0..7 (warm starts from the node's multipliers), and 97..102
    across the end of the start-up ramps: the oracle runs the first 97 steps
    alone and both continue from its state (slots no rule writes then hold
    the uploaded fout on both sides).  By then the flow past the block is
    strongly non-uniform and the step itself amplifies rounding (the target
    Newton stops at |delta| <= 1e-7, the closed-form alpha cancels where it is
    small): the oracle fed its own state with 1-ulp noise moves by ~1e-12 per
    step at the wall nodes.  That late run is held to 20 times the oracle's own
    spread under such noise (and never looser than 1e-9).  The last case has the
    wedge case's inviscid side walls, including links no branch of the
    reference's inviscid table covers (nothing written for them)."""
    cap = pkg.capi
    c, k, st, lev, periodic, b, cb = _wall_case(pkg, o39, seed, outlet_type, mach=mach, wedge=wedge,
                                                nx=20 if wedge else 16, nz=10 if wedge else 8, sidewalls=sidewalls)
    nz, ny, nx = lev.shape
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    for step in range(warm):
        o39.step_links(k, lev, step, st, periodic, b, prev_f, prev_g)
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    fluid = st[0] >= 0
    tol = 1e-12
    if warm:
        # the oracle's own sensitivity: the same steps from the state with 1-ulp noise
        noisy = o39.Level39(nx, ny, nz)
        rng = np.random.default_rng(seed)
        for name in ("fout", "gout", "lm", "w_vel", "rho", "u", "v", "temp"):
            a = getattr(lev, name)
            getattr(noisy, name)[...] = a * (1 + 2.2e-16 * rng.uniform(-1, 1, a.shape))
        nf, ng = noisy.fout.copy(), noisy.gout.copy()
        clean = o39.Level39(nx, ny, nz)
        for name in ("fout", "gout", "lm", "w_vel", "rho", "u", "v", "temp"):
            getattr(clean, name)[...] = getattr(lev, name)
        cf, cg = clean.fout.copy(), clean.gout.copy()
        for step in range(warm, warm + steps):
            o39.step_links(k, noisy, step, st, periodic, b, nf, ng)
            o39.step_links(k, clean, step, st, periodic, b, cf, cg)
        spread = np.max(np.abs(noisy.fout[:, fluid] - clean.fout[:, fluid]) / np.abs(clean.fout[:, fluid]))
        tol = min(max(1e-12, 20 * spread), 1e-9)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=warm, periodic=periodic, damp=0))
    ctx.set_links39(0, 0, st, cb)
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    ctx.upload_macro39(0, 0, np.stack([lev.rho, lev.u, lev.v, lev.w_vel, lev.temp]))
    s = ctx.step(0, steps)
    out = ctx.download39(0)
    for step in range(warm, warm + steps):
        so = o39.step_links(k, lev, step, st, periodic, b, prev_f, prev_g)
    assert np.isfinite(lev.fout[:, fluid]).all()
    assert s["node_updates"] == steps * fluid.sum() and s["fallbacks"] == 0 and so["lm_capped"] == 0
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        rel = np.max(np.abs(out[name][:, fluid] - ref[:, fluid]) / np.abs(ref[:, fluid]))
        assert rel <= tol, (name, rel, tol)
    macro = out["macro"]
    for m, ref in ((0, lev.rho), (4, lev.temp)):
        assert np.max(np.abs(macro[m][fluid] - ref[fluid]) / np.abs(ref[fluid])) <= tol


@pytest.mark.parametrize("seed,outlet_type", [(7, 6), (8, 1)])
def test_d3q39_unshifted_wall_links_parity(pkg, o39, built_lib, seed, outlet_type):
    """Interpolated wall links on the unshifted lattice (Mach 0.5): target_finder's
    unshifted branch, the node's own multipliers as the Newton start, and the
    hand-expanded closure of interpolative_bounceback_bc for direction opp(i)
    (from the coefficient tables) written to fout(x, i) and streamed into
    fi(x, opp(i)); GPU against the oracle's push loop, 1e-12 relative, steps 0..5."""
    cap = pkg.capi
    c, k, st, lev, periodic, b, cb = _wall_case(pkg, o39, seed, outlet_type, mach=0.5, shifted=False)
    assert not c.shifted and (st[1:] <= -1001).any()
    nz, ny, nx = lev.shape
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    fluid = st[0] >= 0
    steps = 6
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0))
    ctx.set_links39(0, 0, st, cb)
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    ctx.upload_macro39(0, 0, np.stack([lev.rho, lev.u, lev.v, lev.w_vel, lev.temp]))
    s = ctx.step(0, steps)
    out = ctx.download39(0)
    for step in range(steps):
        so = o39.step_links(k, lev, step, st, periodic, b, prev_f, prev_g)
    ctx.close()
    assert np.isfinite(lev.fout[:, fluid]).all()
    assert s["node_updates"] == steps * fluid.sum() and s["fallbacks"] == 0 and so["lm_capped"] == 0
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        rel = np.max(np.abs(out[name][:, fluid] - ref[:, fluid]) / np.abs(ref[:, fluid]))
        assert rel <= 1e-12, (name, rel)


def test_d3q39_wall_links_need_macro(pkg, o39, built_lib):
    cap = pkg.capi
    c, k, st, lev, periodic, b, cb = _wall_case(pkg, o39, 3, 6)
    nz, ny, nx = lev.shape
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0))
    ctx.set_links39(0, 0, st, cb)
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    with pytest.raises(cap.ElbmError):
        ctx.step(0, 1)


def test_d3q39_initial_state_on_device(pkg, o39, built_lib):
    """elbm_init_level39 (multiplier Newton per node from its macroscopic fields, then
    f = f_eq, g = (2 C_v - 3) T f_eq) and elbm_d3q39_equilibrium against the oracle's
    o39_init_node, 1e-12 relative, on the shifted and the unshifted lattice."""
    setup39, cap = pkg.d3q39_setup, pkg.capi
    for shifted in (1, 0):
        mach = 1.5 if shifted else 0.3
        c = setup39.wedge_case_consts(v_inf_ms=mach * math.sqrt(1.4 * setup39.GAS_CONST_R * 288.15))
        k = o39.consts(c)
        lm0 = setup39.freestream_start_lm(c)
        nx, ny, nz = 7, 5, 4
        rng = np.random.default_rng(21 + shifted)
        shape = (nz, ny, nx)
        macro = np.stack([1 + 0.02 * rng.uniform(-1, 1, shape), c.mach * (1 + 0.02 * rng.uniform(-1, 1, shape)),
                          0.01 * rng.uniform(-1, 1, shape), 0.01 * rng.uniform(-1, 1, shape),
                          c.temperature * (1 + 0.02 * rng.uniform(-1, 1, shape))])
        ctx = cap.Context(0)
        params = cap.make_d3q39_params(c, timestep=0, periodic=7, damp=0)
        ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
        ctx.set_d3q39_params(0, params)
        assert ctx.init_level39(0, 0, macro, lm0) == 0
        out = ctx.download39(0)
        for z in range(nz):
            for y in range(ny):
                for x in range(nx):
                    lm, f, g, _ = o39.init_node(k, *macro[:, z, y, x], lm0)
                    for name, ref in (("fout", f), ("gout", g), ("lm", lm)):
                        got = out[name][:, z, y, x]
                        # relative for the populations; multipliers near zero against max(|lm|, 1)
                        scale = np.abs(ref) if name != "lm" else np.maximum(np.abs(ref), 1.0)
                        assert np.max(np.abs(got - ref) / scale) <= 1e-12, name
        assert np.array_equal(out["w_vel"], macro[3])
        lm_e, f_e, g_e = ctx.d3q39_equilibrium(params, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
        lm_r, f_r, g_r, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
        assert np.max(np.abs(f_e - f_r) / f_r) <= 1e-12 and np.max(np.abs(g_e - g_r) / g_r) <= 1e-12
        ctx.close()


@pytest.mark.parametrize("shifted", [0, 1])
def test_d3q39_repair_with_link_codes(pkg, o39, built_lib, shifted):
    """The fout and gout parts of damp_it.f95 after the step on a box with link codes (inlet, outlet,
    bounce-back floor, freestream top, periodic span), past the start-up ramps: a few
    populations are inflated so that the over-relaxed collision drives isolated neighbours
    negative; GPU against the oracle's in-place sweep, 1e-12 relative."""
    setup39, cap = pkg.d3q39_setup, pkg.capi
    mach = 1.5 if shifted else 0.3
    c = setup39.wedge_case_consts(v_inf_ms=mach * math.sqrt(1.4 * setup39.GAS_CONST_R * 288.15))
    k = o39.consts(c)
    lm0 = setup39.freestream_start_lm(c)
    _, ff, gf, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    nx, ny, nz, periodic = 20, 6, 14, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = setup39.box_state39(nx, ny, nz, faces, shifted, 1, periodic=periodic)
    lev = _init(o39, setup39, c, k, nx, ny, nz, noise=0.005, seed=31 + shifted)
    rng = np.random.default_rng(7 + shifted)
    # inflate one population at isolated nodes (every fourth node along x and z)
    picks = [(int(i), int(z), int(y), int(x)) for i, z, y, x in zip(
        rng.integers(1, 39, 6), [2, 5, 9, 12, 3, 10], rng.integers(0, ny, 6), [2, 6, 10, 14, 17, 8])]
    for i, z, y, x in picks:
        lev.fout[i, z, y, x] *= 6.0
        lev.gout[i, z, y, x] *= 6.0
    bc_args = ([1] * 8, [6] + [1] * 7, ff, gf, [ff] * 8, [gf] * 8, [ff] * 8, [gf] * 8,
               (c.mach, 0.0, 0.0, c.temperature))
    ctx = cap.Context(0)
    lo, hi = (0, 0, 0), (nx - 1, ny - 1, nz - 1)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [list(lo) + list(hi)])
    start = 150
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=start, periodic=periodic, damp=1))
    ctx.set_links39(0, 0, st, cap.make_d3q39_bc(*bc_args))
    ctx.upload39(0, 0, lev.fout, lev.gout, lev.lm, lev.w_vel)
    steps = 2
    s = ctx.step(0, steps)
    out = ctx.download39(0)
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    b = o39.bc(*bc_args)
    damped = 0
    for step in range(start, start + steps):
        so = o39.step_links_damp(k, lev, step, st, periodic, b, prev_f, prev_g, lo, hi)
        damped += so["damped"]
    assert damped > 0 and s["exact_path_nodes"] == damped
    fluid = st[0] >= 0
    for name, ref in (("fout", lev.fout), ("gout", lev.gout)):
        rel = np.max(np.abs(out[name][:, fluid] - ref[:, fluid]) / np.abs(ref[:, fluid]))
        assert rel <= 1e-12, (name, rel)
    assert (out["fout"][:, fluid] >= 0).all()


@pytest.mark.parametrize("variable,scheme", [(1, 0), (7, 1), (5, 2), (6, 1)])
def test_d3q39_ggm_tags(pkg, o39, built_lib, variable, scheme):
    """Refinement tags by the gradient of the gradient magnitude on the device against the
    numpy restatement of calculate_grad_mag / calculate_gradgrad_mag (ggm to 1e-12, tags
    identical), on a wedge box with link codes after a few steps."""
    from oracle import ggm as og

    s39, cap = pkg.d3q39_setup, pkg.capi
    c = s39.wedge_case_consts(v_inf_ms=0.8 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=True)
    nx, ny, nz, periodic = 22, 6, 12, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = s39.wedge_state39(nx, ny, nz, 6.0, 14.0, 20.0, faces, periodic=periodic)
    lm0 = s39.freestream_start_lm(c)
    params = cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0)
    shape = (nz, ny, nx)
    ctx = cap.Context(0)
    _, f, g = ctx.d3q39_equilibrium(params, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    fs = (c.mach, 0.0, 0.0, c.temperature)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, params)
    ctx.set_links39(0, 0, st, cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8, fs))
    macro = np.stack([np.full(shape, 1.0), np.full(shape, c.mach), np.zeros(shape), np.zeros(shape),
                      np.full(shape, c.temperature)])
    ctx.init_level39(0, 0, macro, lm0)
    ctx.step(0, 4, want_stats=False)
    m = ctx.download39(0)["macro"]
    gm_all = og.ggm_tags(m, st, periodic, variable, scheme, 0.0, (1.0,) + fs)[1]
    limit = float(np.quantile(gm_all[st[0] >= 0], 0.8))  # tag about a fifth of the fluid nodes
    tags, ggm, n = ctx.ggm_tags(0, 0, variable, scheme, limit)
    rt, rg, _ = og.ggm_tags(m, st, periodic, variable, scheme, limit, (1.0,) + fs)
    ctx.close()
    assert np.max(np.abs(ggm - rg)) <= 1e-12 * max(1e-300, np.max(np.abs(rg)))
    assert np.array_equal(tags, rt) and n == int(rt.sum()) > 0


@pytest.mark.parametrize("reach,variable", [(4, 1), (2, 7)])
def test_d3q39_ggm_predictive_splitting(pkg, o39, built_lib, reach, variable):
    """Predictive splitting (predictive_splitter.f95) on the device after the GGM tags: the
    tags equal the GGM tags of the device's own ggm plus the numpy restatement's splitting
    scans over the same ggm (so that no threshold hangs on 1e-12 differences), on the
    wedge box, where the flow along +x makes u dominant almost everywhere."""
    from oracle import ggm as og

    s39, cap = pkg.d3q39_setup, pkg.capi
    c = s39.wedge_case_consts(v_inf_ms=0.8 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=True)
    nx, ny, nz, periodic = 22, 6, 12, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = s39.wedge_state39(nx, ny, nz, 6.0, 14.0, 20.0, faces, periodic=periodic)
    lm0 = s39.freestream_start_lm(c)
    params = cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0)
    shape = (nz, ny, nx)
    ctx = cap.Context(0)
    _, f, g = ctx.d3q39_equilibrium(params, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    fs = (c.mach, 0.0, 0.0, c.temperature)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, params)
    ctx.set_links39(0, 0, st, cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8, fs))
    macro = np.stack([np.full(shape, 1.0), np.full(shape, c.mach), np.zeros(shape), np.zeros(shape),
                      np.full(shape, c.temperature)])
    ctx.init_level39(0, 0, macro, lm0)
    ctx.step(0, 4, want_stats=False)
    m = ctx.download39(0)["macro"]
    # a small v or w on a few nodes takes them out of the u-dominant branch (the isotropic scan)
    m[2, :, :, ::5] = 0.5 * m[1, :, :, ::5]
    ctx.upload_macro39(0, 0, m)
    _, ggm0, _ = ctx.ggm_tags(0, 0, variable, 0, 1e300)
    fluid = st[0] >= 0
    sens = float(np.quantile(ggm0[fluid], 0.9)) / 2.0
    limit = float(np.quantile(ggm0[fluid], 0.97))
    tags, ggm, n = ctx.ggm_tags(0, 0, variable, 0, limit, pgs_sensitivity=sens, pgs_reach=reach)
    base, _, _ = ctx.ggm_tags(0, 0, variable, 0, limit)
    ctx.close()
    assert np.array_equal(ggm, ggm0)
    assert np.array_equal(base, ((ggm0 >= limit) & fluid).astype(np.uint8))
    ref = og.pgs_tags(base.copy(), ggm0, m, st, sens, reach)
    assert np.array_equal(tags, ref) and n == int(ref.sum()) > int(base.sum())


def _f_records(path):
    """Fortran unformatted sequential records of a file (4-byte length markers)."""
    data = open(path, "rb").read()
    out, k = [], 0
    while k < len(data):
        n = int(np.frombuffer(data, np.int32, 1, k)[0])
        out.append(data[k + 4:k + 4 + n])
        assert int(np.frombuffer(data, np.int32, 1, k + 4 + n)[0]) == n
        k += n + 8
    return out


def test_d3q39_plot3d_and_microphones(pkg, o39, built_lib, tmp_path):
    """Plot3D grid and data files written from the device buffers in the reference's record
    layout (plot3d_output.f95), read back and compared with the downloaded fields; microphone
    samples (weighted sums over 8 nodes, mic_write.f95) against numpy on the same fields."""
    s39, cap = pkg.d3q39_setup, pkg.capi
    c = s39.wedge_case_consts(v_inf_ms=0.8 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=True)
    nx, ny, nz, periodic = 22, 6, 12, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = s39.wedge_state39(nx, ny, nz, 6.0, 14.0, 20.0, faces, periodic=periodic)
    lm0 = s39.freestream_start_lm(c)
    params = cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0)
    shape = (nz, ny, nx)
    ctx = cap.Context(0)
    _, f, g = ctx.d3q39_equilibrium(params, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    lo = (4, 0, 2)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[lo[0], lo[1], lo[2], lo[0] + nx - 1, ny - 1,
                                                                   lo[2] + nz - 1]])
    ctx.set_d3q39_params(0, params)
    ctx.set_links39(0, 0, st, cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8,
                                                 (c.mach, 0.0, 0.0, c.temperature)))
    macro0 = np.stack([np.full(shape, 1.0), np.full(shape, c.mach), np.zeros(shape), np.zeros(shape),
                       np.full(shape, c.temperature)])
    ctx.init_level39(0, 0, macro0, lm0)
    ctx.step(0, 3, want_stats=False)
    out = ctx.download39(0)
    hdr = cap.Plot3DHeader(mach=c.mach, reynolds=1.0e5, time=3 * c.dt, gama=c.gama, t_ref=c.t_ref,
                           stag_temperature=1.2, const_vol=c.const_vol, const_press=c.const_press, non_dim_R=1.0)
    origin, dx = (0.5, -1.0, 0.25), 1e-4
    ctx.write_plot3d(0, tmp_path / "g.x", tmp_path / "d.q", origin, dx, hdr)
    rng = np.random.default_rng(2)
    nodes = rng.integers(0, nx * ny * nz, (5, 8)).astype(np.int32)
    wts = rng.uniform(0, 1, (5, 8))
    wts /= wts.sum(axis=1, keepdims=True)
    mic = ctx.mic_sample(0, 0, nodes, wts)
    ctx.close()
    N = nx * ny * nz
    g_rec = _f_records(tmp_path / "g.x")
    d_rec = _f_records(tmp_path / "d.q")
    assert np.frombuffer(g_rec[0], np.int32)[0] == 1 and np.frombuffer(d_rec[0], np.int32)[0] == 1
    assert list(np.frombuffer(g_rec[1], np.int32)) == [nx, ny, nz]
    assert list(np.frombuffer(d_rec[1], np.int32)) == [nx, ny, nz, 6, 0]
    xyz = np.frombuffer(g_rec[2], np.float32, 3 * N).reshape(3, nz, ny, nx)
    blanks = np.frombuffer(g_rec[2], np.int32, N, 12 * N).reshape(shape)
    xs = (origin[0] + lo[0] * dx + dx * np.arange(nx)).astype(np.float32)
    assert np.array_equal(xyz[0, 0, 0], xs)
    assert np.array_equal(blanks, np.where(st[0] >= 0, 1, np.where(st[0] == -666, -1, 0)))
    head = d_rec[2]
    assert len(head) == 8 * 14 + 4 * 2 and np.frombuffer(head, np.float64, 1, 0)[0] == c.mach
    assert np.frombuffer(head, np.int32, 1, len(head) - 4)[0] == 3  # timestep after 3 steps
    vals = np.frombuffer(d_rec[3], np.float64).reshape(6, nz, ny, nx)
    assert np.array_equal(vals[:5], out["macro"]) and np.array_equal(vals[5], out["alpha"])
    m = out["macro"].reshape(5, N)
    press = m[0] * (m[4] + (m[1] ** 2 + m[2] ** 2 + m[3] ** 2) / 2.0)
    for k, field in enumerate([press, m[4], m[0], m[1], m[2], m[3]]):
        ref = (wts * field[nodes]).sum(axis=1)
        assert np.allclose(mic[:, k], ref, rtol=1e-13, atol=0), k
