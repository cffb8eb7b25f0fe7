"""The benchmark configurations at their full sizes, through properties that do
not depend on size (the CPU oracle cannot run these sizes in a test):

- sphere 256x128x128 (5,120-triangle icosphere, r = 16, interpolated wall
  links): the FP32-deviation step against the FP64 step on the same GPU after
  100 steps (rho within 1e-4 relative, u within 1e-4 of the inlet speed), and
  the FP32 entropy condition in check mode;
- boundary layer 512x256x256 in a closed box: mass conserved by the FP32 step,
  every node's |dH| <= 1e-10;
- three nested D3Q27 levels (128x64x64 coarse, 2:1 refinement twice) stepped by
  the graph-driven sub-cycle: finite, no fallbacks, the coarse mass steady;
- D3Q39 384x192x48 on the shifted lattice at Mach 1.5 with inlet, outflow,
  freestream, a bounce-back floor and a periodic span, with and without the
  10-degree wedge's interpolated wall links: finite, every node updated, the
  multiplier solve never capped.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sphere_ctx(pkg, storage, st, f0, bp):
    cap = pkg.capi
    nz, ny, nx = st.shape[1:]
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f0)
    return ctx


def test_sphere_256x128x128_fp32_against_fp64(pkg, built_lib):
    geo, cap, lat = pkg.geometry, pkg.capi, pkg.lattice
    nx, ny, nz = 256, 128, 128
    st = geo.box_state27(nx, ny, nz, geo.sphere_faces())
    cap.mark_triangles(st, (0.0, 0.0, 0.0), 1.0, geo.icosphere(4, 16.0, (64.0, 64.0, 64.0)))
    f0 = geo.perturbed_equilibrium(nx, ny, nz, (0.08, 0.0, 0.0), 1e-3, seed=1236)
    solid = st[0] == -1001
    f0[:, solid] = lat.W[:, None]
    bp = geo.d3q27_boundary_params((0.08, 0.0, 0.0), 5e-4)
    out = {}
    for storage in (cap.ELBM_STORE_FP64, cap.ELBM_STORE_FP32_DEV):
        ctx = _sphere_ctx(pkg, storage, st, f0, bp)
        s = ctx.step(0, 100)
        assert s["fallbacks"] == 0 and s["status"] & 1 == 0
        out[storage] = ctx.download(0)[:, ~solid]
        if storage == cap.ELBM_STORE_FP32_DEV:
            ctx.set_d3q27_params(0, cap.make_d3q27_params(**dict(bp, check_dH=1)))
            v = ctx.step(0, 2)
            assert v["dh_over_tol"] == 0 and v["max_abs_dH"] <= 1e-10
        ctx.close()
    r64, u64 = lat.moments27(out[cap.ELBM_STORE_FP64])
    r32, u32 = lat.moments27(out[cap.ELBM_STORE_FP32_DEV])
    assert np.max(np.abs(r32 - r64) / r64) <= 1e-4
    assert np.max(np.abs(u32 - u64)) / 0.08 <= 1e-4


def test_closed_box_512x256x256_mass_and_entropy(pkg, built_lib):
    geo, cap = pkg.geometry, pkg.capi
    nx, ny, nz = 512, 256, 256
    walls = {k: -10 for k in ("x-", "x+", "y-", "y+", "z-", "z+")}
    st = geo.box_state27(nx, ny, nz, walls)
    f0 = geo.perturbed_equilibrium(nx, ny, nz, (0.0, 0.0, 0.0), 5e-3, seed=1239)
    bp = geo.d3q27_boundary_params((0.0, 0.0, 0.0), 2e-5)
    ctx = _sphere_ctx(pkg, cap.ELBM_STORE_FP32_DEV, st, f0, bp)
    m0 = ctx.download(0).sum(dtype=np.float64)
    ctx.step(0, 6, want_stats=False)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**dict(bp, check_dH=1)))
    v = ctx.step(0, 2)
    assert v["dh_over_tol"] == 0 and v["max_abs_dH"] <= 1e-10 and v["fallbacks"] == 0
    m1 = ctx.download(0).sum(dtype=np.float64)
    assert abs(m1 - m0) <= 1e-6 * m0
    ctx.close()


def _nested_state(n_valid, shell):
    nx, ny, nz = [v + 2 * shell for v in n_valid]
    st = np.zeros((27, nz, ny, nx), np.int32)
    ghost = np.ones((nz, ny, nx), bool)
    ghost[shell:-shell, shell:-shell, shell:-shell] = False
    st[0][ghost] = 10000000
    return st


def test_three_levels_graph_subcycle(pkg, built_lib):
    geo, cap = pkg.geometry, pkg.capi
    walls = {k: -10 for k in ("x-", "x+", "y-", "y+", "z-", "z+")}
    bp = geo.d3q27_boundary_params((0.0, 0.0, 0.0), 2e-3)
    ctx = cap.Context(0)
    # level 0: 128x64x64; level 1 valid [64, 191] x [32, 95] x [32, 95]; level 2 valid [192, 319] x [80, 175] x [80, 175]
    lv = [((0, 0, 0), (127, 63, 63)), ((64, 32, 32), (191, 95, 95)), ((192, 80, 80), (319, 175, 175))]
    shell = 2
    fields = []
    for l, (lo, hi) in enumerate(lv):
        n = [hi[a] - lo[a] + 1 for a in range(3)]
        if l == 0:
            st = geo.box_state27(*n, walls)
            box = list(lo) + list(hi)
        else:
            st = _nested_state(n, shell)
            box = [lo[a] - shell for a in range(3)] + [hi[a] + shell for a in range(3)]
        ctx.level_register(l, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [box])
        ctx.set_d3q27_params(l, cap.make_d3q27_params(**bp))
        ctx.set_links(l, 0, st)
        nb = [box[3 + a] - box[a] + 1 for a in range(3)]
        f = geo.perturbed_equilibrium(*nb, (0.02, 0.0, 0.0), 1e-3, seed=40 + l)
        ctx.upload(l, 0, f)
        fields.append(f)
    ctx.interlevel_setup(1)
    ctx.interlevel_setup(2)
    m0 = ctx.download(0).sum(dtype=np.float64)
    s = ctx.amr_run(3, 6)
    assert s["fallbacks"] == 0 and s["status"] & 1 == 0
    for l in range(3):
        assert np.isfinite(ctx.download(l)).all()
    m1 = ctx.download(0).sum(dtype=np.float64)
    assert abs(m1 - m0) <= 1e-3 * m0
    ctx.close()


def test_d3q39_wedge_384x192x48(pkg, built_lib):
    """The Mach 1.5 wedge case at its full size: a 10-degree wedge on the floor from x = 96 to
    x = 300 with interpolated wall links (wall distances from the geometry), inlet, pure
    outflow, freestream top, bounce-back floor, periodic span; 3 steps from a uniform
    freestream: finite, every fluid node updated, no multiplier solve capped."""
    from oracle import oracle39 as o39

    setup39, cap = pkg.d3q39_setup, pkg.capi
    c = setup39.wedge_case_consts()
    k = o39.consts(c)
    lm, f, g, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, setup39.freestream_start_lm(c))
    nx, ny, nz, periodic = 384, 192, 48, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = setup39.wedge_state39(nx, ny, nz, 96.0, 300.0, 10.0, faces, periodic=periodic)
    shape = (nz, ny, nx)
    fluid = st[0] >= 0
    walls = fluid & (st[1:] <= -1001).any(axis=0)
    assert walls.sum() > 20000
    fout = np.broadcast_to(f[:, None, None, None], (39,) + shape).copy()
    gout = np.broadcast_to(g[:, None, None, None], (39,) + shape).copy()
    lms = np.broadcast_to(lm[:, None, None, None], (13,) + shape).copy()
    macro = np.stack([np.full(shape, 1.0), np.full(shape, c.mach), np.zeros(shape), np.zeros(shape),
                      np.full(shape, c.temperature)])
    bc = cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8,
                           (c.mach, 0.0, 0.0, c.temperature))
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0))
    ctx.set_links39(0, 0, st, bc)
    ctx.upload39(0, 0, fout, gout, lms, np.zeros(shape))
    ctx.upload_macro39(0, 0, macro)
    s = ctx.step(0, 3)
    out = ctx.download39(0)
    assert s["node_updates"] == 3 * fluid.sum() and s["fallbacks"] == 0 and s["status"] & 1 == 0
    assert np.isfinite(out["fout"][:, fluid]).all() and np.isfinite(out["gout"][:, fluid]).all()
    ctx.close()


def test_d3q39_384x192x48_with_link_codes(pkg, built_lib):
    from oracle import oracle39 as o39

    setup39, cap = pkg.d3q39_setup, pkg.capi
    c = setup39.wedge_case_consts()
    assert c.shifted == 1
    k = o39.consts(c)
    lm0 = setup39.freestream_start_lm(c)
    lm, f, g, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    nx, ny, nz, periodic = 384, 192, 48, 2
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
    st = setup39.box_state39(nx, ny, nz, faces, 1, 1, periodic=periodic)
    shape = (nz, ny, nx)
    fout = np.broadcast_to(f[:, None, None, None], (39,) + shape).copy()
    gout = np.broadcast_to(g[:, None, None, None], (39,) + shape).copy()
    lms = np.broadcast_to(lm[:, None, None, None], (13,) + shape).copy()
    w = np.zeros(shape)
    bc = cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0, periodic=periodic, damp=0))
    ctx.set_links39(0, 0, st, bc)
    ctx.upload39(0, 0, fout, gout, lms, w)
    s = ctx.step(0, 3)
    out = ctx.download39(0)
    assert s["node_updates"] == 3 * nx * ny * nz and s["fallbacks"] == 0
    assert np.isfinite(out["fout"]).all() and np.isfinite(out["gout"]).all()
    ctx.close()
