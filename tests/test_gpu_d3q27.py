"""GPU parity of the D3Q27 level step through the C ABI against the CPU oracle.

Tolerances: FP64 storage <= 1e-12 relative in every population; FP32 deviation
storage <= 1e-4 relative in rho and u (velocity error relative to the inlet speed).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U_IN = (0.05, 0.0, 0.0)


def _setup(pkg, nx, ny, nz, storage, u0=U_IN, nu=1e-3, noise=1e-3, faces=None, seed=1234, **pkw):
    geo, cap = pkg.geometry, pkg.capi
    st = geo.box_state27(nx, ny, nz, faces or geo.flat_plate_faces())
    f0 = geo.perturbed_equilibrium(nx, ny, nz, u0, noise, seed=seed)
    bp = geo.d3q27_boundary_params(u0, nu)
    bp.update(pkw)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f0)
    return ctx, st, f0, bp


def _oracle_run(orc, st, f0, bp, steps):
    p = orc.params(bp["nu"], bp["fs_feq"], bp["inl_feq"], bp["outl_feq"], bp["outlet_type"],
                   alpha_mode=bp.get("alpha_mode", 1))
    f = f0
    alpha = None
    for _ in range(steps):
        f, alpha, _, s = orc.step27(st, f, p)
    return f, alpha, s


def test_fp64_parity_small(pkg, orc, built_lib):
    ctx, st, f0, bp = _setup(pkg, 24, 16, 12, pkg.capi.ELBM_STORE_FP64, record_alpha=1)
    stats = ctx.step(0, 100)
    f_gpu = ctx.download(0)
    a_gpu = ctx.download_alpha(0)
    f_ref, a_ref, s_ref = _oracle_run(orc, st, f0, bp, 100)
    rel = np.max(np.abs(f_gpu - f_ref) / np.abs(f_ref))
    assert rel <= 1e-12, rel
    assert np.max(np.abs(a_gpu - a_ref)) <= 1e-6  # alpha is recorded in FP32
    assert stats["node_updates"] == 100 * 24 * 16 * 12
    assert stats["status"] & ~pkg.capi.ELBM_ST_NEWTON_FALLBACK == 0
    assert stats["fallbacks"] == 0 and s_ref["fallbacks"] == 0


def test_fp64_parity_flat_plate_64cubed_200_steps(pkg, orc, built_lib):
    """The 64^3 flat-plate boundary layer, 200 steps, Newton alpha from 2 at tol 1e-12."""
    n = 64
    ctx, st, f0, bp = _setup(pkg, n, n, n, pkg.capi.ELBM_STORE_FP64)
    ctx.step(0, 200, want_stats=False)
    f_gpu = ctx.download(0)
    f_ref, _, s_ref = _oracle_run(orc, st, f0, bp, 200)
    rel = np.max(np.abs(f_gpu - f_ref) / np.abs(f_ref))
    assert rel <= 1e-12, rel
    assert s_ref["fallbacks"] == 0 and s_ref["max_abs_dH"] <= 1e-10


@pytest.mark.parametrize("shape,steps", [((32, 16, 16), 200), ((48, 24, 20), 400)])
def test_fp32_deviation_storage_vs_oracle(pkg, orc, built_lib, shape, steps):
    nx, ny, nz = shape
    ctx, st, f0, bp = _setup(pkg, nx, ny, nz, pkg.capi.ELBM_STORE_FP32_DEV, record_alpha=1)
    stats = ctx.step(0, steps)
    f_gpu = ctx.download(0)
    a_gpu = ctx.download_alpha(0)
    f_ref, a_ref, _ = _oracle_run(orc, st, f0, bp, steps)
    lat = pkg.lattice
    rg, ug = lat.moments27(f_gpu)
    rr, ur = lat.moments27(f_ref)
    err_rho = np.max(np.abs(rg - rr) / rr)
    err_u = np.max(np.abs(ug - ur)) / abs(U_IN[0])
    assert err_rho <= 1e-4, err_rho
    assert err_u <= 1e-4, err_u
    assert np.max(np.abs(a_gpu - a_ref)) <= 1e-3
    assert stats["status"] & pkg.capi.ELBM_ST_NAN == 0


def test_fp32_entropy_condition(pkg, built_lib):
    """Check mode: every node's |H(f + alpha Delta) - H(f)| <= 1e-10 (FP64 evaluation)."""
    ctx, *_ = _setup(pkg, 64, 32, 32, pkg.capi.ELBM_STORE_FP32_DEV, nu=2e-5, noise=5e-3, check_dH=1,
                     u0=(0.06, 0.0, 0.0))
    stats = ctx.step(0, 50)
    assert stats["dh_over_tol"] == 0 and stats["max_abs_dH"] <= 1e-10, stats
    assert stats["fallbacks"] <= 1e-5 * stats["node_updates"], stats


@pytest.mark.parametrize("storage", [0, 1])
def test_closed_box_mass(pkg, built_lib, storage):
    geo = pkg.geometry
    faces = {k: geo.CODE_BOUNCEBACK for k in ("x-", "x+", "y-", "y+", "z-", "z+")}
    ctx, st, f0, bp = _setup(pkg, 20, 18, 16, storage, u0=(0, 0, 0), noise=2e-2, faces=faces)
    ctx.step(0, 100, want_stats=False)
    f = ctx.download(0)
    drift = abs(f.sum() - f0.sum()) / f0.sum()
    assert drift <= (1e-13 if storage == 0 else 1e-6), drift


def test_fab_ghosts_round_trip(pkg, built_lib):
    cap = pkg.capi
    nx, ny, nz, g = 10, 7, 5, 2
    rng = np.random.default_rng(0)
    fab = rng.uniform(0.001, 0.3, size=(27, nz + 2 * g, ny + 2 * g, nx + 2 * g))
    for storage, tol in ((cap.ELBM_STORE_FP64, 0.0), (cap.ELBM_STORE_FP32_DEV, 1e-7)):
        ctx = cap.Context(0)
        ctx.level_register(0, cap.ELBM_D3Q27, storage, [[3, 4, 5, 3 + nx - 1, 4 + ny - 1, 5 + nz - 1]], ngrow=g)
        ctx.upload(0, 0, fab)
        out = np.zeros_like(fab)
        ctx.download(0, 0, out)
        inner = (slice(None), slice(g, g + nz), slice(g, g + ny), slice(g, g + nx))
        # FP32 deviation storage rounds d = f - w to float: error <= 2^-24 |f - w|
        dev = np.abs(fab[inner] - pkg.lattice.W[:, None, None, None])
        assert np.all(np.abs(out[inner] - fab[inner]) <= tol * dev + 1e-300)
        ctx.close()


def test_error_codes(pkg, built_lib):
    cap, geo = pkg.capi, pkg.geometry
    ctx = cap.Context(0)
    with pytest.raises(cap.ElbmError) as e:
        ctx.step(0, 1)
    assert e.value.rc == cap.ELBM_E_ARG
    ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP64, [[0, 0, 0, 7, 7, 7]])
    bp = geo.d3q27_boundary_params(U_IN, 1e-3)
    with pytest.raises(cap.ElbmError) as e:
        ctx.set_links(0, 0, geo.box_state27(8, 8, 8, geo.flat_plate_faces()))
    assert e.value.rc == cap.ELBM_E_STATE
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    faces = geo.flat_plate_faces()
    faces["z+"] = -1  # a code the reference itself cannot honour (bc_switchboard calls rho_v_bc() without arguments)
    with pytest.raises(cap.ElbmError) as e:
        ctx.set_links(0, 0, geo.box_state27(8, 8, 8, faces))
    assert e.value.rc == cap.ELBM_E_UNSUPPORTED
    ctx.set_links(0, 0, geo.box_state27(8, 8, 8, geo.flat_plate_faces()))
    with pytest.raises(cap.ElbmError) as e:
        ctx.step(0, 1)
    assert e.value.rc == cap.ELBM_E_STATE
    bad = cap.make_d3q27_params(**bp)
    bad.nu = -1.0
    with pytest.raises(cap.ElbmError) as e:
        ctx.set_d3q27_params(0, bad)
    assert e.value.rc == cap.ELBM_E_ARG
    ctx.close()


def _sphere_setup(pkg, storage, nx=40, ny=24, nz=24, radius=6.0, center=(12.0, 12.0, 12.0), u0=(0.08, 0.0, 0.0),
                  nu=5e-4, **pkw):
    geo, cap = pkg.geometry, pkg.capi
    st = geo.box_state27(nx, ny, nz, geo.sphere_faces())
    cap.mark_triangles(st, (0.0, 0.0, 0.0), 1.0, geo.icosphere(3, radius, center))
    f0 = geo.perturbed_equilibrium(nx, ny, nz, u0, 1e-3, seed=1236)
    f0[:, st[0] == -1001] = pkg.lattice.W[:, None]  # solid nodes at rest
    bp = geo.d3q27_boundary_params(u0, nu)
    bp.update(pkw)
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, storage, [[0, 0, 0, nx - 1, ny - 1, nz - 1]])
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, f0)
    return ctx, st, f0, bp


def test_sphere_ibb_fp64_parity(pkg, orc, built_lib):
    """Flow past an icosphere with interpolated bounce-back wall links, FP64, 100 steps."""
    ctx, st, f0, bp = _sphere_setup(pkg, pkg.capi.ELBM_STORE_FP64)
    stats = ctx.step(0, 100)
    f_gpu = ctx.download(0)
    f_ref, _, s_ref = _oracle_run(orc, st, f0, bp, 100)
    fluid = st[0] != -1001
    rel = np.max(np.abs(f_gpu[:, fluid] - f_ref[:, fluid]) / np.abs(f_ref[:, fluid]))
    assert rel <= 1e-12, rel
    assert stats["fallbacks"] == 0 and s_ref["fallbacks"] == 0


def test_sphere_ibb_fp32_vs_oracle(pkg, orc, built_lib):
    ctx, st, f0, bp = _sphere_setup(pkg, pkg.capi.ELBM_STORE_FP32_DEV)
    ctx.step(0, 200, want_stats=False)
    f_gpu = ctx.download(0)
    f_ref, _, _ = _oracle_run(orc, st, f0, bp, 200)
    fluid = st[0] != -1001
    lat = pkg.lattice
    rg, ug = lat.moments27(f_gpu[:, fluid])
    rr, ur = lat.moments27(f_ref[:, fluid])
    assert np.max(np.abs(rg - rr) / rr) <= 1e-4
    assert np.max(np.abs(ug - ur)) / 0.08 <= 1e-4


@pytest.mark.parametrize("shape,variant", [((128, 20, 16), 2), ((200, 12, 10), 2), ((200, 12, 10), 3),
                                           ((64, 32, 32), 1), ((64, 32, 32), 5), ((64, 32, 32), 6),
                                           ((64, 32, 32), 7), ((64, 32, 32), 8), ((200, 12, 10), 8),
                                           ((40, 20, 16), 8), ((24, 20, 16), 8), ((260, 6, 5), 8),
                                           ((64, 32, 32), 9), ((200, 12, 10), 9)])
def test_kernel_variants_match_direct(pkg, built_lib, shape, variant):
    """Every step-kernel variant (1, 5, 6, 7: register-capped, 2: bulk-copy
    staged, 3: persistent warps, 8: warp-specialised tensor copies, with
    128-, 64- and 32-wide tiles and partial tiles in x and y, 9: pull offsets
    as kernel parameters) computes the
    same step as the direct kernel (variant 0): same node updates,
    populations equal to FP32 rounding, no copy timeouts."""
    nx, ny, nz = shape
    out = {}
    for v in (0, variant):
        ctx, *_ = _setup(pkg, nx, ny, nz, pkg.capi.ELBM_STORE_FP32_DEV, nu=2e-5, noise=5e-3, u0=(0.06, 0.0, 0.0))
        ctx.set_kernel_variant(0, v)
        s = ctx.step(0, 30)
        out[v] = (s, ctx.download(0))
        ctx.close()
    (s0, f0), (s2, f2) = out[0], out[variant]
    assert s2["status"] & 0x10 == 0
    assert s0["node_updates"] == s2["node_updates"] == 30 * nx * ny * nz
    assert np.max(np.abs(f2 - f0)) <= 1e-6, np.max(np.abs(f2 - f0))
