"""CPU checks of the D3Q39 reference restatement (no GPU).  The reference has no
tests or golden data; these known-answer invariants pin the oracle."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def o39():
    from oracle import oracle39

    oracle39.lib()
    return oracle39


@pytest.fixture(scope="module")
def setup39(pkg):
    import importlib

    return importlib.import_module(pkg.__name__ + ".d3q39_setup")


def test_tables(o39):
    cx, cy, cz, opp = o39.tables(0, 1)
    c = np.stack([cx, cy, cz], 1)
    assert (c[opp] == -c).all() and (opp[opp] == np.arange(39)).all()
    assert sorted(np.abs(c).sum(1)) .count(0) == 1
    sx, sy, sz, sopp = o39.tables(1, 1)  # Galilean shift along +x (directions_and_weights.f95:477-499)
    assert (sx == cx + 1).all() and (sy == cy).all() and (sopp == np.arange(39)).all()


def test_reference_scales(setup39):
    c = setup39.wedge_case_consts()
    assert c.shifted == 1 and abs(c.mach - 1.5) < 1e-12
    assert abs(c.temperature - 1 / 1.4) < 1e-15 and abs(c.const_vol - 2.5) < 1e-12
    # sutherland constants are single-precision literals in the reference
    assert c.dt == c.elbm_epsilon and c.dt > 0


@pytest.mark.parametrize("shifted", [0, 1])
def test_lagrange_reproduces_moments(o39, setup39, shifted):
    c = setup39.wedge_case_consts(use_shifted=bool(shifted))
    if not shifted:
        c = setup39.reference_consts(288.15, 101325.0, 0.3 * 340.29, 1e-4)
    k = o39.consts(c)
    cx, cy, cz, _ = o39.tables(c.shifted, 1)
    cmag = cx * cx + cy * cy + cz * cz
    rng = np.random.default_rng(2)
    for _ in range(5):
        rho = 1 + rng.uniform(-0.05, 0.05)
        u = c.mach * (1 + rng.uniform(-0.05, 0.05)) if shifted else rng.uniform(-0.1, 0.3)
        v, w = rng.uniform(-0.05, 0.05, 2)
        T = c.temperature * (1 + rng.uniform(-0.03, 0.03))
        P = [rho * (T + u * u), rho * (T + v * v), rho * (T + w * w), rho * u * v, rho * u * w, rho * v * w]
        lm, fe, it = o39.lagrange(k, rho, u, v, w, T, P, setup39.freestream_start_lm(c))
        assert 0 < it < 50
        # the returned equilibrium is evaluated before the last update: residual ~ Newton step
        q = (rho * (u * u + v * v + w * w) + 5 * rho * T) * np.array([u, v, w])
        assert abs(fe.sum() - rho) < 1e-6
        assert np.allclose([(cx * fe).sum(), (cy * fe).sum(), (cz * fe).sum()], rho * np.array([u, v, w]), atol=1e-6)
        assert np.allclose([(cx * cx * fe).sum(), (cy * cy * fe).sum(), (cz * cz * fe).sum()], P[:3], atol=1e-6)
        assert np.allclose([(cx * cmag * fe).sum(), (cy * cmag * fe).sum(), (cz * cmag * fe).sum()], q, atol=1e-5)


def _uniform_level(o39, setup39, c, k, nx, ny, nz, noise=0.0, seed=0):
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
                lm, f, g, it = o39.init_node(k, rho, u, v, w, T, lm0)
                lev.fout[:, z, y, x] = f
                lev.gout[:, z, y, x] = g
                lev.lm[:, z, y, x] = lm
                lev.w_vel[z, y, x] = w
    return lev


def test_periodic_uniform_flow_is_steady(o39, setup39):
    c = setup39.wedge_case_consts()
    k = o39.consts(c)
    lev = _uniform_level(o39, setup39, c, k, 4, 3, 3)
    f0 = lev.fout.copy()
    for step in range(3):
        st = o39.step_periodic(k, lev, step)
    assert st["lm_capped"] == 0
    assert np.max(np.abs(lev.fout - f0) / np.abs(f0)) < 1e-6


def test_periodic_box_conserves_mass_and_momentum(o39, setup39):
    c = setup39.wedge_case_consts()
    k = o39.consts(c)
    lev = _uniform_level(o39, setup39, c, k, 5, 4, 4, noise=0.01, seed=3)
    cx, _, _, _ = o39.tables(1, 1)
    m0 = lev.fout.sum()
    j0 = np.tensordot(cx.astype(float), lev.fout, axes=(0, 0)).sum()
    for step in range(4):
        st = o39.step_periodic(k, lev, 150 + step)  # past start-up: closed-form alpha, full betas
    assert st["lm_capped"] == 0
    assert abs(lev.fout.sum() - m0) / m0 < 1e-6
    assert abs(np.tensordot(cx.astype(float), lev.fout, axes=(0, 0)).sum() - j0) / abs(j0) < 1e-6
    assert np.isfinite(lev.alpha).all()


def test_wall_derivative_rule_matches_reference_table(o39):
    """The oracle's rule for the seven-point wall derivatives (which axes take
    the one-sided wall form and with which up-wind flag) against the
    reference's 117-case table of first_order_shifted_vel_cond_unknown and
    first_order_shifted_temp_cond_unknown (tests/golden/ibb_deriv_table.json,
    written by tests/golden/make_ibb_deriv_table.py)."""
    import json
    import pathlib

    data = json.loads((pathlib.Path(__file__).parent / "golden" / "ibb_deriv_table.json").read_text())
    for kind in ("velocity", "temperature"):
        assert len(data[kind]) == 117
        for e in data[kind]:
            wall, up = o39.ibb_wall_axis(e["dir"] - 1, e["card"] - 1)
            assert wall == (e["form"] == "wall"), (kind, e)
            if wall:
                assert up == e["up"], (kind, e)


def test_inviscid_rule_matches_reference_table(o39):
    """The oracle's specular-reflection rule for D3Q39 inviscid links against
    inviscid_edge.f95 itself (tests/golden/inviscid_table.json, written by
    tests/golden/make_inviscid_table.py, which runs the routine through the
    f95_subset interpreter): for every direction and every combination of the
    state components its branch consults being -11, the reflected direction
    and the displacement, or no write where no branch applies; on the shifted
    lattice (primary flow along +x) the routine adds the shift to the
    displacement."""
    import json
    import pathlib

    table = json.loads((pathlib.Path(__file__).parent / "golden" / "inviscid_table.json").read_text())
    checked = 0
    for lattice, shift in (("unshifted", (0, 0, 0)), ("shifted", (1, 0, 0))):
        assert len(table[lattice]) == 38
        for key, entries in table[lattice].items():
            i = int(key) - 1
            for e in entries:
                codes = np.zeros(39, np.int32)
                codes[i] = -11
                for c in e["walls"]:
                    codes[c - 1] = -11
                ok, j, d = o39.inviscid(i, codes)
                if e["dir"] is None:
                    assert not ok, (lattice, key, e)
                else:
                    got = [d[a] + shift[a] for a in range(3)]
                    assert ok and j + 1 == e["dir"] and got == e["loc"], (lattice, key, e, j + 1, got)
                checked += 1
    assert checked == 2 * 298


@pytest.mark.parametrize("shifted", [0, 1])
def test_explode_node_known_answers(o39, setup39, shifted):
    """The ghost-node explosion of interlevel_interpolation.f95:364-440 on an equilibrium
    interpolant keeps f and g, returns the node's own moments, re-solves to the same
    multipliers and gives alpha = 2 (no departure from equilibrium); a negative f or a NaN g
    takes the coarse equilibrium f_eq(rho_c, lm) and g = (2 C_v - 3) T_c f."""
    c = setup39.wedge_case_consts(use_shifted=bool(shifted), v_inf_ms=0.8 * 340.29)
    k = o39.consts(c)
    lm0 = setup39.freestream_start_lm(c)
    rho, u, v, w, T = 1.02, 0.9 * c.mach, 0.01, -0.02, c.temperature * 1.01
    lm, f, g, it = o39.init_node(k, rho, u, v, w, T, lm0)
    assert it > 0
    f2, g2, lm2, m5, a, flags = o39.explode_node(k, 3, f, g, lm, rho, T)
    assert flags == 0 and a == 2.0
    assert np.array_equal(f2, f) and np.array_equal(g2, g)
    assert np.allclose(m5, [rho, u, v, w, T], rtol=1e-9, atol=1e-12)
    assert np.max(np.abs(lm2 - lm)) < 1e-7
    fb, gb = f.copy(), g.copy()
    fb[4], gb[9] = -0.01, np.nan
    f3, g3, _, _, _, flags = o39.explode_node(k, 3, fb, gb, lm, rho, T)
    assert flags & 1
    lead = (2 * c.const_vol - 3) * T
    for i in (4, 9):
        assert abs(f3[i] - f[i]) <= 1e-14 * f[i]  # the equilibrium of (rho_c, lm) is the uploaded f
        assert abs(g3[i] - f3[i] * lead) <= 1e-15 * g3[i]
    assert np.array_equal(np.delete(f3, [4, 9]), np.delete(fb, [4, 9]))


def test_unshifted_wall_closure_matches_reference_formulas(o39):
    """The coefficient tables of the unshifted D3Q39 wall closure (generated from
    interpolative_bounceback_bc.f95:834-2838) evaluated by the oracle against the
    reference's own statements run in float64 (tests/golden/ibb39_unshifted_golden.json):
    fi_neq / k_fi and gi_neq / k_gi of all 38 directions, 3 input sets each, to 1e-12."""
    import ctypes as ct
    import json
    import pathlib

    L = o39.lib()
    L.o39_ibb39_unshifted_terms.restype = None
    L.o39_ibb39_unshifted_terms.argtypes = [ct.c_int, ct.c_void_p] + [ct.c_double] * 7 + [ct.POINTER(ct.c_double)] * 2
    gold = json.loads((pathlib.Path(__file__).parent / "golden" / "ibb39_unshifted_golden.json").read_text())
    assert sorted(int(d) for d in gold) == list(range(1, 39))
    for d, rows in gold.items():
        for r in rows:
            D = np.ascontiguousarray(r["D"], np.float64)
            fp, gp = ct.c_double(), ct.c_double()
            L.o39_ibb39_unshifted_terms(int(d), D.ctypes.data, r["u"], r["v"], r["w"], r["T"], r["b1"], r["b2"],
                                        r["cv"], ct.byref(fp), ct.byref(gp))
            assert abs(fp.value - r["fpoly"]) <= 1e-12 * abs(r["fpoly"]), (d, fp.value, r["fpoly"])
            assert abs(gp.value - r["gpoly"]) <= 1e-12 * abs(r["gpoly"]), (d, gp.value, r["gpoly"])


@pytest.mark.parametrize("u,expect", [(0.1, [2, 3, 4, 5]), (-0.1, [0, 1, 2])])
def test_predictive_splitting_known_answers(u, expect):
    """predictive_splitter.f95 on a line of 10 nodes with one ggm spike at x = 2, reach 3:
    flow along +x tags from the spike to every node up to 3 downstream of it; flow along -x
    tags the nodes up to 3 upstream of the spike (scan from the node outwards)."""
    from oracle import ggm as og

    nx = 10
    macro = np.zeros((5, 1, 1, nx))
    macro[1] = u
    ggm = np.zeros((1, 1, nx))
    ggm[0, 0, 2] = 1.0
    tags = og.pgs_tags(np.zeros((1, 1, nx), np.uint8), ggm, macro, None, 0.4, 3)
    assert np.nonzero(tags[0, 0])[0].tolist() == expect
    # no dominant component: only the spike itself, when it reaches 3 x sensitivity
    macro[2] = u
    assert og.pgs_tags(np.zeros((1, 1, nx), np.uint8), ggm, macro, None, 0.3, 3)[0, 0].tolist() == \
        [0, 0, 1] + [0] * 7
    assert og.pgs_tags(np.zeros((1, 1, nx), np.uint8), ggm, macro, None, 0.4, 3).sum() == 0


def test_explode39_uniform_coarse_state_is_kept(o39, setup39):
    """The D3Q39 explosion restatement on a uniform coarse equilibrium: every fine ghost
    node takes that state unchanged (means of equal values, no population replaced, the
    multiplier solve converging where it starts, alpha = 2), and the coalescence copies a
    valid fine node's arrays onto the coarse node under it."""
    from oracle import interlevel as il

    c = setup39.wedge_case_consts(use_shifted=True, v_inf_ms=0.8 * 340.29)
    k = o39.consts(c)
    lm0 = setup39.freestream_start_lm(c)
    rho, u, T = 1.0, c.mach, c.temperature
    lm, f, g, _ = o39.init_node(k, rho, u, 0.0, 0.0, T, lm0)
    shape = (4, 4, 4)
    coarse = {"f": np.broadcast_to(f[:, None, None, None], (39,) + shape).copy(),
              "g": np.broadcast_to(g[:, None, None, None], (39,) + shape).copy(),
              "lm": np.broadcast_to(lm[:, None, None, None], (13,) + shape).copy(),
              "w": np.zeros(shape), "alpha": np.full(shape, 2.0),
              "macro": np.broadcast_to(np.array([rho, u, 0.0, 0.0, T])[:, None, None, None], (5,) + shape).copy()}
    fshape = (5, 5, 5)
    fine = {"f": np.zeros((39,) + fshape), "g": np.zeros((39,) + fshape), "lm": np.zeros((13,) + fshape),
            "w": np.ones(fshape), "alpha": np.zeros(fshape), "macro": np.zeros((5,) + fshape)}
    ghost = np.zeros(fshape, bool)
    ghost[0] = ghost[-1] = True
    rep, capped = il.explode39(k, 3, coarse, (0, 0, 0), fine, (1, 1, 1), ghost)
    assert rep == 0 and capped == 0
    assert np.allclose(fine["f"][:, ghost], f[:, None], rtol=1e-14, atol=0)
    assert np.allclose(fine["g"][:, ghost], g[:, None], rtol=1e-14, atol=0)
    assert np.max(np.abs(fine["lm"][:, ghost] - lm[:, None])) < 1e-7
    assert np.allclose(fine["alpha"][ghost], 2.0) and np.allclose(fine["macro"][1][ghost], u, rtol=1e-12)
    assert np.all(fine["f"][:, ~ghost] == 0.0)  # valid fine nodes untouched
    fine["f"][:, 1, 1, 1] = 7.0  # fine (1,1,1) at global (2,2,2) lies over coarse (1,1,1)
    il.average_down39(fine, (1, 1, 1), ~ghost, coarse, (0, 0, 0), np.ones(shape, bool))
    assert np.all(coarse["f"][:, 1, 1, 1] == 7.0) and np.all(coarse["f"][:, 0, 0, 0] == f)
