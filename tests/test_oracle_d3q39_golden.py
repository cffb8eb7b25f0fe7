"""The D3Q39 oracle's core against golden values run from the reference's own
Fortran statements (tests/golden/d3q39_core_golden.json, made by
tests/golden/make_d3q39_core_golden.py through the f95_subset interpreter):
lattice tables, equilibrium, the multiplier Jacobian of both branches (the
unshifted one hand-expanded in calculate_lagrangian_mults.f95:341-695, the
shifted one generic, :696-1097), the LU update with its two index quirks
(lu_decomp.f95:105, :441), the whole multiplier solve, the closed-form alpha
(calculate_alpha.f95), the heat-flux corrections (find_q_bar.f95,
find_little_q_bar.f95), the flow variables of a node
(calculate_flow_variables.f95:192-228, with the pressure-tensor target P_zz
read from the stored w), the wall targets (target_finder.f95), the shifted
lattice's wall closure (shifted_ibb.f95 with the derivatives module), the
per-node explosion of interlevel_interpolation.f95, the
two-population collision of a node
(collision.f95), inside and after the start-up ramps, and the negative-
population repair's sweep over a box (damp_it.f95, d3q39_damp_golden.json),
and the push loop of streaming.f95 with its boundary routines
(d3q39_push_golden.json).

The oracle sums in its own order (generic loops where the reference spells
terms out), so the bar is 1e-13 relative to each quantity's scale; the LU
update, written in the reference's statement order, matches bit for bit."""
import json
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "d3q39_core_golden.json"
DATA = json.loads(GOLDEN.read_text())
LATTICES = sorted(DATA["lattices"])
DAMP = json.loads((GOLDEN.parent / "d3q39_damp_golden.json").read_text())
PUSH = json.loads((GOLDEN.parent / "d3q39_push_golden.json").read_text())


@pytest.fixture(scope="module")
def o39():
    from oracle import oracle39

    return oracle39


def _consts(o39, lat):
    k = o39.O39Consts()
    for name, v in lat["consts"].items():
        setattr(k, name, v)
    for i, v in enumerate(lat["su_lm"]):
        k.su_lm[i] = v
    k.max_lm_iters = 200
    return k


def _close(a, b, tol=1e-13):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale) <= tol, float(np.max(np.abs(a - b)) / scale)


@pytest.mark.parametrize("name", LATTICES)
def test_tables(o39, name):
    lat = DATA["lattices"][name]
    cx, cy, cz, opp = o39.tables(lat["consts"]["shifted"], lat["consts"]["primary_flow_dir"])
    assert cx.tolist() == lat["tables"]["cx"]
    assert cy.tolist() == lat["tables"]["cy"]
    assert cz.tolist() == lat["tables"]["cz"]
    assert (opp + 1).tolist() == lat["tables"]["opp"] or opp.tolist() == lat["tables"]["opp"]


@pytest.mark.parametrize("name", LATTICES)
def test_equilibrium_and_jacobian(o39, name):
    lat = DATA["lattices"][name]
    sh, pfd = lat["consts"]["shifted"], lat["consts"]["primary_flow_dir"]
    for c in lat["cases"]:
        lu0 = c["lu"][0]
        ok, err = _close(o39.fieq(sh, pfd, c["rho"], lu0["lm_in"]), c["expo0"], 1e-14)
        assert ok, f"equilibrium: {err}"
        ok, err = _close(o39.jacobian(sh, pfd, c["expo0"]).ravel(), lu0["jacobian"])
        assert ok, f"jacobian: {err}"
        for rec in c["lu"][1:]:
            ok, err = _close(o39.jacobian(sh, pfd, o39.fieq(sh, pfd, c["rho"], rec["lm_in"])).ravel(),
                             rec["jacobian"])
            assert ok, f"jacobian of a later iteration: {err}"


def _target(m):
    rho, u, v, w = m[0], m[1], m[2], m[3]
    return [rho, rho * u, rho * v, rho * w] + list(m[4:13])


@pytest.mark.parametrize("name", LATTICES)
def test_lu_update_bitwise(o39, name):
    lat = DATA["lattices"][name]
    for c in lat["cases"]:
        for rec in c["lu"]:
            lm, md = o39.lu_update(rec["jacobian"], _target(rec["moments"]), rec["lm_in"])
            assert lm.tolist() == rec["lm_out"]
            assert md == rec["max_diff"]


@pytest.mark.parametrize("name", LATTICES)
def test_multiplier_solve(o39, name):
    lat = DATA["lattices"][name]
    k = _consts(o39, lat)
    for c in lat["cases"]:
        lm, fe, it = o39.lagrange(k, c["rho"], c["u"], c["v"], c["w"], c["T"], c["P"], c["lm0"])
        assert it == c["iterations"]
        ok, err = _close(lm, c["lm"], 1e-12)
        assert ok, f"multipliers: {err}"
        ok, err = _close(fe, c["fieq"], 1e-12)
        assert ok, f"equilibrium: {err}"


@pytest.mark.parametrize("name", LATTICES)
def test_alpha_heat_flux_and_collision(o39, name):
    lat = DATA["lattices"][name]
    k = _consts(o39, lat)
    for c in lat["cases"]:
        u, v, w, T = c["u"], c["v"], c["w"], c["T"]
        for step_s, ref in c["steps"].items():
            step = int(step_s)
            a = o39.alpha(k, np.array(c["f"]), np.array(c["fd"]), T, step)
            assert abs(a - ref["alpha"]) <= 1e-12, (step, a, ref["alpha"])
            ok, err = _close(o39.q_bar(k, c["fd"], u, v, w, T, step), ref["q_bar"])
            assert ok, f"q_bar step {step}: {err}"
            ok, err = _close(o39.little_q_bar(k, c["gd"], u, v, w, T, step), ref["little_q_bar"])
            assert ok, f"little q_bar step {step}: {err}"
            fo, go = o39.collide_node(k, c["f"], c["g"], c["lm"], c["rho"], u, v, w, T, ref["alpha"], step)
            ok, err = _close(fo, ref["fout"])
            assert ok, f"fout step {step}: {err}"
            ok, err = _close(go, ref["gout"])
            assert ok, f"gout step {step}: {err}"


@pytest.mark.parametrize("name", LATTICES)
def test_flow_variables(o39, name):
    """rho, u, v, w, T, the six pressure-tensor targets and the pressure from f and g:
    the same sums in the same order as the reference's statements, so bit for bit;
    P_zz takes the stored w, the new w enters P_xz and P_yz."""
    lat = DATA["lattices"][name]
    k = _consts(o39, lat)
    for c in lat["cases"]:
        fl = c["flow"]
        out = o39.flow_vars(k, c["f"], c["g"], fl["w_old"])
        assert out.tolist() == fl["out"], (out.tolist(), fl["out"])
        rho, u, v, w, T = out[:5]
        assert out[7] == rho * (T + fl["w_old"] ** 2) and out[7] != rho * (T + w * w)


@pytest.mark.parametrize("name", LATTICES)
def test_alpha_branches(o39, name):
    """calculate_alpha.f95 on deviations from equilibrium scaled from 1e-12 to 0.9 of the
    populations, before and after the start-up ramp: the alpha = 2 branch below the chi_3
    threshold, the quadratic root and its clamps, within 1e-12."""
    lat = DATA["lattices"][name]
    k = _consts(o39, lat)
    seen = set()
    for c in lat["alpha_branches"]:
        a = o39.alpha(k, np.array(c["f"]), np.array(c["fd"]), c["T"], c["step"])
        assert abs(a - c["alpha"]) <= 1e-12, (a, c["alpha"], c["step"])
        seen.add(round(c["alpha"], 12) == 2.0)
    assert seen == {True, False}


@pytest.mark.parametrize("name", LATTICES)
def test_wall_targets(o39, name):
    """target_finder.f95's rho, u, v, w, T targets of a wall node from its link codes,
    the fields at x + c_j and its slots (unshifted: the node across a fluid opposite
    link, else the node itself at the freestream temperature; shifted: x + c_j beside
    a null link, else direction 5), bit for bit."""
    lat = DATA["lattices"][name]
    k = _consts(o39, lat)
    for c in lat["targets"]:
        out = o39.target_finder(k, c["code"], c["u"], c["v"], c["w"], c["T"], c["fi"], c["fs_temp"])
        assert out.tolist() == c["out"], (out.tolist(), c["out"])


@pytest.mark.parametrize("name", LATTICES)
def test_explode_node(o39, name):
    """interlevel_interpolation.f95's per-node explosion of a fine ghost node (after the
    coarse-to-fine interpolation, which is AMReX's): the populations with a negative f
    or a NaN g replaced by the coarse equilibrium, the moments, the multiplier solve from
    the coarse multipliers and alpha.  f, g and the moments bit for bit; the multipliers
    (the Newton stops at |delta| <= 1e-7, with its sums ordered the oracle's way) within
    1e-10 of their scale, alpha within 1e-12."""
    lat = DATA["lattices"][name]
    k = _consts(o39, lat)
    for c in lat["explode"]:
        f = np.array([np.nan if x is None else x for x in c["f"]])
        g = np.array([np.nan if x is None else x for x in c["g"]])
        f2, g2, lm2, m5, a, flags = o39.explode_node(k, c["step"], f, g, np.array(c["lm"]), c["rho"], c["T"])
        ref = c["out"]
        assert f2.tolist() == ref["f"] and g2.tolist() == ref["g"]
        assert list(m5) == ref["m5"]
        lm_ref = np.array(ref["lm"])
        assert np.max(np.abs(lm2 - lm_ref)) <= 1e-10 * np.max(np.abs(lm_ref))
        assert abs(a - ref["alpha"]) <= 1e-12
        assert bool(flags) == (None in c["f"] or None in c["g"])


def test_shifted_wall_closure(o39):
    """shifted_ibb.f95 (the Grad-type closure of a wall link on the shifted lattice, with
    the derivatives module's one-sided wall and local stencil derivatives) against the
    oracle's shifted_ibb39: fout and gout bit for bit, before and after the start-up
    ramps, with interior, solid and null stencil nodes."""
    lat = DATA["lattices"]["shifted"]
    k = _consts(o39, lat)
    for c in lat["shifted_ibb"]:
        out = o39.shifted_ibb(k, c["i"] - 1, c["step"], c["fieq"], c["gieq"], c["rho"], c["tgt"], c["u"], c["v"],
                              c["w"], c["T"], c["sp"])
        assert out.tolist() == [c["fout"], c["gout"]], (c["i"], c["step"], out.tolist(), c["fout"], c["gout"])


@pytest.mark.parametrize("name", sorted(n for n in PUSH if "fi_wall" in PUSH[n]))
def test_push_loop_with_wall_links(o39, pkg, name):
    """The push loop with interpolated wall links against streaming.f95 run through the
    interpreter: the shifted lattice's double-ramp wedge (target_finder at each wall
    node's first wall link, the target multiplier solve from the start-up multipliers at
    timestep 0 or the node's own ones later, the seven-point stencil and shifted_ibb) and
    an unshifted box with a solid block (interpolative_bounceback_bc's 38 closures):
    every slot a wall closure cannot reach bit for bit; those it can (slots i and opp(i)
    of wall link i), whose multiplier and closure sums the oracle orders its own way,
    within 1e-13."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    import push39_inputs as P

    ref = PUSH[name]
    if name == "unshifted_walls":
        c, cs = P.unshifted_wall_case(pkg.d3q39_setup)
    else:
        c, cs = pkg.d3q39_setup.wedge_case_consts(), P.wall_case(name, pkg.d3q39_setup)
    k = o39.consts(c)
    lev = o39.Level39(P.WNX, P.WNY, P.WNZ)
    lev.fout[...], lev.gout[...], lev.lm[...] = cs["fout"], cs["gout"], cs["lm"]
    lev.rho[...], lev.u[...], lev.v[...], lev.w_vel[...], lev.temp[...] = cs["fields"]
    pf, pg = cs["prev_f"].copy(), cs["prev_g"].copy()
    b = o39.bc(cs["inlet_type"], cs["outlet_type"], cs["ff"], cs["gf"], [cs["fi"]] * 8, [cs["gi"]] * 8,
               [cs["fo"]] * 8, [cs["go"]] * 8, cs["fs_uvwT"])
    o39.step_links(k, lev, cs["step"], cs["state"], 0, b, pf, pg)
    fluid = cs["state"][0] >= 0
    wall = (cs["state"] <= -1001) & fluid[None]
    wall[0] = False
    wall = wall | wall[pkg.d3q39_setup.lattice39(cs["shifted"], 1)[3]]
    assert int(fluid.sum()) == ref["fluid_nodes"] and int(wall.sum()) == ref["wall_slots"]
    other = fluid[None] & ~wall
    assert P.digest(pf[other]) == ref["fi"] and P.digest(pg[other]) == ref["gi"]
    for got, key in ((pf[wall], "fi_wall"), (pg[wall], "gi_wall")):
        want = np.array(ref[key])
        assert np.max(np.abs(got - want) / np.abs(want)) <= 1e-13, key


@pytest.mark.parametrize("name", sorted(n for n in PUSH if "fi_wall" not in PUSH[n]))
def test_push_loop(o39, pkg, name):
    """The oracle's push loop (o39_step_links) against streaming.f95's own sweep with
    the boundary routines it calls, on boxes with inlet, outlet, bounce-back,
    freestream, inviscid and null links: the post-streaming fi and gi of every fluid
    node bit for bit (sha-256 digests of the reference's arrays; slots no rule writes
    keep the previous step's values on both sides)."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    import push39_inputs as P

    ref = PUSH[name]
    k = o39.O39Consts()
    for n, v in ref["consts"].items():
        setattr(k, n, v)
    k.max_lm_iters = 200
    cs = P.case(name, pkg.d3q39_setup)
    lev = o39.Level39(P.NX, P.NY, P.NZ)
    lev.fout[...] = cs["fout"]
    lev.gout[...] = cs["gout"]
    pf, pg = cs["prev_f"].copy(), cs["prev_g"].copy()
    b = o39.bc(cs["inlet_type"], cs["outlet_type"], cs["ff"], cs["gf"], [cs["fi"]] * 8, [cs["gi"]] * 8,
               [cs["fo"]] * 8, [cs["go"]] * 8)
    o39.step_links(k, lev, 0, cs["state"], cs["periodic"], b, pf, pg)
    fluid = cs["state"][0] >= 0
    assert int(fluid.sum()) == ref["fluid_nodes"]
    assert P.digest(pf[:, fluid]) == ref["fi"]
    assert P.digest(pg[:, fluid]) == ref["gi"]


@pytest.mark.parametrize("name", sorted(DAMP))
def test_damp_sweep(o39, name):
    """damp_it.f95's in-place sweep over a box with link codes, fout and gout (the same
    rules on each), against the reference's statements: every population bit for bit,
    the repaired ones and the negative ones no rule changes (shifted lattice: link and
    upstream node type both below -500 away from the band) alike."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    import damp39_inputs as D

    ref = DAMP[name]
    k = o39.O39Consts()
    for n, v in ref["consts"].items():
        setattr(k, n, v)
    fo, go, st, fs_f, fs_g = D.case(name)
    lo, hi = D.bounds(name)
    assert list(lo) == ref["lo"] and list(hi) == ref["hi"]
    for pop, fs, key, nneg in ((fo, fs_f, "changed_f", "negative_f"), (go, fs_g, "changed_g", "negative_g")):
        assert int((pop < 0).sum()) == ref[nneg]
        out, count = o39.damp(k, pop, st, lo, hi, fs)
        want = pop.ravel().copy()
        for j, v in ref[key]:
            want[j] = v
        assert count == ref[nneg]
        assert np.array_equal(out.ravel(), want), (key, int((out.ravel() != want).sum()))


def test_ggm_derivative():
    """The GGM restatement's derivative (oracle/ggm.py windage2) against
    derivative_windage_secondord / _firstord of derivatives.f95 run through the
    interpreter: every combination of the four link states, the central, upwind and
    downwind schemes and both wind signs, bit for bit (the central form's sign and the
    upwind forms' use of the minus-side values on the plus side included)."""
    from oracle import ggm as og

    assert len(DATA["windage"]) == 96
    for r in DATA["windage"]:
        s = r["state"]
        got = og.windage2(r["q"], (s[1] >= 0, s[2] >= 0, s[3] >= 0, s[4] >= 0), r["wind"], r["scheme"])
        assert got == r["dq"], r


def test_ggm_gradients():
    """oracle/ggm.py's gradient magnitudes and tags against calculate_grad_mag.f95 and
    calculate_gradgrad_mag.f95 run through the interpreter on seeded boxes (boundary
    links, solid and null nodes; central, upwind and downwind schemes): gm at every node
    and ggm and the tags where the +-2 stencil stays inside the box, bit for bit."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    import pgs_inputs as P
    import push39_inputs as Q
    from oracle import ggm as og

    for ref in DATA["ggm"]:
        rho, u, v, w, state, rho_fs = P.ggm_case(ref["scheme"])
        macro = np.stack([rho, u, v, w, np.ones_like(rho)])
        tags, ggm, gm = og.ggm_tags(macro, state, 0, 1, ref["scheme"], ref["limit"], (rho_fs, 0.0, 0.0, 0.0, 1.0))
        inner = np.zeros(rho.shape, bool)
        inner[2:-2, 2:-2, 2:-2] = True
        assert Q.digest(gm) == ref["gm"]
        assert Q.digest(ggm[inner]) == ref["ggm_inner"]
        assert np.flatnonzero(tags[inner]).tolist() == ref["tagged_inner"]


def test_predictive_splitting():
    """oracle/ggm.py's predictive splitting against predictive_splitter.f95's loop run
    through the interpreter on a seeded box (dominant-velocity scans upstream and
    downstream, the isotropic scans, solid nodes): the same tags."""
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    import pgs_inputs as P
    from oracle import ggm as og

    ggm, u, v, w, s0 = P.case()
    macro = np.stack([np.ones_like(u), u, v, w, np.ones_like(u)])
    state = np.zeros((39,) + s0.shape, np.int32)
    state[0] = s0
    tags = np.zeros(s0.shape, np.uint8)
    og.pgs_tags(tags, ggm, macro, state, P.SENSITIVITY, P.MAX_SCAN)
    assert np.flatnonzero(tags.ravel()).tolist() == DATA["pgs"]["tagged"]


def test_lu_update_dense_bitwise_with_quirks(o39):
    """lu_decomp on dense matrices: the oracle matches bit for bit, and the
    golden results differ from a plain LU solve at O(1e-3) or more, so the
    comparison exercises both index quirks."""
    for rec in DATA["lu_dense"]:
        J = np.array(rec["jacobian"]).reshape(13, 13)
        t = _target(rec["moments"])
        lm, md = o39.lu_update(J, t, rec["lm_in"])
        assert lm.tolist() == rec["lm_out"]
        assert md == rec["max_diff"]
        clean = np.array(rec["lm_in"]) - np.linalg.solve(J, J[0] - np.array(t))
        assert np.max(np.abs(clean - np.array(rec["lm_out"]))) > 1e-3
