"""A D3Q39 level made of several boxes steps exactly like the same domain held
as one box: the shifted Mach 1.5 wedge (inlet, outlet, bounce-back floor,
freestream top, inviscid side walls, the double ramp's interpolated wall
links) on a 96 x 12 x 48 domain split into five boxes of uneven sizes, the
initial state solved per box, 20 steps with the negative-population repair;
f, g, the multipliers, w, alpha and the fields of every box bit for bit equal
to the one-box run, and so are the GGM tags of each box.  Each box gets its
slice of the level's state with one ghost layer, as AMReX's fill_boundary
would give it; links, wall targets and the repair that reach into a
neighbouring box read it in place."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, NZ = 96, 12, 48
BOXES = [((0, 0, 0), (39, 11, 19)), ((40, 0, 0), (95, 11, 19)), ((0, 0, 20), (39, 5, 47)), ((0, 6, 20), (39, 11, 47)),
         ((40, 0, 20), (95, 11, 47))]


def _slice(st, lo, hi, g=1):
    q, nz, ny, nx = st.shape
    out = np.full((q, hi[2] - lo[2] + 1 + 2 * g, hi[1] - lo[1] + 1 + 2 * g, hi[0] - lo[0] + 1 + 2 * g), -1, np.int32)
    src = [slice(max(lo[a] - g, 0), min(hi[a] + g, n - 1) + 1) for a, n in enumerate((nx, ny, nz))]
    dst = [slice(sl.start - (lo[a] - g), sl.stop - (lo[a] - g)) for a, sl in enumerate(src)]
    out[:, dst[2], dst[1], dst[0]] = st[:, src[2], src[1], src[0]]
    return out


def _run(pkg, boxes, steps):
    from oracle import oracle39 as o39

    s39, cap = pkg.d3q39_setup, pkg.capi
    c = s39.wedge_case_consts(nu_lattice=2e-4)
    k = o39.consts(c)
    lm0 = s39.freestream_start_lm(c)
    _, f, g, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    st = s39.wedge_case_state(NX, NY, NZ)
    bc = cap.make_d3q39_bc([1] * 8, [6] + [1] * 7, f, g, [f] * 8, [g] * 8, [f] * 8, [g] * 8,
                           (c.mach, 0.0, 0.0, c.temperature))
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [list(lo) + list(hi) for lo, hi in boxes])
    ctx.set_d3q39_params(0, cap.make_d3q39_params(c, timestep=0, periodic=0, damp=1))
    rng = np.random.default_rng(5)
    macro = np.stack([1.0 + 0.01 * rng.uniform(-1, 1, (NZ, NY, NX)), np.full((NZ, NY, NX), c.mach),
                      np.zeros((NZ, NY, NX)), np.zeros((NZ, NY, NX)), np.full((NZ, NY, NX), c.temperature)])
    for b, (lo, hi) in enumerate(boxes):
        ctx.set_links39(0, b, _slice(st, lo, hi), bc, ngrow_state=1)
    for b, (lo, hi) in enumerate(boxes):
        ctx.init_level39(0, b, np.ascontiguousarray(macro[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]), lm0)
    s = ctx.step(0, steps)
    out = {}
    tags = np.zeros((NZ, NY, NX), np.uint8)
    for b, (lo, hi) in enumerate(boxes):
        d = ctx.download39(0, b)
        for name, v in d.items():
            if name not in out:
                out[name] = np.zeros(v.shape[:-3] + (NZ, NY, NX))
            out[name][..., lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = v
        tags[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = ctx.ggm_tags(0, b, 1, 0, 1e-3)[0]
    ctx.close()
    return s, out, tags, st


def test_multibox_d3q39_matches_single_box(pkg, built_lib):
    one = [((0, 0, 0), (NX - 1, NY - 1, NZ - 1))]
    s1, o1, t1, st = _run(pkg, one, 20)
    s5, o5, t5, _ = _run(pkg, BOXES, 20)
    fluid = st[0] >= 0
    assert s1["node_updates"] == s5["node_updates"] == 20 * fluid.sum()
    assert s1["fallbacks"] == s5["fallbacks"] == 0 and s1["status"] & 1 == 0
    assert np.isfinite(o1["fout"][:, fluid]).all()
    for name in ("fout", "gout", "lm", "w_vel", "alpha", "macro"):
        assert np.array_equal(o1[name][..., fluid], o5[name][..., fluid]), name
    assert np.array_equal(t1, t5)
