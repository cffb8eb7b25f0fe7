"""A D3Q27 level made of several boxes of uneven sizes (one launch per step,
links that cross box faces read the neighbouring box in place) must step
exactly like the same domain held as one box.  Each box gets its slice of the
level's state with one ghost layer, as AMReX's fill_boundary would give it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# uneven boxes tiling a 40 x 24 x 24 domain (x, y, z inclusive ranges)
BOXES = [((0, 0, 0), (16, 23, 23)), ((17, 0, 0), (28, 11, 23)), ((17, 12, 0), (28, 23, 23)),
         ((29, 0, 0), (39, 23, 9)), ((29, 0, 10), (39, 23, 23))]


def _slice_state(st, lo, hi, g=1):
    """The box's state FAB with g ghost layers; outside the domain: not fluid (-1)."""
    q, nz, ny, nx = st.shape
    out = np.full((q, hi[2] - lo[2] + 1 + 2 * g, hi[1] - lo[1] + 1 + 2 * g, hi[0] - lo[0] + 1 + 2 * g), -1, np.int32)
    for z in range(out.shape[1]):
        gz = lo[2] - g + z
        if not 0 <= gz < nz:
            continue
        for y in range(out.shape[2]):
            gy = lo[1] - g + y
            if not 0 <= gy < ny:
                continue
            x0, x1 = max(lo[0] - g, 0), min(hi[0] + g, nx - 1)
            out[:, z, y, x0 - (lo[0] - g):x1 - (lo[0] - g) + 1] = st[:, gz, gy, x0:x1 + 1]
    return out


def _box_view(f, lo, hi):
    return f[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]


def _run(pkg, st, f0, bp, storage, boxes, steps):
    cap = pkg.capi
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, storage, [list(lo) + list(hi) for lo, hi in boxes])
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    for k, (lo, hi) in enumerate(boxes):
        ctx.set_links(0, k, _slice_state(st, lo, hi), ngrow_state=1)
        ctx.upload(0, k, np.ascontiguousarray(_box_view(f0, lo, hi)))
    s = ctx.step(0, steps)
    out = np.zeros_like(f0)
    for k, (lo, hi) in enumerate(boxes):
        _box_view(out, lo, hi)[...] = ctx.download(0, k)
    ctx.close()
    return s, out


def _sphere(pkg):
    geo, cap, lat = pkg.geometry, pkg.capi, pkg.lattice
    st = geo.box_state27(40, 24, 24, geo.sphere_faces())
    cap.mark_triangles(st, (0.0, 0.0, 0.0), 1.0, geo.icosphere(3, 6.5, (16.3, 11.6, 12.2)))
    f0 = geo.perturbed_equilibrium(40, 24, 24, (0.08, 0.0, 0.0), 1e-3, seed=4321)
    f0[:, st[0] == -1001] = lat.W[:, None]
    return st, f0, geo.d3q27_boundary_params((0.08, 0.0, 0.0), 5e-4)


def _plate(pkg):
    geo = pkg.geometry
    st = geo.box_state27(40, 24, 24, geo.flat_plate_faces())
    f0 = geo.perturbed_equilibrium(40, 24, 24, (0.06, 0.0, 0.0), 5e-3, seed=4322)
    return st, f0, geo.d3q27_boundary_params((0.06, 0.0, 0.0), 2e-5)


@pytest.mark.parametrize("case,storage", [("sphere", 0), ("sphere", 1), ("plate", 0), ("plate", 1)])
def test_multibox_level_matches_single_box(pkg, built_lib, case, storage):
    st, f0, bp = (_sphere if case == "sphere" else _plate)(pkg)
    one = [((0, 0, 0), (39, 23, 23))]
    s1, f1 = _run(pkg, st, f0, bp, storage, one, 40)
    s5, f5 = _run(pkg, st, f0, bp, storage, BOXES, 40)
    assert s1["node_updates"] == s5["node_updates"]
    assert s1["fallbacks"] == s5["fallbacks"] == 0
    fluid = st[0] != -1001
    assert np.array_equal(f1[:, fluid], f5[:, fluid])


def test_multibox_rejects_overlap_and_gaps(pkg, built_lib):
    cap = pkg.capi
    ctx = cap.Context(0)
    with pytest.raises(cap.ElbmError):
        ctx.level_register(0, cap.ELBM_D3Q27, 0, [[0, 0, 0, 9, 9, 9], [5, 0, 0, 14, 9, 9]])
    # a fluid link that leaves every box of the level (a gap between boxes) is refused
    st, f0, bp = _plate(pkg)
    ctx.level_register(1, cap.ELBM_D3Q27, 0, [[0, 0, 0, 15, 23, 23], [17, 0, 0, 39, 23, 23]])
    ctx.set_d3q27_params(1, cap.make_d3q27_params(**bp))
    with pytest.raises(cap.ElbmError):
        ctx.set_links(1, 0, _slice_state(st, (0, 0, 0), (15, 23, 23)), ngrow_state=1)
    ctx.close()


# boxes whose widths are whole 16-byte rows (nx % 4 == 0), so that the tensor-copy
# variant serves them: 32-, 64- and 128-node-wide tiles in one launch
BOXES4 = [((0, 0, 0), (19, 23, 23)), ((20, 0, 0), (27, 11, 23)), ((20, 12, 0), (27, 23, 23)),
          ((28, 0, 0), (39, 23, 9)), ((28, 0, 10), (39, 23, 23))]


@pytest.mark.parametrize("case", ["plate", "sphere"])
def test_multibox_tensor_copy_variant(pkg, built_lib, case):
    """The tensor-copy step variant (8) over a level of uneven boxes agrees
    with the same domain held as one box and stepped by the direct kernel to
    FP32 rounding, and with itself on one box bit for bit (its bulk nodes read
    their pulls from the copied tiles, boundary and cross-box links from their
    words)."""
    cap = pkg.capi
    if case == "sphere":
        st, f0, bp = _sphere(pkg)
    else:
        geo = pkg.geometry
        st = geo.box_state27(40, 24, 24, geo.flat_plate_faces())
        f0 = geo.perturbed_equilibrium(40, 24, 24, (0.05, 0.0, 0.0), 2e-3, seed=99)
        bp = geo.d3q27_boundary_params((0.05, 0.0, 0.0), 1e-3)

    def run(boxes, variant):
        ctx = cap.Context(0)
        ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [list(lo) + list(hi) for lo, hi in boxes])
        ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
        for k, (lo, hi) in enumerate(boxes):
            ctx.set_links(0, k, _slice_state(st, lo, hi), ngrow_state=1)
            ctx.upload(0, k, np.ascontiguousarray(_box_view(f0, lo, hi)))
        ctx.set_kernel_variant(0, variant)
        s = ctx.step(0, 20)
        out = np.zeros_like(f0)
        for k, (lo, hi) in enumerate(boxes):
            _box_view(out, lo, hi)[...] = ctx.download(0, k)
        ctx.close()
        return s, out

    one = [((0, 0, 0), (39, 23, 23))]
    s_multi, f_multi = run(BOXES4, 8)
    s_one8, f_one8 = run(one, 8)
    s_one0, f_one0 = run(one, 0)
    assert s_multi["status"] & 0x10 == 0 and s_one8["status"] & 0x10 == 0
    assert s_multi["node_updates"] == s_one8["node_updates"] == s_one0["node_updates"]
    assert np.array_equal(f_multi, f_one8)
    assert np.max(np.abs(f_one8 - f_one0)) <= 1e-6
