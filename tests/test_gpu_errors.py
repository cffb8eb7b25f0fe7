"""Error paths on a GPU: calls out of order, unknown levels and boxes, unsupported codes and
bad sizes come back as ELBM_E_* codes with a message, and the context stays usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_error_codes_and_recovery(pkg, built_lib, tmp_path):
    geo, cap, s39 = pkg.geometry, pkg.capi, pkg.d3q39_setup
    ctx = cap.Context(0)

    def code(fn, *a):
        with pytest.raises(cap.ElbmError) as e:
            fn(*a)
        assert ctx.lib.elbm_last_error_string(ctx.h)  # a message is kept
        return e.value.rc

    # unknown level, step before registration / parameters / upload
    assert code(ctx.step, 3, 1) == cap.ELBM_E_ARG
    ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [[0, 0, 0, 15, 7, 7]])
    assert code(ctx.step, 0, 1) == cap.ELBM_E_STATE
    bp = geo.d3q27_boundary_params((0.05, 0.0, 0.0), 1e-3)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    assert code(ctx.step, 0, 1) == cap.ELBM_E_STATE
    # an unknown box, a link code outside the supported set
    st = geo.box_state27(16, 8, 8, geo.flat_plate_faces())
    assert code(ctx.set_links, 0, 5, st) == cap.ELBM_E_ARG
    bad = st.copy()
    bad[3, 2, 2, 2] = -77
    assert code(ctx.set_links, 0, 0, bad) == cap.ELBM_E_UNSUPPORTED
    # the context recovers: the same level runs once its inputs are right
    ctx.set_links(0, 0, st)
    ctx.upload(0, 0, geo.perturbed_equilibrium(16, 8, 8, (0.05, 0.0, 0.0), 1e-3, seed=1))
    s = ctx.step(0, 2)
    assert s["node_updates"] == 2 * 16 * 8 * 8
    # D3Q39: a level that is not periodic everywhere needs its link codes; GGM wants D3Q39 fields
    c = s39.wedge_case_consts()
    ctx.level_register(1, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, 7, 5, 4]])
    ctx.set_d3q39_params(1, cap.make_d3q39_params(c, timestep=0, periodic=2, damp=0))
    shape = (5, 6, 8)
    lm0 = s39.freestream_start_lm(c)
    macro = np.stack([np.full(shape, 1.0), np.full(shape, c.mach), np.zeros(shape), np.zeros(shape),
                      np.full(shape, c.temperature)])
    assert ctx.init_level39(1, 0, macro, lm0) == 0
    assert code(ctx.step, 1, 1) == cap.ELBM_E_STATE
    assert code(ctx.ggm_tags, 0, 0, 1, 0, 1.0) == cap.ELBM_E_UNSUPPORTED
    assert code(ctx.ggm_tags, 1, 0, 9, 0, 1.0) == cap.ELBM_E_ARG
    # a checkpoint of another layout is refused
    ctx.checkpoint_write(0, tmp_path / "l0.ckp")
    assert code(ctx.checkpoint_read, 1, tmp_path / "l0.ckp") == cap.ELBM_E_ARG
    assert code(ctx.checkpoint_read, 0, tmp_path / "missing.ckp") == cap.ELBM_E_ARG
    ctx.close()
