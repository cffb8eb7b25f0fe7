"""The ctypes wrapper refuses arrays shorter than what the library reads or
writes through their pointers (a host overrun otherwise), before any library
call, and passes every call whose level or box it does not know straight to
the library, which reports those with its own error codes.  Run against a
stand-in for the library: no GPU needed."""
import numpy as np
import pytest


class _FakeLib:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def fn(*args):
            self.calls.append(name)
            return 0

        return fn


@pytest.fixture
def ctx(pkg):
    cap = pkg.capi
    c = cap.Context.__new__(cap.Context)
    c.lib, c.h, c._boxes = _FakeLib(), object(), {}
    c.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [[0, 0, 0, 7, 5, 3]], ngrow=1)
    c.level_register(1, cap.ELBM_D3Q39, cap.ELBM_STORE_FP64, [[0, 0, 0, 4, 3, 2], [5, 0, 0, 9, 3, 2]])
    yield c
    c.h = None


def _called(c, name):
    return c.lib.calls.count(name)


def test_d3q27_sizes(ctx):
    fab = (10, 8, 6)  # 8 x 6 x 4 nodes with one ghost layer: (nz, ny, nx) = (6, 8, 10)
    ctx.upload(0, 0, np.zeros((27,) + fab[::-1]))
    assert _called(ctx, "elbm_upload_level") == 1
    with pytest.raises(ValueError):
        ctx.upload(0, 0, np.zeros((27, 4, 6, 8)))  # the valid region only: the ghost layer is missing
    assert _called(ctx, "elbm_upload_level") == 1
    ctx.set_links(0, 0, np.zeros((27, 4, 6, 8), np.int32))  # state without ghosts
    with pytest.raises(ValueError):
        ctx.set_links(0, 0, np.zeros((27, 4, 6, 8), np.int32), ngrow_state=1)
    assert _called(ctx, "elbm_set_links") == 1
    out = np.zeros((27,) + fab[::-1])
    assert ctx.download(0, 0, out) is out
    with pytest.raises(ValueError):
        ctx.download(0, 0, np.zeros((27, 4, 6, 8)))
    with pytest.raises(ValueError):
        ctx.download(0, 0, np.zeros((27,) + fab[::-1], np.float32))
    assert _called(ctx, "elbm_download_level") == 1


def test_unknown_level_or_box_goes_to_the_library(ctx):
    ctx.upload(0, 5, np.zeros(3))
    ctx.upload(7, 0, np.zeros(3))
    ctx.set_links(0, 9, np.zeros(3, np.int32))
    assert _called(ctx, "elbm_upload_level") == 2 and _called(ctx, "elbm_set_links") == 1


def test_d3q39_sizes(ctx, pkg):
    bc = pkg.capi.D3Q39Bc()
    shp = (3, 4, 5)  # each box of level 1: 5 x 4 x 3 nodes, no ghosts
    f = np.zeros((39,) + shp)
    ctx.upload39(1, 1, f, f, np.zeros((13,) + shp), np.zeros(shp))
    assert _called(ctx, "elbm_upload_level39") == 1
    with pytest.raises(ValueError):
        ctx.upload39(1, 1, f, f, np.zeros((12,) + shp), np.zeros(shp))
    with pytest.raises(ValueError):
        ctx.upload39(1, 0, np.zeros((27,) + shp), f, np.zeros((13,) + shp), np.zeros(shp))
    assert _called(ctx, "elbm_upload_level39") == 1
    ctx.init_level39(1, 0, np.zeros((5,) + shp), np.zeros(13))
    with pytest.raises(ValueError):
        ctx.init_level39(1, 0, np.zeros((4,) + shp), np.zeros(13))
    with pytest.raises(ValueError):
        ctx.init_level39(1, 0, np.zeros((5,) + shp), np.zeros(12))
    assert _called(ctx, "elbm_init_level39") == 1
    ctx.upload_macro39(1, 1, np.zeros((5,) + shp))
    with pytest.raises(ValueError):
        ctx.upload_macro39(1, 1, np.zeros((5, 2, 4, 5)))
    assert _called(ctx, "elbm_upload_macro39") == 1
    ctx.set_links39(1, 0, np.zeros((39,) + shp, np.int32), bc)
    with pytest.raises(ValueError):
        ctx.set_links39(1, 0, np.zeros((39,) + shp, np.int32), bc, ngrow_state=1)
    assert _called(ctx, "elbm_set_links39") == 1


def test_network_weights(ctx, pkg):
    cap = pkg.capi
    w = cap.mlp_init_weights(0)
    assert w.size == cap.MLP_PARAMS
    ctx.set_alpha_mlp(0, w)
    with pytest.raises(ValueError):
        ctx.set_alpha_mlp(0, w[:-1])
    with pytest.raises(ValueError):
        ctx.alpha_mlp_infer(w[:100], np.zeros((4, 27), np.float32))
    assert _called(ctx, "elbm_set_alpha_mlp") == 1 and _called(ctx, "elbm_alpha_mlp_infer") == 0
