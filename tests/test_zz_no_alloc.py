"""The allocation-free upload (elbm_upload_level_noalloc) must put exactly the
same FP32 deviation populations on the device as elbm_upload_level.  It exists
for callers that cannot let the library allocate device memory after set-up
(an AMReX arena that already reserved the GPU, or a time loop that must not
stall on cudaMalloc); it stages through a fixed 32 MiB buffer compiled into
the library instead.  Collected last so that a failure here stops a -x run
only after every other test has run."""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAGE_BYTES = 32 << 20


def _noalloc_fn(lib):
    fn = lib.elbm_upload_level_noalloc
    fn.restype = ct.c_int
    fn.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p]
    return fn


def _level(cap, geo, nx, ny, nz, g):
    ctx = cap.Context(0)
    ctx.level_register(0, cap.ELBM_D3Q27, cap.ELBM_STORE_FP32_DEV, [[2, 3, 4, 2 + nx - 1, 3 + ny - 1, 4 + nz - 1]],
                       ngrow=g)
    bp = geo.d3q27_boundary_params((0.05, 0.0, 0.0), 1e-3)
    ctx.set_d3q27_params(0, cap.make_d3q27_params(**bp))
    ctx.set_links(0, 0, geo.box_state27(nx, ny, nz, geo.flat_plate_faces()))
    return ctx


def _fab(geo, nx, ny, nz, g, seed):
    f = geo.perturbed_equilibrium(nx + 2 * g, ny + 2 * g, nz + 2 * g, (0.05, 0.0, 0.0), 1e-3, seed=seed)
    return np.ascontiguousarray(f)


def _free_device_bytes():
    """cudaMemGetInfo's free bytes of the current device (the CUDA runtime the library uses)."""
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            rt = ct.CDLL(name)
            break
        except OSError:
            continue
    else:
        pytest.skip("no CUDA runtime library to query free memory")
    free, total = ct.c_size_t(0), ct.c_size_t(0)
    assert rt.cudaMemGetInfo(ct.byref(free), ct.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("g", [1, 0])
def test_noalloc_upload_matches_upload(pkg, built_lib, g):
    cap, geo = pkg.capi, pkg.geometry
    nx, ny, nz = 24, 16, 12
    ref = _level(cap, geo, nx, ny, nz, g)
    new = _level(cap, geo, nx, ny, nz, g)
    upload_noalloc = _noalloc_fn(new.lib)
    for call, seed in enumerate((7, 8)):  # two calls in a row: the shared buffer is reused
        fab = _fab(geo, nx, ny, nz, g, seed)
        ref.upload(0, 0, fab)
        rc = upload_noalloc(new.h, 0, 0, fab.ctypes.data_as(ct.c_void_p))
        assert rc == cap.ELBM_OK, new.lib.elbm_last_error_string(new.h).decode()
        a = ref.download(0, 0)
        b = new.download(0, 0)
        assert np.array_equal(a, b), f"call {call}: max diff {np.max(np.abs(a - b))}"
        # both states advance identically
        ref.step(0, 3, want_stats=False)
        new.step(0, 3, want_stats=False)
        assert np.array_equal(ref.download(0, 0), new.download(0, 0))
    ref.close()
    new.close()


def test_noalloc_upload_rejects_oversized_box(pkg, built_lib):
    cap, geo = pkg.capi, pkg.geometry
    n = 60  # 60^3 nodes x 27 x 8 bytes = 46.7 MB > 32 MiB of staging
    assert n ** 3 * 27 * 8 > STAGE_BYTES
    ctx = _level(cap, geo, n, n, n, 0)
    fab = np.ones((27, n, n, n))
    rc = _noalloc_fn(ctx.lib)(ctx.h, 0, 0, fab.ctypes.data_as(ct.c_void_p))
    assert rc == cap.ELBM_E_ARG
    assert "at most" in ctx.lib.elbm_last_error_string(ctx.h).decode()
    ctx.close()


def test_noalloc_upload_allocates_nothing(pkg, built_lib):
    """The property the entry point exists for: once the context is created and
    the level set up, uploads through it leave the device's free memory as it
    was, while the ordinary upload's first call allocates its staging buffer
    (which shows that the measurement sees an allocation of this size)."""
    cap, geo = pkg.capi, pkg.geometry
    nx, ny, nz = 64, 64, 32  # 131,072 nodes: 28.3 MB of FP64 staging, inside the 32 MiB buffer
    new = _level(cap, geo, nx, ny, nz, 0)
    upload_noalloc = _noalloc_fn(new.lib)
    fab = _fab(geo, nx, ny, nz, 0, 11)
    free0 = _free_device_bytes()
    for _ in range(3):
        rc = upload_noalloc(new.h, 0, 0, fab.ctypes.data_as(ct.c_void_p))
        assert rc == cap.ELBM_OK, new.lib.elbm_last_error_string(new.h).decode()
    assert _free_device_bytes() == free0
    ref = _level(cap, geo, nx, ny, nz, 0)
    free1 = _free_device_bytes()
    ref.upload(0, 0, fab)
    assert free1 - _free_device_bytes() >= nx * ny * nz * 27 * 8
    assert np.array_equal(ref.download(0, 0), new.download(0, 0))
    ref.close()
    new.close()
