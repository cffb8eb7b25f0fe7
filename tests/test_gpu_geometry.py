"""Wall links from a triangulated surface on the device: elbm_mark_triangles_gpu
gives the same state codes as the host elbm_mark_triangles (bit for bit) for the
benchmark's icosphere and a coarser one off the lattice; and the time of both
on the 256x128x128 sphere box."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,sub,radius,center", [((64, 48, 40), 3, 9.3, (30.2, 23.7, 19.1)),
                                                     ((256, 128, 128), 4, 16.0, (64.0, 64.0, 64.0))])
def test_device_marking_matches_host(pkg, built_lib, shape, sub, radius, center):
    geo, cap = pkg.geometry, pkg.capi
    nx, ny, nz = shape
    tri = geo.icosphere(sub, radius, center)
    host = geo.box_state27(nx, ny, nz, geo.sphere_faces())
    dev = host.copy()
    t0 = time.perf_counter()
    cap.mark_triangles(host, (0.0, 0.0, 0.0), 1.0, tri)
    t_host = time.perf_counter() - t0
    ctx = cap.Context(0)
    ctx.mark_triangles(dev.copy(), (0.0, 0.0, 0.0), 1.0, tri)  # warm-up
    t0 = time.perf_counter()
    ctx.mark_triangles(dev, (0.0, 0.0, 0.0), 1.0, tri)
    t_dev = time.perf_counter() - t0
    ctx.close()
    assert (host == -1001).any() and (host < -1001).any()
    assert np.array_equal(dev, host)
    print(f"marking {shape}: host {t_host:.3f} s, device {t_dev:.3f} s")
