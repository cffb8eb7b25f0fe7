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


@pytest.mark.parametrize("shifted,pfd,periodic,shape", [(1, 1, 0, "sphere"), (0, 1, 2, "sphere"), (1, 4, 5, "sphere"),
                                                        (1, 1, 0, "wedge")])
def test_mark_triangles39_device_matches_host(pkg, built_lib, shifted, pfd, periodic, shape):
    """The D3Q39 codes of a triangulated surface on the device equal the host
    marker's bit for bit: an icosphere (1,280 triangles) on the shifted lattice
    along +x and along -x and on the unshifted lattice, with periodic axes, and
    the double-ramp wedge prism at the wedge case's full size."""
    geo, s39, cap = pkg.geometry, pkg.d3q39_setup, pkg.capi
    if shape == "sphere":
        nx, ny, nz = 96, 48, 40
        tri = geo.icosphere(3, 9.5, (40.3, 23.7, 19.6))
        faces = {"x-": -101, "x+": -201, "y-": -1000, "y+": -1000, "z-": -1000, "z+": -1000}
        st = s39.box_state39(nx, ny, nz, faces, shifted, pfd, periodic=periodic)
    else:
        nx, ny, nz = 384, 48, 192
        tri = s39.wedge_triangles(96.0, 216.0, 336.0, 10.0, ny)
        st = s39.box_state39(nx, ny, nz, s39.WEDGE_FACES, 1, 1, periodic=0, priority=s39.WEDGE_PRIORITY)
    host = st.copy()
    cap.mark_triangles39(host, (0.0, 0.0, 0.0), 1.0, tri, shifted, pfd, periodic)
    ctx = cap.Context(0)
    dev = st.copy()
    ctx.mark_triangles39(dev, (0.0, 0.0, 0.0), 1.0, tri, shifted, pfd, periodic)
    ctx.close()
    assert (host[0] == -1001).sum() > 1000
    assert ((host <= -1001) & (host >= -1100000000) & (host[0] >= 0)[None]).sum() > 1000
    assert np.array_equal(host, dev)
