"""Solid marking and wall-link fractions of a triangulated sphere: the library's
accelerated set-up code (elbm_mark_triangles) must match the oracle's
every-triangle search bit for bit, in the reference's packed encoding."""
import numpy as np
import pytest


def test_icosphere_counts(pkg):
    tri = pkg.geometry.icosphere(4, 16.0, (64.0, 64.0, 64.0))
    assert tri.shape == (5120, 3, 3)
    r = np.linalg.norm(tri.reshape(-1, 3) - 64.0, axis=1)
    assert np.allclose(r, 16.0)
    # outward orientation: normals point away from the centre
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    c = tri.mean(axis=1) - 64.0
    assert (np.einsum("ij,ij->i", n, c) > 0).all()


@pytest.mark.parametrize("sub,radius,center", [(2, 5.3, (14.3, 12.1, 11.7)), (3, 6.0, (16.0, 12.0, 12.0)),
                                               (4, 7.5, (15.5, 11.25, 12.0)), (3, 6.0, (12.0, 12.0, 12.0))])
def test_marking_matches_bruteforce(pkg, orc, built_lib, sub, radius, center):
    geo = pkg.geometry
    tri = geo.icosphere(sub, radius, center)
    a = geo.box_state27(32, 24, 24, geo.sphere_faces())
    b = a.copy()
    pkg.capi.mark_triangles(a, (0.0, 0.0, 0.0), 1.0, tri)
    orc.mark_triangles(b, (0.0, 0.0, 0.0), 1.0, tri)
    assert np.array_equal(a, b)
    solid = a[0] == -1001
    # the marked solid volume approximates the sphere's
    assert abs(solid.sum() - 4 / 3 * np.pi * radius ** 3) < 0.12 * 4 / 3 * np.pi * radius ** 3
    # no solid node outside the sphere (rays through the icosphere's vertices on
    # lattice lines must not flip the inside test)
    zs, ys, xs = np.nonzero(solid)
    assert np.sqrt((xs - center[0]) ** 2 + (ys - center[1]) ** 2 + (zs - center[2]) ** 2).max() <= radius + 1e-9
    # wall links join fluid nodes to solid nodes only
    zf, yf, xf = np.nonzero(~solid)
    for i in range(1, 27):
        wl = a[i][~solid] < -1001
        xt, yt, zt = xf + pkg.lattice.CX[i], yf + pkg.lattice.CY[i], zf + pkg.lattice.CZ[i]
        inside = (xt >= 0) & (xt < 32) & (yt >= 0) & (yt < 24) & (zt >= 0) & (zt < 24)
        assert not (wl & inside & ~solid[np.clip(zt, 0, 23), np.clip(yt, 0, 23), np.clip(xt, 0, 31)]).any()
    q = np.abs(a[a < -1001].astype(np.float64) + 1001) / 1e9
    assert q.size > 0 and q.min() > 0 and q.max() <= 1.0
    # every wall link of a fluid node points at a solid node or across the surface
    z, y, x = np.nonzero(~solid)
    for i in range(1, 27):
        wl = a[i][~solid] < -1001
        tgt_solid = solid[np.clip(z + pkg.lattice.CZ[i], 0, 23), np.clip(y + pkg.lattice.CY[i], 0, 23),
                          np.clip(x + pkg.lattice.CX[i], 0, 31)]
        assert (tgt_solid <= wl).all()  # links into the solid are wall links
