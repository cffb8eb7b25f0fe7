"""D3Q39 codes from a triangulated surface (elbm_mark_triangles39, host):
the double-ramp wedge as a closed 8-triangle prism gives the same solid
nodes, the same wall links and, within the last digit of the packed fraction,
the same codes as the analytic wedge of d3q39_setup.wedge_state39 on the
shifted lattice; the box-face codes it does not touch stay as they were."""
import numpy as np
import pytest


@pytest.mark.parametrize("angle", [10.0, 20.0])
def test_mark_triangles39_matches_analytic_wedge(pkg, angle):
    s39, cap = pkg.d3q39_setup, pkg.capi
    nx, ny, nz = 64, 6, 24
    x0, xa, x1 = 16.3, 36.7, 57.1  # no node on a ramp plane
    ref = s39.wedge_state39(nx, ny, nz, x0, x1, angle, s39.WEDGE_FACES, periodic=0, priority=s39.WEDGE_PRIORITY,
                            x_apex=xa)
    st = s39.box_state39(nx, ny, nz, s39.WEDGE_FACES, 1, 1, periodic=0, priority=s39.WEDGE_PRIORITY)
    cap.mark_triangles39(st, (0.0, 0.0, 0.0), 1.0, s39.wedge_triangles(x0, xa, x1, angle, ny), shifted=1,
                         primary_flow_dir=1, periodic=0)
    assert (ref[0] == -1001).sum() > 100
    assert np.array_equal(st[0], ref[0])
    wall_ref = (ref <= -1001) & (ref >= -1100000000)
    wall = (st <= -1001) & (st >= -1100000000)
    assert np.array_equal(wall, wall_ref)
    assert np.max(np.abs(st[wall].astype(np.int64) - ref[wall].astype(np.int64))) <= 2
    assert np.array_equal(st[~wall], ref[~wall])
