"""Seeded inputs of the predictive-splitting case (GGM/PGS/predictive_splitter.f95),
shared by the golden generator and the test: a 12 x 10 x 8 box of ggm values, velocities
with a dominant component (x, y or z) at three quarters of the nodes, 10% solid nodes,
sensitivity 0.2 and a scan of at most 4 nodes.  The legacy RandomState stream is frozen
across numpy versions."""
import numpy as np

NX, NY, NZ = 12, 10, 8
SENSITIVITY, MAX_SCAN = 0.2, 4


def case():
    """ggm, u, v, w, node types s0 (each (nz, ny, nx))."""
    rs = np.random.RandomState(77)
    shape = (NZ, NY, NX)
    ggm = rs.uniform(0, 1, shape) ** 4
    u, v, w = (rs.uniform(-1, 1, shape) for _ in range(3))
    dom = rs.randint(0, 4, shape)
    u[dom == 0] *= 20
    v[dom == 1] *= 20
    w[dom == 2] *= 20
    s0 = np.where(rs.uniform(0, 1, shape) < 0.1, -1001, 0)
    return ggm, u, v, w, s0


def ggm_case(scheme: int):
    """rho (the tagged variable), u, v, w, the 39 link codes (10% of the links boundary
    codes, 10% of the nodes solid or null) and the freestream rho of the gradient case."""
    rs = np.random.RandomState(300 + scheme)
    shape = (NZ, NY, NX)
    rho = 1.0 + 0.05 * rs.uniform(-1, 1, shape) + 0.2 * (rs.uniform(0, 1, shape) < 0.05)
    u, v, w = (rs.uniform(-1, 1, shape) for _ in range(3))
    state = np.where(rs.uniform(0, 1, (39,) + shape) < 0.1, -10, 0).astype(np.int32)
    node = rs.uniform(0, 1, shape)
    state[0] = np.where(node < 0.05, -1001, np.where(node < 0.1, -666, 0))
    return rho, u, v, w, state, 1.0
