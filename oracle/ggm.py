"""TEST INFRASTRUCTURE ONLY: numpy restatement of the reference's GGM
refinement tagging on one box (the checker of elbm_ggm_tags).

  GGM/derivatives/calculate_grad_mag.f95      gm = |grad q| (nodes with state < 0 and != -666: 0)
  GGM/derivatives/calculate_gradgrad_mag.f95  ggm = |grad gm| (state < 0: 0), tag where ggm >= limit
  GGM/populate_q.f95, complicated_properties/calculate_v_mag.f95   the variables
  derivatives/modules/derivatives.f95:644-760 derivative_windage_secondord / _firstord

Per axis the points q(0), q(+1), q(+2), q(-1), q(-2) are used according to the
node's state components (1-based) 2, 16, 5, 19 (x), 3, 17, 6, 20 (y), 4, 18,
7, 21 (z) being >= 0; points outside the box on a non-periodic axis hold the
freestream value of q, and gm = 0 there.  Loops in the reference's statement
order, scalar FP64 (no fused multiply-adds), small boxes only."""
import math

import numpy as np

COMPS = [(1, 15, 4, 18), (2, 16, 5, 19), (3, 17, 6, 20)]  # 0-based state components per axis


def variable(var, rho, u, v, w, T):
    if var == 1:
        return rho
    if var == 2:
        return u
    if var == 3:
        return v
    if var == 4:
        return w
    if var == 5:
        return rho * (T + (u * u + v * v + w * w) / 2.0)
    if var == 6:
        return T
    if var == 7:
        return math.sqrt(u * u + v * v + w * w)
    return 0.5 * rho * math.sqrt(u * u + v * v + w * w)


def windage2(q, s, wind, scheme):
    p1, p2, m1, m2 = s
    if scheme == 0:
        if p1 and m1:
            return (q[3] - q[1]) / 2.0
        if p1:
            return q[1] - q[0]
        if m1:
            return q[0] - q[3]
        return 0.0
    pos = wind > 0.0 if scheme == 1 else wind < 0.0
    if pos:
        if m1 and m2:
            return (3 * q[0] - 4 * q[3] + q[4]) / 2
        return q[3] - q[0] if m1 else 0.0
    if p1 and p2:
        return (-3 * q[0] + 4 * q[3] - q[4]) / 2
    return q[0] - q[1] if p1 else 0.0


def ggm_tags(macro, state, periodic, var, scheme, limit, fs):
    """macro (5, nz, ny, nx): rho, u, v, w, T; state (39, nz, ny, nx) int32 (None: every link interior,
    node type 0); fs: freestream (rho, u, v, w, T).  Returns tags (uint8), ggm, gm."""
    _, nz, ny, nx = macro.shape
    dims = (nx, ny, nz)

    def node(x, y, z):
        p = [x, y, z]
        for a in range(3):
            if periodic & (1 << a):
                p[a] %= dims[a]
            elif not 0 <= p[a] < dims[a]:
                return None
        return p[2], p[1], p[0]

    def s0(z, y, x):
        return 0 if state is None else int(state[0, z, y, x])

    def links(z, y, x, ax):
        if state is None:
            return (True, True, True, True)
        return tuple(int(state[c, z, y, x]) >= 0 for c in COMPS[ax])

    qf = variable(var, *fs)
    q = np.zeros((nz, ny, nx))
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                q[z, y, x] = variable(var, *macro[:, z, y, x])

    def grad(field, outside, z, y, x):
        total = 0.0
        for ax in range(3):
            d = [0, 0, 0]
            d[ax] = 1
            pts = []
            for k in (0, 1, 2, -1, -2):
                m = node(x + k * d[0], y + k * d[1], z + k * d[2])
                pts.append(outside if m is None else field[m])
            dq = windage2(pts, links(z, y, x, ax), macro[1 + ax, z, y, x], scheme)
            total = dq * dq if ax == 0 else total + dq * dq
        return math.sqrt(total)

    gm = np.zeros((nz, ny, nx))
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                t = s0(z, y, x)
                gm[z, y, x] = 0.0 if (t < 0 and t != -666) else grad(q, qf, z, y, x)
    ggm = np.zeros((nz, ny, nx))
    tags = np.zeros((nz, ny, nx), np.uint8)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                if s0(z, y, x) < 0:
                    continue
                ggm[z, y, x] = grad(gm, 0.0, z, y, x)
                tags[z, y, x] = 1 if ggm[z, y, x] >= limit else 0
    return tags, ggm, gm


def pgs_tags(tags, ggm, macro, state, sensitivity, reach):
    """Predictive splitting (GGM/PGS/predictive_splitter.f95:36-316) added to tags (in place),
    the scans kept inside the box.  state (39, nz, ny, nx) or None (node type 0 everywhere)."""
    _, nz, ny, nx = macro.shape
    dims = (nx, ny, nz)
    s0 = np.zeros((nz, ny, nx), np.int64) if state is None else state[0].astype(np.int64)
    limit, upper = 2 * sensitivity, 3 * sensitivity

    def at(p):
        return p[2], p[1], p[0]

    def eligible(p):
        return 0 <= s0[at(p)] < 100000

    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                if s0[z, y, x] < 0:
                    continue
                u, v, w = macro[1:4, z, y, x]
                p = [x, y, z]
                lo = [p[a] - reach if p[a] > reach else 0 for a in range(3)]
                hi = [p[a] + reach if dims[a] - 1 - p[a] > reach else dims[a] - 1 for a in range(3)]
                if abs(u) > 5 * abs(v) and abs(u) > 5 * abs(w):
                    ax, vel = 0, u
                elif abs(v) > 5 * abs(u) and abs(v) > 5 * abs(w):
                    ax, vel = 1, v
                elif abs(w) > 5 * abs(v) and abs(w) > 5 * abs(u):
                    ax, vel = 2, w
                else:
                    ax = None
                if ax is not None:
                    def pt(q):
                        r = list(p)
                        r[ax] = q
                        return r
                    scan = range(lo[ax], p[ax] + 1) if vel > 0.0 else range(p[ax], hi[ax] + 1)
                    hit = next((q for q in scan if eligible(pt(q)) and ggm[at(pt(q))] >= limit), None)
                    if hit is not None:
                        a, b = (hit, p[ax]) if vel > 0.0 else (p[ax], hit)
                        for q in range(a, b + 1):
                            if s0[at(pt(q))] >= 0:
                                tags[at(pt(q))] = 1
                    continue
                for b in range(3):
                    for q in range(lo[b], hi[b] + 1):
                        r = list(p)
                        r[b] = q
                        if eligible(r) and ggm[at(r)] >= upper:
                            tags[at(r)] = 1
    return tags
