"""D3Q39 link codes: the pull tables the library builds (elbm_links39_tables,
host code, no GPU) must reproduce, slot by slot, the post-streaming
populations of the reference's push loop as restated by the oracle
(o39_step_links), on the unshifted and the shifted lattice, over several
steps (slots no rule writes keep the previous step's value)."""
import math

import numpy as np
import pytest

from oracle import oracle39 as o39


def _case(pkg, shifted):
    s39 = pkg.d3q39_setup
    if shifted:
        c = s39.wedge_case_consts()
    else:
        c = s39.wedge_case_consts(v_inf_ms=0.3 * math.sqrt(1.4 * 287.052874 * 288.15))
    k = o39.consts(c)
    k.shifted = shifted
    lm0 = s39.freestream_start_lm(c)
    _, ff, gf, _ = o39.init_node(k, 1.0, c.mach, 0.0, 0.0, c.temperature, lm0)
    _, fi, gi, _ = o39.init_node(k, 1.02, c.mach, 0.0, 0.0, c.temperature, lm0)
    _, fo, go, _ = o39.init_node(k, 0.98, c.mach, 0.0, 0.0, c.temperature, lm0)
    return c, k, lm0, (ff, gf, fi, gi, fo, go)


def pull39(words_kind, lev_f, lev_g, ntype, rec, words, prev_f, prev_g, eqf, eqg, cx, cy, cz, periodic):
    """Post-streaming populations from the pull tables (numpy restatement of the kernel's gather)."""
    q, nz, ny, nx = lev_f.shape
    F = np.zeros_like(lev_f)
    G = np.zeros_like(lev_g)
    z, y, x = np.nonzero(ntype == 1)
    for j in range(q):
        sx, sy, sz = (x - cx[j]) % nx, (y - cy[j]) % ny, (z - cz[j]) % nz
        F[j, z, y, x] = lev_f[j, sz, sy, sx]
        G[j, z, y, x] = lev_g[j, sz, sy, sx]
    for r, n in enumerate(rec):
        zz, yy, xx = n // (nx * ny), (n // nx) % ny, n % nx
        for j in range(q):
            w = int(words[r, j])
            kind, pop, tab, off = w & 3, (w >> 2) & 63, (w >> 8) & 31, w >> 13
            if kind == 1:
                dx, dy, dz = off % 9 - 4, (off // 9) % 9 - 4, off // 81 - 4
                sx, sy, sz = (xx + dx) % nx, (yy + dy) % ny, (zz + dz) % nz
                F[j, zz, yy, xx] = lev_f[pop, sz, sy, sx]
                G[j, zz, yy, xx] = lev_g[pop, sz, sy, sx]
            elif kind == 2:
                F[j, zz, yy, xx] = eqf[tab][pop]
                G[j, zz, yy, xx] = eqg[tab][pop]
            else:
                F[j, zz, yy, xx] = prev_f[j, zz, yy, xx]
                G[j, zz, yy, xx] = prev_g[j, zz, yy, xx]
    return F, G


@pytest.mark.parametrize("shifted,outlet_type,side", [(0, 6, 0), (0, 1, 0), (1, 6, 0), (1, 2, 0), (0, 6, -11),
                                                      (1, 1, -11), (1, 6, -11), (0, 2, -11)])
def test_pull_tables_match_push_loop(pkg, built_lib, shifted, outlet_type, side):
    """side 0: periodic in y; -11 / -12: inviscid side walls (specular reflection), which take the
    links that also cross another face (so every inviscid link has an inviscid axis link)."""
    s39, cap = pkg.d3q39_setup, pkg.capi
    c, k, lm0, (ff, gf, fi, gi, fo, go) = _case(pkg, shifted)
    nx, ny, nz, periodic = 14, 6, 7, (2 if side == 0 else 0)
    faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": side, "y+": side}
    prio = ("x-", "x+", "z-", "z+", "y-", "y+") if side == 0 else ("y-", "y+", "x-", "x+", "z-", "z+")
    st = s39.box_state39(nx, ny, nz, faces, shifted, 1, periodic=periodic, priority=prio)
    # a few solid nodes with bounce-back links around them, and a null link
    st[0, 3, 2:4, 5:7] = -1
    cx, cy, cz, opp = s39.lattice39(shifted, 1)
    for i in range(1, 39):
        for zz in range(nz):
            for yy in range(ny):
                for xx in range(nx):
                    if st[0, zz, yy, xx] < 0:
                        continue
                    tx, ty, tz = xx + cx[i], (yy + cy[i]) % ny, zz + cz[i]
                    if 0 <= tx < nx and 0 <= tz < nz and st[0, tz, ty, tx] < 0:
                        st[i, zz, yy, xx] = -10
    st[5, 1, 1, 1] = -666
    inl_t, out_t = [1] * 8, [outlet_type] + [1] * 7
    b = o39.bc(inl_t, out_t, ff, gf, [fi] * 8, [gi] * 8, [fo] * 8, [go] * 8)
    eqf = [ff] + [fi] * 8 + [fo] * 8
    eqg = [gf] + [gi] * 8 + [go] * 8
    ntype, rec, words = cap.links39_tables(st, periodic, shifted, 1, inl_t, out_t)
    assert (ntype == 2).sum() == len(rec) and (ntype == 0).sum() == 4
    lev = o39.Level39(nx, ny, nz)
    rng = np.random.default_rng(5)
    for zz in range(nz):
        for yy in range(ny):
            for xx in range(nx):
                _, f, g, _ = o39.init_node(k, 1 + 0.02 * rng.uniform(-1, 1), c.mach * (1 + 0.02 * rng.uniform(-1, 1)),
                                           0.01 * rng.uniform(-1, 1), 0.0, c.temperature, lm0)
                lev.fout[:, zz, yy, xx], lev.gout[:, zz, yy, xx] = f, g
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    fluid = st[0] >= 0
    for step in range(3):
        fout0, gout0 = lev.fout.copy(), lev.gout.copy()
        F, G = pull39(None, fout0, gout0, ntype, rec, words, prev_f, prev_g, eqf, eqg, cx, cy, cz, periodic)
        o39.step_links(k, lev, step, st, periodic, b, prev_f, prev_g)  # prev_* become this step's post-streaming
        assert np.array_equal(F[:, fluid], prev_f[:, fluid]), step
        assert np.array_equal(G[:, fluid], prev_g[:, fluid]), step


@pytest.mark.parametrize("shifted", [1, 0, "wedge"])
def test_wall_link_slots_match_push_loop(pkg, built_lib, shifted):
    """Interpolated wall links on the shifted and the unshifted lattice: every
    slot the tables do not mark as a wall value matches the oracle's push loop
    bit for bit, and every wall-value slot carries a wall link of its node.  On
    the shifted lattice those slots are exactly the wall links (opp(i) = i);
    on the unshifted one slot opp(i) of wall link i, unless a later rule of the
    loop writes it (a bounce-back of link opp(i) through a face writes slot i
    from the fout(x, i) the closure rewrote in place).  "wedge": the shifted
    lattice's double-ramp wedge between inviscid side walls (the inviscid
    reflections next to the walls, the wall links of the ramp)."""
    s39, cap = pkg.d3q39_setup, pkg.capi
    wedge = shifted == "wedge"
    shifted = 1 if wedge else shifted
    c, k, lm0, (ff, gf, fi, gi, fo, go) = _case(pkg, shifted)
    rng = np.random.default_rng(9)
    if wedge:
        nx, ny, nz, periodic = 20, 6, 10, 0
        st = s39.wedge_state39(nx, ny, nz, 5.0, 12.0, 20.0, s39.WEDGE_FACES, periodic=0,
                               priority=s39.WEDGE_PRIORITY)
    else:
        nx, ny, nz, periodic = 14, 6, 7, 2
        faces = {"x-": -101, "x+": -201, "z-": -10, "z+": -1000, "y-": 0, "y+": 0}
        st = s39.box_state39(nx, ny, nz, faces, shifted, 1, periodic=periodic)
        solid = np.zeros((nz, ny, nx), bool)
        solid[0:2, 1:4, 5:8] = True
        s39.wall_links39(st, solid, rng.uniform(0.05, 0.95, (39, nz, ny, nx)), shifted, 1, periodic=periodic)
    opp = s39.lattice39(shifted, 1)[3]
    inl_t, out_t = [1] * 8, [6] + [1] * 7
    fs = (c.mach, 0.0, 0.0, c.temperature)
    b = o39.bc(inl_t, out_t, ff, gf, [fi] * 8, [gi] * 8, [fo] * 8, [go] * 8, fs)
    eqf = [ff] + [fi] * 8 + [fo] * 8
    eqg = [gf] + [gi] * 8 + [go] * 8
    ntype, rec, words = cap.links39_tables(st, periodic, shifted, 1, inl_t, out_t)
    fluid = st[0] >= 0
    wall_link = (st <= -1001) & fluid[None]
    wall_link[0] = False
    link_at_slot = wall_link[opp]  # slot j holds the wall value of link opp(j)
    assert (ntype == 3).sum() == wall_link.any(axis=0).sum() > 0
    wall_slot = np.zeros_like(wall_link)
    for r, n in enumerate(rec):
        zz, yy, xx = n // (nx * ny), (n // nx) % ny, n % nx
        wall_slot[:, zz, yy, xx] = (words[r] & 3) == 3
        for j in np.nonzero((words[r] & 3) == 3)[0]:
            assert wall_link[(int(words[r, j]) >> 2) & 63, zz, yy, xx]
    if shifted:
        assert np.array_equal(wall_slot, link_at_slot)
    else:
        assert (wall_slot & link_at_slot).sum() >= 0.9 * link_at_slot.sum() > 0
    lev = o39.Level39(nx, ny, nz)
    for zz in range(nz):
        for yy in range(ny):
            for xx in range(nx):
                rho, u = 1 + 0.02 * rng.uniform(-1, 1), c.mach * (1 + 0.02 * rng.uniform(-1, 1))
                v = 0.01 * rng.uniform(-1, 1)
                lm, f, g, _ = o39.init_node(k, rho, u, v, 0.0, c.temperature, lm0)
                lev.fout[:, zz, yy, xx], lev.gout[:, zz, yy, xx], lev.lm[:, zz, yy, xx] = f, g, lm
                lev.rho[zz, yy, xx], lev.u[zz, yy, xx], lev.v[zz, yy, xx] = rho, u, v
                lev.temp[zz, yy, xx] = c.temperature
    prev_f, prev_g = lev.fout.copy(), lev.gout.copy()
    cx, cy, cz, _ = s39.lattice39(shifted, 1)
    check = fluid[None] & ~wall_slot
    for step in range(3):
        fout0, gout0 = lev.fout.copy(), lev.gout.copy()
        F, G = pull39(None, fout0, gout0, ntype, rec, words, prev_f, prev_g, eqf, eqg, cx, cy, cz, periodic)
        o39.step_links(k, lev, step, st, periodic, b, prev_f, prev_g)
        assert np.isfinite(prev_f[:, fluid]).all()
        assert np.array_equal(F[check], prev_f[check]), step
        assert np.array_equal(G[check], prev_g[check]), step
