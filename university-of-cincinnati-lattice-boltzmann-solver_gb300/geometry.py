"""Node-type / link-code (`state`) arrays and initial states for the benchmark
geometries, in the reference's encoding.

The reference builds its integer `state` MultiFab at set-up time in lbgrid/
(state_directions.f95:190-275 for the domain-edge codes, inter_bb_setup.f95:44-246
for wall links with packed fractions) with this encoding
(looping/timestepping/loop.f95:71-89):
  component 1 (index 0 here): node type, >= 0 fluid;
  component i: the link from the node along c_i, >= 0 interior,
  -10 bounce-back, -11 inviscid (specular), -100-k inlet k, -200-k outlet k,
  -1000 freestream, < -1001 wall link with the fraction packed
  (linkwise.f95:45-57).
These builders produce the same encoding for axis-aligned boxes; links that
cross two faces at once take the code of the face listed first in `priority`.
"""
from __future__ import annotations

import numpy as np

from .lattice import CX, CY, CZ, Q27, W, equilibrium27

CODE_BOUNCEBACK = -10
CODE_INVISCID = -11
CODE_FREESTREAM = -1000


def inlet_code(k: int) -> int:
    return -100 - k


def outlet_code(k: int) -> int:
    return -200 - k


def box_state27(nx: int, ny: int, nz: int, faces: dict, priority=("x-", "x+", "z-", "z+", "y-", "y+")) -> np.ndarray:
    """int32 state array (27, nz, ny, nx) for a box whose six faces carry the
    given link codes (keys 'x-','x+','y-','y+','z-','z+')."""
    st = np.zeros((Q27, nz, ny, nx), np.int32)
    x = np.arange(nx)[None, None, :]
    y = np.arange(ny)[None, :, None]
    z = np.arange(nz)[:, None, None]
    for i in range(1, Q27):
        comp = np.zeros((nz, ny, nx), np.int32)
        crossed = {
            "x-": np.broadcast_to(x + CX[i] < 0, comp.shape),
            "x+": np.broadcast_to(x + CX[i] >= nx, comp.shape),
            "y-": np.broadcast_to(y + CY[i] < 0, comp.shape),
            "y+": np.broadcast_to(y + CY[i] >= ny, comp.shape),
            "z-": np.broadcast_to(z + CZ[i] < 0, comp.shape),
            "z+": np.broadcast_to(z + CZ[i] >= nz, comp.shape),
        }
        for face in reversed(priority):
            comp[crossed[face]] = faces[face]
        st[i] = comp
    return st


def flat_plate_faces() -> dict:
    """Boundary-layer box: inlet 1 at x=0, outlet 1 at x=nx-1, no-slip bounce-back
    wall at z=0, freestream at z=nz-1, inviscid walls at y=0 and y=ny-1."""
    return {
        "x-": inlet_code(1),
        "x+": outlet_code(1),
        "z-": CODE_BOUNCEBACK,
        "z+": CODE_FREESTREAM,
        "y-": CODE_INVISCID,
        "y+": CODE_INVISCID,
    }


def perturbed_equilibrium(nx: int, ny: int, nz: int, u0, noise: float, seed: int) -> np.ndarray:
    """Populations (27, nz, ny, nx) at equilibrium of rho = 1 and u = u0 plus
    seeded uniform noise in [-noise, noise] per component."""
    rng = np.random.default_rng(seed)
    u = np.empty((nz, ny, nx, 3), np.float64)
    u[...] = np.asarray(u0, np.float64)
    u += rng.uniform(-noise, noise, size=u.shape)
    return equilibrium27(np.ones((nz, ny, nx)), u)


def d3q27_boundary_params(u_in, nu: float, outlet_type: int = 1, tol_alpha: float = 1e-12, tol_dH: float = 1e-10,
                          max_newton: int = 30, alpha_mode: int = 1):
    """Field values for elbm_d3q27_params: inlet 1, outlet 1 and the freestream at
    rho = 1, u = u_in (the host-side equilibria of freestream_basis_calcs.f90)."""
    feq = equilibrium27(np.ones(()), np.asarray(u_in, np.float64)[None])[:, 0]
    return {
        "nu": nu,
        "tol_alpha": tol_alpha,
        "tol_dH": tol_dH,
        "max_newton": max_newton,
        "alpha_mode": alpha_mode,
        "outlet_type": [outlet_type] + [1] * 7,
        "fs_feq": feq,
        "inl_feq": np.tile(feq, (8, 1)),
        "outl_feq": np.tile(feq, (8, 1)),
    }


def icosphere(subdivisions: int, radius: float, center) -> np.ndarray:
    """Triangles (ntri, 3, 3) of an icosphere: the icosahedron with every
    triangle split in four `subdivisions` times and the vertices projected on
    the sphere (20 * 4**subdivisions triangles; 5120 for 4), outward normals."""
    phi = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, phi, 0), (1, phi, 0), (-1, -phi, 0), (1, -phi, 0), (0, -1, phi), (0, 1, phi), (0, -1, -phi),
         (0, 1, -phi), (phi, 0, -1), (phi, 0, 1), (-phi, 0, -1), (-phi, 0, 1)]
    verts = [np.array(x, np.float64) / np.linalg.norm(x) for x in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    cache = {}

    def mid(a, b):
        key = (min(a, b), max(a, b))
        if key not in cache:
            m = verts[a] + verts[b]
            verts.append(m / np.linalg.norm(m))
            cache[key] = len(verts) - 1
        return cache[key]

    for _ in range(subdivisions):
        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts) * radius + np.asarray(center, np.float64)
    return np.ascontiguousarray(V[np.array(faces)])


def sphere_faces() -> dict:
    """Flow past a sphere: inlet 1 at x=0, outlet 1 at x=nx-1, freestream on the other faces."""
    return {"x-": inlet_code(1), "x+": outlet_code(1), "y-": CODE_FREESTREAM, "y+": CODE_FREESTREAM,
            "z-": CODE_FREESTREAM, "z+": CODE_FREESTREAM}


def sphere_state27(nx: int, ny: int, nz: int, radius: float, center, subdivisions: int = 4) -> np.ndarray:
    """state array of a box with sphere_faces() and an icosphere whose wall links
    carry packed fractions (elbm_mark_triangles, the library's set-up code)."""
    from .capi import mark_triangles

    st = box_state27(nx, ny, nz, sphere_faces())
    tri = icosphere(subdivisions, radius, center)
    mark_triangles(st, (0.0, 0.0, 0.0), 1.0, tri)
    return st


def slice_state27(st: np.ndarray, lo, hi, g: int = 1) -> np.ndarray:
    """The state FAB of box [lo, hi] (inclusive, indices into st) with g ghost
    layers, as AMReX's fill_boundary gives it; outside st: not fluid (-1)."""
    q, nz, ny, nx = st.shape
    out = np.full((q, hi[2] - lo[2] + 1 + 2 * g, hi[1] - lo[1] + 1 + 2 * g, hi[0] - lo[0] + 1 + 2 * g), -1, np.int32)
    src = [slice(max(lo[a] - g, 0), min(hi[a] + g, n - 1) + 1) for a, n in enumerate((nx, ny, nz))]
    dst = [slice(sl.start - (lo[a] - g), sl.stop - (lo[a] - g)) for a, sl in enumerate(src)]
    out[:, dst[2], dst[1], dst[0]] = st[:, src[2], src[1], src[0]]
    return out


def _segments(rng, total: int, count: int, edges) -> list:
    """count lengths drawn from edges that sum to total (rejection sampling)."""
    for _ in range(1000000):
        seg = rng.choice(edges, count)
        if int(seg.sum()) == total:
            return [int(v) for v in seg]
    raise ValueError(f"no {count} lengths from {edges} sum to {total}")


AMR_GHOST = 10000000  # node type of a fine level's ghost nodes (filled from the coarser level)


def amr_sphere_hierarchy(seed: int = 2024, shell: int = 2, edges=(16, 24, 32, 40, 48)):
    """The 3-level AMR case around the sphere of the 256x128x128 case, at ratio 2:
    level 0 is that domain at half resolution (128x64x64, sphere of radius 8 at
    (32, 32, 32)); level 1 holds 24 boxes and level 2 holds 96 boxes with seeded
    edge lengths from `edges` (multiples of 8) that tile a block around the
    sphere and its wake (level 1: x [16, 128), y [16, 112), z [24, 104) in its own
    index space, split 4 x 3 x 2; level 2: x [88, 232), y [72, 184), z [72, 184),
    split 6 x 4 x 4), so that the refinement covers the shell of radius 10..28
    (level-0 units) on the sphere's sides and its near wake.  Each fine level is
    framed by `shell` ghost layers (node type AMR_GHOST, filled from the coarser
    level), held in six slab boxes; a level-2 box's ghost nodes lie over valid
    level-1 nodes.  Returns a list over levels of dicts: 'boxes' (inclusive
    (lo, hi) in the level's index space, valid boxes first), 'nvalid', 'origin'
    and 'state' (the level-wide state array from origin, sphere wall links
    marked) and 'scale' (2^level)."""
    from .capi import mark_triangles

    rng = np.random.default_rng(seed)
    tri = icosphere(4, 8.0, (32.0, 32.0, 32.0))
    levels = []
    st0 = box_state27(128, 64, 64, sphere_faces())
    mark_triangles(st0, (0.0, 0.0, 0.0), 1.0, tri)
    levels.append({"boxes": [((0, 0, 0), (127, 63, 63))], "nvalid": 1, "origin": (0, 0, 0), "state": st0, "scale": 1})
    regions = {1: (((16, 128), (16, 112), (24, 104)), (4, 3, 2)), 2: (((88, 232), (72, 184), (72, 184)), (6, 4, 4))}
    for lvl in (1, 2):
        (rx, ry, rz), counts = regions[lvl]
        r = (rx, ry, rz)
        cuts = []
        for a in range(3):
            seg = _segments(rng, r[a][1] - r[a][0], counts[a], edges)
            cuts.append(np.concatenate([[r[a][0]], r[a][0] + np.cumsum(seg)]))
        boxes = []
        for k in range(counts[2]):
            for j in range(counts[1]):
                for i in range(counts[0]):
                    lo = (int(cuts[0][i]), int(cuts[1][j]), int(cuts[2][k]))
                    hi = (int(cuts[0][i + 1]) - 1, int(cuts[1][j + 1]) - 1, int(cuts[2][k + 1]) - 1)
                    boxes.append((lo, hi))
        a0, b0 = [v[0] for v in r], [v[1] for v in r]
        s = shell
        # the ghost frame as six disjoint slabs (z faces over the full frame, then y, then x)
        slabs = [((a0[0] - s, a0[1] - s, a0[2] - s), (b0[0] + s - 1, b0[1] + s - 1, a0[2] - 1)),
                 ((a0[0] - s, a0[1] - s, b0[2]), (b0[0] + s - 1, b0[1] + s - 1, b0[2] + s - 1)),
                 ((a0[0] - s, a0[1] - s, a0[2]), (b0[0] + s - 1, a0[1] - 1, b0[2] - 1)),
                 ((a0[0] - s, b0[1], a0[2]), (b0[0] + s - 1, b0[1] + s - 1, b0[2] - 1)),
                 ((a0[0] - s, a0[1], a0[2]), (a0[0] - 1, b0[1] - 1, b0[2] - 1)),
                 ((b0[0], a0[1], a0[2]), (b0[0] + s - 1, b0[1] - 1, b0[2] - 1))]
        origin = tuple(v - s for v in a0)
        dims = [b0[a] - a0[a] + 2 * s for a in range(3)]
        st = np.zeros((Q27, dims[2], dims[1], dims[0]), np.int32)
        ghost = np.ones((dims[2], dims[1], dims[0]), bool)
        ghost[s:-s, s:-s, s:-s] = False
        st[0][ghost] = AMR_GHOST
        scale = 2 ** lvl
        mark_triangles(st, tuple(o / scale for o in origin), 1.0 / scale, tri)
        levels.append({"boxes": boxes + slabs, "nvalid": len(boxes), "origin": origin, "state": st, "scale": scale})
    return levels


def register_amr_hierarchy(ctx, levels, storage, u_in=(0.08, 0.0, 0.0), nu_level1: float = 5e-4,
                           noise: float = 1e-3, seed: int = 77) -> list:
    """Register the levels of amr_sphere_hierarchy on a context: boxes, D3Q27
    parameters (the viscosity of the 256x128x128 case, 5e-4, on level 1; a
    level's lattice viscosity doubles with each refinement at fixed physical
    viscosity under acoustic scaling), per-box state slices with one ghost
    layer, populations at the equilibrium of u_in with seeded noise (solid nodes
    at w), and the coarse-fine maps.  Returns the level-wide initial
    populations."""
    from .capi import ELBM_D3Q27, make_d3q27_params

    f_all = []
    for lvl, L in enumerate(levels):
        st, o = L["state"], L["origin"]
        ctx.level_register(lvl, ELBM_D3Q27, storage, [list(lo) + list(hi) for lo, hi in L["boxes"]])
        bp = d3q27_boundary_params(u_in, nu_level1 * 2.0 ** (lvl - 1))
        ctx.set_d3q27_params(lvl, make_d3q27_params(**bp))
        nz, ny, nx = st.shape[1:]
        f = perturbed_equilibrium(nx, ny, nz, u_in, noise, seed=seed + lvl)
        f[:, st[0] == -1001] = W[:, None]
        for k, (lo, hi) in enumerate(L["boxes"]):
            rl = [lo[a] - o[a] for a in range(3)]
            rh = [hi[a] - o[a] for a in range(3)]
            ctx.set_links(lvl, k, slice_state27(st, rl, rh, 1), ngrow_state=1)
            ctx.upload(lvl, k, np.ascontiguousarray(f[:, rl[2]:rh[2] + 1, rl[1]:rh[1] + 1, rl[0]:rh[0] + 1]))
        f_all.append(f)
    for lvl in range(1, len(levels)):
        ctx.interlevel_setup(lvl)
    return f_all


__all__ = [
    "icosphere",
    "sphere_faces",
    "sphere_state27",
    "box_state27",
    "flat_plate_faces",
    "perturbed_equilibrium",
    "d3q27_boundary_params",
    "inlet_code",
    "slice_state27",
    "amr_sphere_hierarchy",
    "register_amr_hierarchy",
    "AMR_GHOST",
    "outlet_code",
    "CODE_BOUNCEBACK",
    "CODE_INVISCID",
    "CODE_FREESTREAM",
    "W",
]
