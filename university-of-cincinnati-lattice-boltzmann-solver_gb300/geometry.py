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


__all__ = [
    "icosphere",
    "sphere_faces",
    "sphere_state27",
    "box_state27",
    "flat_plate_faces",
    "perturbed_equilibrium",
    "d3q27_boundary_params",
    "inlet_code",
    "outlet_code",
    "CODE_BOUNCEBACK",
    "CODE_INVISCID",
    "CODE_FREESTREAM",
    "W",
]
