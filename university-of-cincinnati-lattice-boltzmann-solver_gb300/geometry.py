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


__all__ = [
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
