"""GB300-native entropic lattice Boltzmann level step for the University of
Cincinnati Lattice Boltzmann Solver.

The product is libelbm_gb300.so (csrc/, C ABI in include/elbm_gb300.h).  This
package holds its build recipe, the ctypes binding used by Python callers and
tests, and host-side set-up helpers (lattice tables, boundary equilibria,
state arrays for box geometries).
"""
from . import capi, d3q39_setup, geometry, lattice  # noqa: F401
from .build import build  # noqa: F401
from .capi import Context, ElbmError, make_d3q27_params  # noqa: F401
