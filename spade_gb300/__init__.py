"""spade_gb300 — GB300-native (sm_103a) explicit right-hand side of SPADE's
compressible Navier–Stokes solver.

The Python API mirrors the reference's names and argument meaning
(spade::pde_algs::flux_div, convective / viscous functors, viscous_laws,
omni::compose, grid_array, make_exchange, boundary_fill, integrator_t);
every compute call goes through the C ABI of libgbns.so (include/gbns.h).
"""
from . import _abi
from . import fluid_state, coords, boundary, state_sensor, viscous_laws, viscous, convective, omni
from . import grid, algs, pde_algs, time_integration, io, parallel
from ._native import SpadeError, lib as native_lib, LIB_PATH

__all__ = ["fluid_state", "coords", "boundary", "state_sensor", "viscous_laws", "viscous", "convective",
           "omni", "grid", "algs", "pde_algs", "time_integration", "io", "parallel", "SpadeError", "native_lib",
           "LIB_PATH"]
