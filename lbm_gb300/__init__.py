"""lbm_gb300: a lattice Boltzmann time step for one GB300 GPU, behind the reference's API.

The compute path is liblbm_gb300.so (CUDA, sm_103a), reached through the C ABI declared in
include/lbm_gb300.h. This package is the Python mirror of the reference's model / domain /
collision / boundary interface on top of it, plus the scenario descriptions.
"""
from . import capi, model
from .capi import LbmError, load_library
from .domain import (BGKCollision, BoundaryKeeper, Collision, Domain, FluidCollision, FreeSlipBoundary,
                     InflowBoundary, MovingWallBoundary, NoSlipBoundary, NonFluidCollision,
                     OutflowBoundary, PressureBoundary)
from .model import C_S, d3q15, d3q19, d3q27
from .scenario import Boundary, Scenario, build_domain

__all__ = [
    "capi", "model", "LbmError", "load_library", "BGKCollision", "BoundaryKeeper", "Collision", "Domain",
    "FluidCollision", "FreeSlipBoundary", "InflowBoundary", "MovingWallBoundary", "NoSlipBoundary",
    "NonFluidCollision", "OutflowBoundary", "PressureBoundary", "C_S", "d3q15", "d3q19", "d3q27",
    "Boundary", "Scenario", "build_domain",
]
