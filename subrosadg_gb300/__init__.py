"""GB300-native explicit DG residual-and-update path of SubrosaDG (FP64, sm_103a).

The compute path is libsdg_gpu.so (hand-written CUDA kernels behind the C ABI of
include/sdg_gpu.h); this package is the host-side mirror of the reference's
System/Solver interface.
"""
from . import _abi
from ._abi import (ADIABATIC_NONSLIP_WALL, ADIABATIC_SLIP_WALL, BR1, BR2, CENTRAL, EULER, EXACT, FORWARD_EULER,
                   HEUN_RK2, HEXAHEDRON, HLLC, INCOMPRESSIBLE_EULER, INCOMPRESSIBLE_NAVIER_STOKES, LINE,
                   ISOTHERMAL_NONSLIP_WALL, LAX_FRIEDRICHS, NAVIER_STOKES, PERIODIC, PRESSURE_OUTFLOW, QUADRANGLE,
                   RIEMANN_FARFIELD, ROE, SHOCK_NONE, ARTIFICIAL_VISCOSITY, SOURCE_BOUSSINESQ, SOURCE_NONE, SSPRK3, TRANSPORT_CONSTANT,
                   TETRAHEDRON, TRANSPORT_NONE, TRANSPORT_SUTHERLAND, TRIANGLE, VELOCITY_INFLOW, VISCOUS_NONE, SdgError)
from .solver import (BOUNDARY_STEADY, BOUNDARY_TIME_VARYING, INITIAL_FUNCTION, INITIAL_LAST_STEP,
                     INITIAL_SPECIFIC_FILE, Batch, GpuSolver, Mesh, System, make_config)

__all__ = [n for n in dir() if not n.startswith("_")]
