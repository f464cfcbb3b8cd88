"""ctypes binding of the C ABI declared in include/sdg_gpu.h.

The shared library is built in-tree (subrosadg_gb300/lib/libsdg_gpu.so) by
subrosadg_gb300.build.build_library().  Loading fails loudly when it is missing:
there is no CPU fallback for the GPU path.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int32, c_int64, c_uint32, c_uint64, c_void_p

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(_HERE, "lib", "libsdg_gpu.so")

SDG_OK = 0
ERRORS = {
    1: "SDG_ERR_INVALID_ARGUMENT",
    2: "SDG_ERR_CUDA",
    3: "SDG_ERR_OUT_OF_MEMORY",
    4: "SDG_ERR_MESH",
    5: "SDG_ERR_UNSUPPORTED",
    6: "SDG_ERR_NONFINITE",
    7: "SDG_ERR_TIMEOUT",
    8: "SDG_ERR_STATE",
}
globals().update({name: code for code, name in ERRORS.items()})

LINE, TRIANGLE, QUADRANGLE, TETRAHEDRON, HEXAHEDRON = 1, 2, 3, 4, 5
EULER, NAVIER_STOKES, INCOMPRESSIBLE_EULER, INCOMPRESSIBLE_NAVIER_STOKES = 0, 1, 2, 3
SOURCE_NONE, SOURCE_BOUSSINESQ = 0, 1
SHOCK_NONE, ARTIFICIAL_VISCOSITY = 0, 1
CENTRAL, LAX_FRIEDRICHS, HLLC, ROE, EXACT = 0, 1, 2, 3, 4
VISCOUS_NONE, BR1, BR2 = 0, 1, 2
FORWARD_EULER, HEUN_RK2, SSPRK3 = 0, 1, 2
TRANSPORT_NONE, TRANSPORT_CONSTANT, TRANSPORT_SUTHERLAND = 0, 1, 2
(RIEMANN_FARFIELD, VELOCITY_INFLOW, PRESSURE_OUTFLOW, ISOTHERMAL_NONSLIP_WALL,
 ADIABATIC_SLIP_WALL, ADIABATIC_NONSLIP_WALL, PERIODIC) = range(7)

_p_double = POINTER(c_double)
_p_int32 = POINTER(c_int32)


class SdgMesh(ctypes.Structure):
    _fields_ = [
        ("dimension", c_int32),
        ("node_count", c_int64),
        ("node_coordinate", _p_double),
        ("periodic_master", _p_int32),
        ("triangle_count", c_int64),
        ("triangle_node", _p_int32),
        ("quadrangle_count", c_int64),
        ("quadrangle_node", _p_int32),
        ("hexahedron_count", c_int64),
        ("hexahedron_node", _p_int32),
        ("boundary_count", c_int64),
        ("boundary_node", _p_int32),
        ("boundary_physical", _p_int32),
        ("physical_count", c_int32),
        ("physical_boundary_condition", _p_int32),
        ("line_count", c_int64),
        ("line_node", _p_int32),
        ("tetrahedron_count", c_int64),
        ("tetrahedron_node", _p_int32),
        ("geometry_order", c_int32),
        ("triangle_geometry_node", _p_int32),
        ("quadrangle_geometry_node", _p_int32),
        ("hexahedron_geometry_node", _p_int32),
    ]


class SdgConfig(ctypes.Structure):
    _fields_ = [
        ("polynomial_order", c_int32),
        ("equation", c_int32),
        ("convective_flux", c_int32),
        ("viscous_flux", c_int32),
        ("time_integration", c_int32),
        ("transport_model", c_int32),
        ("specific_heat_ratio", c_double),
        ("specific_heat_constant_pressure", c_double),
        ("specific_heat_constant_volume", c_double),
        ("dynamic_viscosity", c_double),
        ("prandtl_number", c_double),
        ("reference_sound_speed", c_double),
        ("reference_density", c_double),
        ("source_term", c_int32),
        ("thermal_expansion_coefficient", c_double),
        ("reference_temperature", c_double),
        ("shock_capturing", c_int32),
        ("empirical_tolerance", c_double),
        ("artificial_viscosity_factor", c_double),
    ]


class SdgCounts(ctypes.Structure):
    _fields_ = [
        ("dimension", c_int32),
        ("conserved_variable_count", c_int32),
        ("block_count", c_int32),
        ("block_element_type", c_int32 * 2),
        ("block_element_count", c_int64 * 2),
        ("block_basis_count", c_int32 * 2),
        ("block_volume_point_count", c_int32 * 2),
        ("element_count", c_int64),
        ("volume_point_count", c_int64),
        ("degree_of_freedom_count", c_int64),
        ("interior_face_count", c_int64),
        ("boundary_face_count", c_int64),
        ("face_point_count", c_int32),
        ("boundary_point_count", c_int64),
    ]


class SdgGeneratedMesh(ctypes.Structure):
    _fields_ = [("mesh", SdgMesh), ("storage", c_void_p)]


class SdgBatchCounts(ctypes.Structure):
    _fields_ = [
        ("instance_count", c_int32),
        ("launches_per_step", c_int32),
        ("sequential_launches_per_step", c_int32),
        ("persistent_ctas_per_sm", c_int32),
        ("work_items_per_step", c_int64),
        ("element_count", c_int64),
        ("degree_of_freedom_count", c_int64),
        ("stage_count", c_int32),
    ]


AUTOTUNE_RETIME = 1


# name -> (restype, argtypes); every symbol include/sdg_gpu.h declares.
SIGNATURES = {
    "sdg_last_error": (c_char_p, [c_void_p]),
    "sdg_create": (c_int32, [POINTER(SdgMesh), POINTER(SdgConfig), c_int32, POINTER(c_void_p)]),
    "sdg_destroy": (c_int32, [c_void_p]),
    "sdg_get_counts": (c_int32, [c_void_p, POINTER(SdgCounts)]),
    "sdg_volume_point_coordinate": (c_int32, [c_void_p, _p_double]),
    "sdg_boundary_point_coordinate": (c_int32, [c_void_p, _p_double, _p_int32]),
    "sdg_set_initial_primitive": (c_int32, [c_void_p, _p_double]),
    "sdg_set_boundary_primitive": (c_int32, [c_void_p, _p_double]),
    "sdg_set_state_point": (c_int32, [c_void_p, _p_double]),
    "sdg_get_state_point": (c_int32, [c_void_p, _p_double]),
    "sdg_set_state_modal": (c_int32, [c_void_p, _p_double]),
    "sdg_get_state_modal": (c_int32, [c_void_p, _p_double]),
    "sdg_calculate_delta_time": (c_int32, [c_void_p, c_double, _p_double]),
    "sdg_step": (c_int32, [c_void_p, c_int32, c_double]),
    "sdg_step_async": (c_int32, [c_void_p, c_int32, c_double]),
    "sdg_step_state_point": (c_int32, [c_void_p, c_double, _p_double, _p_double]),
    "sdg_step_state_point_from": (c_int32, [c_void_p, c_double, _p_double, _p_double, _p_double]),
    "sdg_step_state_point_from_async": (c_int32, [c_void_p, c_double, _p_double, _p_double]),
    "sdg_relative_error": (c_int32, [c_void_p, _p_double]),
    "sdg_residual_point": (c_int32, [c_void_p, _p_double]),
    "sdg_synchronize": (c_int32, [c_void_p]),
    "sdg_launch_count": (c_int32, [c_void_p, POINTER(c_int64)]),
    "sdg_adjacency": (c_int32, [c_void_p, _p_int32, _p_int32]),
    "sdg_get_stream": (c_int32, [c_void_p, POINTER(c_void_p)]),
    "sdg_set_kernel_timing": (c_int32, [c_void_p, c_int32]),
    "sdg_kernel_time": (c_int32, [c_void_p, _p_double, POINTER(c_int64)]),
    "sdg_measure_fp64_peak": (c_int32, [c_int32, c_double, _p_double]),
    "sdg_measure_dmma_peak": (c_int32, [c_int32, c_int32, c_double, _p_double]),
    "sdg_probe_reciprocal": (c_int32, [c_int32, _p_double, _p_double, c_int64]),
    "sdg_delta_time_noalloc": (c_int32, [c_void_p, c_void_p, c_int64, c_int32, c_int32, c_int32, c_double, c_double,
                                         c_double, c_void_p, c_void_p]),
    "sdg_mesh_generate_2d": (c_int32, [c_double, c_double, c_double, c_double, c_int32, c_int32, c_double,
                                       c_double, c_uint64, c_int32, _p_int32, POINTER(SdgGeneratedMesh)]),
    "sdg_mesh_generate_1d": (c_int32, [c_double, c_double, c_int32, c_int32, _p_int32, c_void_p]),
    "sdg_mesh_generate_annulus": (c_int32, [c_double, c_double, c_int32, c_int32, c_int32, c_double, c_uint64,
                                            _p_int32, POINTER(SdgGeneratedMesh)]),
    "sdg_mesh_generate_3d": (c_int32, [c_double, c_double, c_double, c_double, c_double, c_double, c_int32,
                                       c_int32, c_int32, c_int32, _p_int32, POINTER(SdgGeneratedMesh)]),
    "sdg_mesh_generate_3d_tetrahedra": (c_int32, [c_double, c_double, c_double, c_double, c_double, c_double,
                                                  c_int32, c_int32, c_int32, c_int32, _p_int32,
                                                  POINTER(SdgGeneratedMesh)]),
    "sdg_mesh_read_msh": (c_int32, [c_char_p, POINTER(SdgGeneratedMesh)]),
    "sdg_mesh_free": (c_int32, [POINTER(SdgGeneratedMesh)]),
    "sdg_get_node_artificial_viscosity": (c_int32, [c_void_p, _p_double]),
    "sdg_adjoint_boundary_cotangent": (c_int32, [c_void_p, _p_double]),
    "sdg_surface_force": (c_int32, [c_void_p, c_int32, _p_double]),
    "sdg_surface_force_cotangent": (c_int32, [c_void_p, c_int32, _p_double, _p_double]),
    "sdg_write_raw_binary": (c_int32, [c_void_p, c_char_p]),
    "sdg_set_boundary_face_order": (c_int32, [c_void_p, c_int64, _p_int32]),
    "sdg_read_raw_binary": (c_int32, [c_void_p, c_char_p, c_int32]),
    "sdg_set_graph": (c_int32, [c_void_p, c_int32]),
    "sdg_set_wait_check": (c_int32, [c_void_p, c_uint32, c_uint32]),
    "sdg_get_tile": (c_int32, [c_void_p, c_int32, _p_int32, _p_int32, _p_int32, _p_int32]),
    "sdg_set_tile": (c_int32, [c_void_p, c_int32, c_int32, c_int32, c_int32, c_int32]),
    "sdg_autotune": (c_int32, [c_void_p, c_int32]),
    "sdg_batch_create": (c_int32, [POINTER(c_void_p), c_int32, POINTER(c_void_p)]),
    "sdg_batch_destroy": (c_int32, [c_void_p]),
    "sdg_batch_get_counts": (c_int32, [c_void_p, POINTER(SdgBatchCounts)]),
    "sdg_batch_set_delta_time": (c_int32, [c_void_p, _p_double]),
    "sdg_batch_set_persistence": (c_int32, [c_void_p, c_int32]),
    "sdg_batch_step_async": (c_int32, [c_void_p, c_int32]),
    "sdg_batch_step_sequential_async": (c_int32, [c_void_p, c_int32]),
    "sdg_batch_synchronize": (c_int32, [c_void_p]),
    "sdg_batch_autotune": (c_int32, [c_void_p, c_int32]),
    "sdg_batch_get_stream": (c_int32, [c_void_p, POINTER(c_void_p)]),
    "sdg_batch_last_error": (c_char_p, [c_void_p]),
    "sdg_volume_point_weight": (c_int32, [c_void_p, _p_double]),
    "sdg_set_viscosity": (c_int32, [c_void_p, c_double]),
    "sdg_jvp_residual": (c_int32, [c_void_p, _p_double, c_double, _p_double]),
    "sdg_vjp_residual": (c_int32, [c_void_p, _p_double, _p_double, _p_double]),
    "sdg_jvp_steps": (c_int32, [c_void_p, c_int32, c_double, _p_double, c_double, _p_double]),
    "sdg_adjoint_steps": (c_int32, [c_void_p, c_int32, c_double, c_int32, _p_double, _p_double, _p_double]),
    "sdg_adjoint_memory": (c_int32, [c_void_p, POINTER(c_int64)]),
    "sdg_set_adjoint_trajectory_store": (c_int32, [c_void_p, c_int32]),
    "sdg_forward_steps": (c_int32, [c_void_p, c_int32, c_double, c_int32]),
    "sdg_adjoint_recorded": (c_int32, [c_void_p, _p_double, _p_double, _p_double]),
}

_lib = None


class SdgError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


def load(path: str | None = None):
    """Load libsdg_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIBRARY_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int, handle=None):
    if rc != SDG_OK:
        lib = load()
        msg = lib.sdg_last_error(handle)
        raise SdgError(rc, msg.decode() if msg else "")
