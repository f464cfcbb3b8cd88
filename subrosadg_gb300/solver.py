"""Host-side mirror of SubrosaDG's System/Solver interface over the GB300 C ABI.

`Mesh` holds first-order mesh arrays (generated, read from MSH 4.1, or given);
`GpuSolver` owns one sdg_handle and exposes the members the reference's
System<SC>::solve drives (src/Utils/SystemControl.cpp:159-195):
initializeSolver, calculateDeltaTime, stepSolver, relative_error_;
`System` mirrors the reference's System facade (setMesh, addBoundaryCondition,
setThermodynamicModel, setTransportModel, setTimeIntegration, setDeltaTime,
synchronize, solve) so a driver reads like examples/*.cpp.
"""
from __future__ import annotations

import ctypes
import math
import os
import shutil
from ctypes import POINTER, byref, c_double, c_int32, c_int64, c_void_p

import numpy as np

from . import _abi
from ._abi import SdgConfig, SdgCounts, SdgGeneratedMesh, SdgMesh, check

_pd = POINTER(c_double)
_pi = POINTER(c_int32)


def _ptr(a, kind=_pd):
    return a.ctypes.data_as(kind) if a is not None else None


class Mesh:
    """First-order mesh in gmsh vertex order (the input format of sdg_create)."""

    def __init__(self, dimension, nodes, triangles=None, quadrangles=None, hexahedra=None, boundary=None,
                 boundary_physical=None, physical_conditions=None, periodic_master=None, lines=None,
                 tetrahedra=None, geometry_order=1, triangle_geometry=None, quadrangle_geometry=None,
                 hexahedron_geometry=None):
        self.dimension = int(dimension)
        # curved meshes: order-q geometry nodes per element in gmsh order (corners first)
        self.geometry_order = int(geometry_order)
        q = self.geometry_order
        self.triangle_geometry = None if triangle_geometry is None or len(triangle_geometry) == 0 else \
            np.ascontiguousarray(triangle_geometry, np.int32).reshape(-1, (q + 1) * (q + 2) // 2)
        self.quadrangle_geometry = None if quadrangle_geometry is None or len(quadrangle_geometry) == 0 else \
            np.ascontiguousarray(quadrangle_geometry, np.int32).reshape(-1, (q + 1) ** 2)
        self.hexahedron_geometry = None if hexahedron_geometry is None or len(hexahedron_geometry) == 0 else \
            np.ascontiguousarray(hexahedron_geometry, np.int32).reshape(-1, (q + 1) ** 3)
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1, 3)
        self.lines = None if lines is None or len(lines) == 0 else np.ascontiguousarray(lines, np.int32).reshape(-1, 2)
        self.triangles = None if triangles is None or len(triangles) == 0 else np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
        self.quadrangles = None if quadrangles is None or len(quadrangles) == 0 else np.ascontiguousarray(quadrangles, np.int32).reshape(-1, 4)
        self.hexahedra = None if hexahedra is None or len(hexahedra) == 0 else np.ascontiguousarray(hexahedra, np.int32).reshape(-1, 8)
        self.tetrahedra = None if tetrahedra is None or len(tetrahedra) == 0 else np.ascontiguousarray(tetrahedra, np.int32).reshape(-1, 4)
        nbv = {1: 1, 2: 2}.get(self.dimension, 4)
        self.boundary = np.zeros((0, nbv), np.int32) if boundary is None else np.ascontiguousarray(boundary, np.int32).reshape(-1, nbv)
        self.boundary_physical = np.zeros(0, np.int32) if boundary_physical is None else np.ascontiguousarray(boundary_physical, np.int32)
        self.physical_conditions = np.zeros(0, np.int32) if physical_conditions is None else np.ascontiguousarray(physical_conditions, np.int32)
        self.periodic_master = None if periodic_master is None else np.ascontiguousarray(periodic_master, np.int32)

    @classmethod
    def _from_generated(cls, g: SdgGeneratedMesh):
        m = g.mesh
        def arr(p, n, w, dt):
            if not p or n == 0:
                return None
            return np.ctypeslib.as_array(p, shape=(n * w,)).astype(dt).copy()
        nbv = {1: 1, 2: 2}.get(m.dimension, 4)
        out = cls(m.dimension, arr(m.node_coordinate, m.node_count, 3, np.float64),
                  arr(m.triangle_node, m.triangle_count, 3, np.int32),
                  arr(m.quadrangle_node, m.quadrangle_count, 4, np.int32),
                  arr(m.hexahedron_node, m.hexahedron_count, 8, np.int32),
                  arr(m.boundary_node, m.boundary_count, nbv, np.int32),
                  arr(m.boundary_physical, m.boundary_count, 1, np.int32),
                  arr(m.physical_boundary_condition, m.physical_count, 1, np.int32),
                  arr(m.periodic_master, m.node_count, 1, np.int32),
                  arr(m.line_node, m.line_count, 2, np.int32),
                  arr(m.tetrahedron_node, m.tetrahedron_count, 4, np.int32))
        q = m.geometry_order
        if q > 1:
            out.geometry_order = q
            if m.triangle_count:
                out.triangle_geometry = arr(m.triangle_geometry_node, m.triangle_count, (q + 1) * (q + 2) // 2,
                                            np.int32).reshape(m.triangle_count, -1)
            if m.quadrangle_count:
                out.quadrangle_geometry = arr(m.quadrangle_geometry_node, m.quadrangle_count, (q + 1) ** 2,
                                              np.int32).reshape(m.quadrangle_count, -1)
            if m.hexahedron_count and m.hexahedron_geometry_node:
                out.hexahedron_geometry = arr(m.hexahedron_geometry_node, m.hexahedron_count, (q + 1) ** 3,
                                              np.int32).reshape(m.hexahedron_count, -1)
        _abi.load().sdg_mesh_free(byref(g))
        return out

    @classmethod
    def line_1d(cls, x0, lx, nx, periodic=True, boundary_conditions=None):
        """[x0, x0 + lx] in nx lines: periodic (one group) or groups 1 (x0 end) and 2 (x0 + lx end)."""
        lib = _abi.load()
        g = SdgGeneratedMesh()
        bc = None if boundary_conditions is None else np.ascontiguousarray(boundary_conditions, np.int32)
        check(lib.sdg_mesh_generate_1d(x0, lx, nx, int(periodic), _ptr(bc, _pi), byref(g)))
        return cls._from_generated(g)

    @classmethod
    def box_2d(cls, x0, y0, lx, ly, nx, ny, periodic=True, jitter=0.0, split_fraction=0.0, seed=0,
               boundary_conditions=None):
        lib = _abi.load()
        g = SdgGeneratedMesh()
        bc = None if boundary_conditions is None else np.ascontiguousarray(boundary_conditions, np.int32)
        check(lib.sdg_mesh_generate_2d(x0, y0, lx, ly, nx, ny, jitter, split_fraction, seed, int(periodic),
                                       _ptr(bc, _pi), byref(g)))
        return cls._from_generated(g)

    @classmethod
    def box_3d(cls, x0, y0, z0, lx, ly, lz, nx, ny, nz, periodic=True, boundary_conditions=None):
        lib = _abi.load()
        g = SdgGeneratedMesh()
        bc = None if boundary_conditions is None else np.ascontiguousarray(boundary_conditions, np.int32)
        check(lib.sdg_mesh_generate_3d(x0, y0, z0, lx, ly, lz, nx, ny, nz, int(periodic), _ptr(bc, _pi), byref(g)))
        return cls._from_generated(g)

    @classmethod
    def box_3d_tetrahedra(cls, x0, y0, z0, lx, ly, lz, nx, ny, nz, periodic=True, boundary_conditions=None):
        """box_3d with every hexahedron split into six tetrahedra (triangular boundary elements, same groups)."""
        lib = _abi.load()
        g = SdgGeneratedMesh()
        bc = None if boundary_conditions is None else np.ascontiguousarray(boundary_conditions, np.int32)
        check(lib.sdg_mesh_generate_3d_tetrahedra(x0, y0, z0, lx, ly, lz, nx, ny, nz, int(periodic), _ptr(bc, _pi),
                                                  byref(g)))
        return cls._from_generated(g)

    @classmethod
    def annulus(cls, inner_radius, outer_radius, nr, ntheta, geometry_order=1, split_fraction=0.0, seed=0,
                boundary_conditions=(_abi.RIEMANN_FARFIELD, _abi.RIEMANN_FARFIELD)):
        """Curved annulus of nr x ntheta elements of geometry order q (nodes on the exact circles); groups 1 (inner
        circle) and 2 (outer circle)."""
        lib = _abi.load()
        g = SdgGeneratedMesh()
        bc = np.ascontiguousarray(boundary_conditions, np.int32)
        check(lib.sdg_mesh_generate_annulus(inner_radius, outer_radius, nr, ntheta, geometry_order, split_fraction,
                                            seed, _ptr(bc, _pi), byref(g)))
        return cls._from_generated(g)

    @classmethod
    def read_msh(cls, path):
        lib = _abi.load()
        g = SdgGeneratedMesh()
        check(lib.sdg_mesh_read_msh(str(path).encode(), byref(g)))
        return cls._from_generated(g)

    def set_boundary_condition(self, physical_index, condition):
        """System::addBoundaryCondition<BC>(physical_index) (src/Utils/SystemControl.cpp:76-80)."""
        if physical_index < 1 or physical_index > len(self.physical_conditions):
            raise ValueError("physical index out of range")
        self.physical_conditions[physical_index - 1] = condition

    def struct(self) -> SdgMesh:
        m = SdgMesh()
        m.dimension = self.dimension
        m.node_count = self.nodes.shape[0]
        m.node_coordinate = _ptr(self.nodes)
        m.periodic_master = _ptr(self.periodic_master, _pi)
        m.triangle_count = 0 if self.triangles is None else self.triangles.shape[0]
        m.triangle_node = _ptr(self.triangles, _pi)
        m.quadrangle_count = 0 if self.quadrangles is None else self.quadrangles.shape[0]
        m.quadrangle_node = _ptr(self.quadrangles, _pi)
        m.hexahedron_count = 0 if self.hexahedra is None else self.hexahedra.shape[0]
        m.hexahedron_node = _ptr(self.hexahedra, _pi)
        m.boundary_count = self.boundary.shape[0]
        m.boundary_node = _ptr(self.boundary, _pi)
        m.boundary_physical = _ptr(self.boundary_physical, _pi)
        m.physical_count = len(self.physical_conditions)
        m.physical_boundary_condition = _ptr(self.physical_conditions, _pi)
        m.line_count = 0 if self.lines is None else self.lines.shape[0]
        m.line_node = _ptr(self.lines, _pi)
        m.tetrahedron_count = 0 if self.tetrahedra is None else self.tetrahedra.shape[0]
        m.tetrahedron_node = _ptr(self.tetrahedra, _pi)
        m.geometry_order = self.geometry_order if self.geometry_order > 1 else 0
        m.triangle_geometry_node = _ptr(self.triangle_geometry, _pi)
        m.quadrangle_geometry_node = _ptr(self.quadrangle_geometry, _pi)
        m.hexahedron_geometry_node = _ptr(self.hexahedron_geometry, _pi)
        return m


def make_config(polynomial_order, equation=_abi.EULER, convective_flux=_abi.HLLC, viscous_flux=_abi.VISCOUS_NONE,
                time_integration=_abi.SSPRK3, cp=2.5, cv=25.0 / 14.0, gamma=1.4, mu=0.0, prandtl=0.71,
                transport=_abi.TRANSPORT_CONSTANT, sound_speed=0.0, density=1.0, source=_abi.SOURCE_NONE,
                thermal_expansion=0.0, reference_temperature=0.0, shock_capturing=_abi.SHOCK_NONE,
                empirical_tolerance=0.0, artificial_viscosity_factor=1.0) -> SdgConfig:
    c = SdgConfig()
    c.polynomial_order = polynomial_order
    c.equation = equation
    c.convective_flux = convective_flux
    c.viscous_flux = viscous_flux
    c.time_integration = time_integration
    c.transport_model = transport
    c.specific_heat_ratio = gamma
    c.specific_heat_constant_pressure = cp
    c.specific_heat_constant_volume = cv
    c.dynamic_viscosity = mu
    c.prandtl_number = prandtl
    c.reference_sound_speed = sound_speed
    c.reference_density = density
    c.source_term = source
    c.thermal_expansion_coefficient = thermal_expansion
    c.reference_temperature = reference_temperature
    c.shock_capturing = shock_capturing
    c.empirical_tolerance = empirical_tolerance
    c.artificial_viscosity_factor = artificial_viscosity_factor
    return c


class GpuSolver:
    """The GPU Solver<SC>: one sdg_handle on one device."""

    def __init__(self, mesh: Mesh, config: SdgConfig, device: int = 0):
        self.lib = _abi.load()
        self.mesh = mesh
        self.config = config
        self._m = mesh.struct()
        h = c_void_p()
        check(self.lib.sdg_create(byref(self._m), byref(config), device, byref(h)))
        self.h = h
        c = SdgCounts()
        check(self.lib.sdg_get_counts(self.h, byref(c)), self.h)
        self.counts = c
        self.nv = c.conserved_variable_count
        self.relative_error_ = np.zeros(self.nv)

    def close(self):
        if getattr(self, "h", None):
            self.lib.sdg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        check(rc, self.h)

    # geometry ----------------------------------------------------------------------------------
    def volume_points(self):
        out = np.zeros((self.counts.volume_point_count, 3))
        self._chk(self.lib.sdg_volume_point_coordinate(self.h, _ptr(out)))
        return out

    def boundary_points(self):
        out = np.zeros((self.counts.boundary_point_count, 3))
        phys = np.zeros(self.counts.boundary_face_count, np.int32)
        self._chk(self.lib.sdg_boundary_point_coordinate(self.h, _ptr(out), _ptr(phys, _pi)))
        return out, phys

    def adjacency(self):
        ni, nb = self.counts.interior_face_count, self.counts.boundary_face_count
        a = np.zeros((ni, 7), np.int32)
        b = np.zeros((nb, 5), np.int32)
        self._chk(self.lib.sdg_adjacency(self.h, _ptr(a, _pi), _ptr(b, _pi)))
        return a, b

    # state -------------------------------------------------------------------------------------
    def initialize_primitive(self, primitive):
        p = np.ascontiguousarray(primitive, np.float64)
        assert p.shape == (self.counts.volume_point_count, self.nv)
        self._chk(self.lib.sdg_set_initial_primitive(self.h, _ptr(p)))

    def set_boundary_primitive(self, primitive):
        p = np.ascontiguousarray(primitive, np.float64)
        assert p.shape == (self.counts.boundary_point_count, self.nv)
        self._chk(self.lib.sdg_set_boundary_primitive(self.h, _ptr(p)))

    def set_state_point(self, conserved):
        p = np.ascontiguousarray(conserved, np.float64)
        self._chk(self.lib.sdg_set_state_point(self.h, _ptr(p)))

    def state_point(self, out=None):
        if out is None:
            out = np.zeros((self.counts.volume_point_count, self.nv))
        self._chk(self.lib.sdg_get_state_point(self.h, _ptr(out)))
        return out

    def set_state_modal(self, coef):
        p = np.ascontiguousarray(coef, np.float64)
        self._chk(self.lib.sdg_set_state_modal(self.h, _ptr(p)))

    def state_modal(self):
        out = np.zeros(self.counts.degree_of_freedom_count)
        self._chk(self.lib.sdg_get_state_modal(self.h, _ptr(out)))
        return out

    def residual_point(self):
        out = np.zeros((self.counts.volume_point_count, self.nv))
        self._chk(self.lib.sdg_residual_point(self.h, _ptr(out)))
        return out

    # reference Solver<SC> members --------------------------------------------------------------
    def calculateDeltaTime(self, cfl):
        dt = c_double()
        self._chk(self.lib.sdg_calculate_delta_time(self.h, cfl, byref(dt)))
        return dt.value

    def stepSolver(self, dt, steps=1):
        self._chk(self.lib.sdg_step(self.h, steps, dt))
        self._chk(self.lib.sdg_relative_error(self.h, _ptr(self.relative_error_)))
        return self.relative_error_

    def step_state_point(self, dt, out=None):
        """One stepSolver step returning the new state at the volume points (sdg_step_state_point): a pinned
        `out` is filled by the last stage itself on tensor blocks.  Returns (state, relative error)."""
        if out is None:
            out = np.zeros((self.counts.volume_point_count, self.nv))
        self._chk(self.lib.sdg_step_state_point(self.h, dt, _ptr(out), _ptr(self.relative_error_)))
        return out, self.relative_error_

    def step_state_point_from(self, dt, conserved_in, out=None, asynchronous=False):
        """One step from a host state to a host state (sdg_step_state_point_from[_async]).  Synchronous: returns
        (state, relative error).  Asynchronous: enqueues and returns `out`; both buffers stay in use until
        synchronize(), and relative_error() then gives the last call's relative error."""
        p = conserved_in if conserved_in.flags.c_contiguous and conserved_in.dtype == np.float64 else \
            np.ascontiguousarray(conserved_in, np.float64)
        if out is None:
            out = np.zeros((self.counts.volume_point_count, self.nv))
        if asynchronous:
            self._chk(self.lib.sdg_step_state_point_from_async(self.h, dt, _ptr(p), _ptr(out)))
            return out
        self._chk(self.lib.sdg_step_state_point_from(self.h, dt, _ptr(p), _ptr(out), _ptr(self.relative_error_)))
        return out, self.relative_error_

    def step_async(self, dt, steps=1):
        self._chk(self.lib.sdg_step_async(self.h, steps, dt))

    def synchronize(self):
        self._chk(self.lib.sdg_synchronize(self.h))

    def relative_error(self):
        out = np.zeros(self.nv)
        self._chk(self.lib.sdg_relative_error(self.h, _ptr(out)))
        return out

    def launch_count(self):
        n = c_int64()
        self._chk(self.lib.sdg_launch_count(self.h, byref(n)))
        return n.value

    def surface_force(self, physical):
        """Force on boundary group `physical`: sum of w |J_f| (p n - tau n) over its face points."""
        out = np.zeros(self.counts.dimension)
        self._chk(self.lib.sdg_surface_force(self.h, int(physical), _ptr(out)))
        return out

    def surface_force_cotangent(self, physical, direction):
        """d(direction . force)/dU at the volume points (Euler)."""
        d = np.ascontiguousarray(np.asarray(direction, dtype=np.float64).reshape(-1)[: self.counts.dimension])
        out = np.zeros((self.counts.volume_point_count, self.nv))
        self._chk(self.lib.sdg_surface_force_cotangent(self.h, int(physical), _ptr(d), _ptr(out)))
        return out

    def adjoint_boundary_cotangent(self):
        """Cotangent of each boundary point's ghost primitive (rho, u, T) from the last adjoint call (Euler)."""
        out = np.zeros((self.counts.boundary_point_count, self.nv))
        self._chk(self.lib.sdg_adjoint_boundary_cotangent(self.h, _ptr(out)))
        return out

    def node_artificial_viscosity(self):
        """Artificial viscosity of the current state at every mesh node (zeros without shock capturing)."""
        out = np.zeros(len(self.mesh.nodes))
        self._chk(self.lib.sdg_get_node_artificial_viscosity(self.h, _ptr(out)))
        return out

    # raw-binary files ---------------------------------------------------------------------------
    def writeRawBinary(self, path):
        """Solver::writeRawBinary: the reference's zstd raw-binary solution file."""
        self._chk(self.lib.sdg_write_raw_binary(self.h, str(path).encode()))

    def set_boundary_face_order(self, faces):
        """The caller's boundary-face order of the raw-binary boundary block: rows (element type, element index
        within its type, local face), every boundary face once (the reference's adjacency order)."""
        f = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
        self._chk(self.lib.sdg_set_boundary_face_order(self.h, len(f), _ptr(f, _pi)))

    def read_raw_binary(self, path, lower_order=False):
        """Restart from a raw-binary file (LastStep; lower_order: SpecificFile written at order P-1)."""
        self._chk(self.lib.sdg_read_raw_binary(self.h, str(path).encode(), int(bool(lower_order))))

    # launch shapes -----------------------------------------------------------------------------
    def set_graph(self, enable: bool):
        self._chk(self.lib.sdg_set_graph(self.h, int(bool(enable))))

    def tile(self, block=0):
        """(stage elements/CTA, stage threads, gradient elements/CTA, gradient threads) of a block."""
        v = [ctypes.c_int32() for _ in range(4)]
        self._chk(self.lib.sdg_get_tile(self.h, block, *[byref(x) for x in v]))
        return tuple(x.value for x in v)

    def set_tile(self, block, epb, threads, gradient_epb, gradient_threads):
        self._chk(self.lib.sdg_set_tile(self.h, block, epb, threads, gradient_epb, gradient_threads))

    def autotune(self, retime=False):
        self._chk(self.lib.sdg_autotune(self.h, _abi.AUTOTUNE_RETIME if retime else 0))
        return [self.tile(b) for b in range(self.counts.block_count)]

    # derivatives -------------------------------------------------------------------------------
    def _points(self):
        return np.zeros((self.counts.volume_point_count, self.nv))

    def volume_weights(self):
        """w_q |J|_q per volume point (integrals of point values)."""
        w = np.zeros(self.counts.volume_point_count)
        self._chk(self.lib.sdg_volume_point_weight(self.h, _ptr(w)))
        return w

    def set_viscosity(self, mu):
        self._chk(self.lib.sdg_set_viscosity(self.h, float(mu)))
        self.config.dynamic_viscosity = float(mu)

    def jvp_residual(self, tangent, viscosity_tangent=0.0):
        t = np.ascontiguousarray(tangent, np.float64)
        out = self._points()
        self._chk(self.lib.sdg_jvp_residual(self.h, _ptr(t), float(viscosity_tangent), _ptr(out)))
        return out

    def vjp_residual(self, cotangent):
        c = np.ascontiguousarray(cotangent, np.float64)
        out = self._points()
        mu = c_double()
        self._chk(self.lib.sdg_vjp_residual(self.h, _ptr(c), _ptr(out), byref(mu)))
        return out, mu.value

    def jvp_steps(self, dt, steps, tangent, viscosity_tangent=0.0):
        t = np.ascontiguousarray(tangent, np.float64)
        out = self._points()
        self._chk(self.lib.sdg_jvp_steps(self.h, steps, dt, _ptr(t), float(viscosity_tangent), _ptr(out)))
        return out

    def adjoint_steps(self, dt, steps, final_cotangent, checkpoint_interval=25):
        c = np.ascontiguousarray(final_cotangent, np.float64)
        out = self._points()
        mu = c_double()
        self._chk(self.lib.sdg_adjoint_steps(self.h, steps, dt, checkpoint_interval, _ptr(c), _ptr(out), byref(mu)))
        return out, mu.value

    def adjoint_memory(self):
        """Device bytes held by the adjoint's checkpoints, stage states and forward store."""
        b = c_int64()
        self._chk(self.lib.sdg_adjoint_memory(self.h, byref(b)))
        return b.value

    def set_adjoint_trajectory_store(self, enable=True):
        """Keep every stage input of the forward sweep in device memory when it fits, so the reverse sweep
        recomputes no checkpoint interval (sdg_set_adjoint_trajectory_store)."""
        self._chk(self.lib.sdg_set_adjoint_trajectory_store(self.h, 1 if enable else 0))

    def forward_steps(self, dt, steps, checkpoint_interval=25):
        """Advance `steps` steps keeping the checkpoints of the trajectory (for adjoint_recorded)."""
        self._chk(self.lib.sdg_forward_steps(self.h, steps, dt, checkpoint_interval))

    def adjoint_recorded(self, final_cotangent):
        """Reverse sweep of the last forward_steps trajectory (the state must still be its U_N)."""
        c = np.ascontiguousarray(final_cotangent, np.float64)
        out = self._points()
        mu = c_double()
        self._chk(self.lib.sdg_adjoint_recorded(self.h, _ptr(c), _ptr(out), byref(mu)))
        return out, mu.value

    def kinetic_energy(self, state=None, weights=None):
        """J = integral of rho |u|^2 / 2 and dJ/dU in the point layout."""
        u = self.state_point() if state is None else state
        w = self.volume_weights() if weights is None else weights
        d = self.nv - 2
        rho, m = u[:, 0], u[:, 1:1 + d]
        vel = m / rho[:, None]
        J = float(np.sum(w * 0.5 * np.sum(m * vel, 1)))
        g = np.zeros_like(u)
        g[:, 0] = -0.5 * w * np.sum(vel * vel, 1)
        g[:, 1:1 + d] = w[:, None] * vel
        return J, g


class Batch:
    """Many independent GpuSolver instances advanced together (sdg_batch_*): one persistent launch per
    kernel variant and dependency level per RK stage, the step captured in a CUDA graph."""

    def __init__(self, solvers):
        self.lib = _abi.load()
        self.solvers = list(solvers)
        arr = (c_void_p * len(self.solvers))(*[s.h for s in self.solvers])
        b = c_void_p()
        rc = self.lib.sdg_batch_create(arr, len(self.solvers), byref(b))
        check(rc, None)
        self.b = b

    def close(self):
        if getattr(self, "b", None):
            self.lib.sdg_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != _abi.SDG_OK:
            msg = self.lib.sdg_batch_last_error(self.b)
            raise _abi.SdgError(rc, msg.decode() if msg else "")

    def counts(self):
        c = _abi.SdgBatchCounts()
        self._chk(self.lib.sdg_batch_get_counts(self.b, byref(c)))
        return {k: getattr(c, k) for k, _ in c._fields_}

    def set_delta_time(self, dts):
        d = np.ascontiguousarray(dts, np.float64)
        assert d.shape == (len(self.solvers),)
        self._chk(self.lib.sdg_batch_set_delta_time(self.b, _ptr(d)))

    def set_persistence(self, ctas_per_sm):
        self._chk(self.lib.sdg_batch_set_persistence(self.b, ctas_per_sm))

    def step_async(self, steps=1):
        self._chk(self.lib.sdg_batch_step_async(self.b, steps))

    def step_sequential_async(self, steps=1):
        self._chk(self.lib.sdg_batch_step_sequential_async(self.b, steps))

    def synchronize(self):
        self._chk(self.lib.sdg_batch_synchronize(self.b))

    def step(self, steps=1):
        self.step_async(steps)
        self.synchronize()

    def autotune(self, retime=False):
        self._chk(self.lib.sdg_batch_autotune(self.b, _abi.AUTOTUNE_RETIME if retime else 0))

    def stream(self):
        s = c_void_p()
        self._chk(self.lib.sdg_batch_get_stream(self.b, byref(s)))
        return s.value


# InitialConditionEnum (src/Utils/Enum.cpp): the driver's function, a given raw-binary file, or the last written
# step of the same run (raw/{prefix}_{iteration_start}.zst)
INITIAL_FUNCTION, INITIAL_SPECIFIC_FILE, INITIAL_LAST_STEP = 0, 1, 2
# BoundaryTimeEnum (src/Utils/Enum.cpp:102-105)
BOUNDARY_STEADY, BOUNDARY_TIME_VARYING = 0, 1


class System:
    """Mirror of SubrosaDG's System<SimulationControl> (src/Utils/SystemControl.cpp:42-236): setup, then solve()
    with the reference's outputs -- raw/{prefix}_{i}.zst every io_interval steps (and step 0) and error.txt with
    one line of relative errors per step (SystemControl.cpp:159-195, View/CommandLine.cpp:95-150,
    View/IOControl.cpp:318-337)."""

    def __init__(self, dimension, polynomial_order, equation=_abi.EULER, convective_flux=_abi.HLLC,
                 viscous_flux=_abi.VISCOUS_NONE, time_integration=_abi.SSPRK3, device=0,
                 initial_condition_kind=INITIAL_FUNCTION, boundary_time=BOUNDARY_STEADY):
        self.dimension = dimension
        self.boundary_time = boundary_time  # SolveControl's BoundaryTimeEnum
        self.cfg = dict(polynomial_order=polynomial_order, equation=equation, convective_flux=convective_flux,
                        viscous_flux=viscous_flux, time_integration=time_integration)
        self.device = device
        self.mesh = None
        self.cfl = 1.0
        self.iteration_start, self.iteration_end = 0, 0
        self.delta_time = 0.0
        self.solver = None
        self.initial_condition = None   # callable(coords[n,3]) -> primitive[n, d+2]
        # callable(coords[n,3], physical[n]) -> primitive[n, d+2]; with BOUNDARY_TIME_VARYING
        # callable(coords[n,3], time, physical[n]) (the reference's TimeVarying signature)
        self.boundary_condition = None
        self.initial_condition_kind = initial_condition_kind
        self.initial_condition_file = None
        self.initial_condition_lower_order = False
        self.output_directory = None    # setViewConfig: raw/ files and error.txt (no outputs when unset)
        self.output_file_name_prefix = ""
        self.io_interval = 0
        self.error_history = []

    def setMesh(self, mesh: Mesh):
        self.mesh = mesh

    def addBoundaryCondition(self, condition, physical_index):
        self.mesh.set_boundary_condition(physical_index, condition)

    def setThermodynamicModel(self, cp, cv):
        self.cfg.update(cp=cp, cv=cv)

    def setTransportModel(self, mu, transport=_abi.TRANSPORT_CONSTANT, prandtl=0.71):
        self.cfg.update(mu=mu, transport=transport, prandtl=prandtl)

    def setEquationOfState(self, reference_sound_speed, reference_density):
        """Weakly compressible fluid of the incompressible models (PhysicalModel.cpp:57-78)."""
        self.cfg.update(sound_speed=reference_sound_speed, density=reference_density)

    def setSourceTerm(self, thermal_expansion_coefficient, reference_temperature):
        """Boussinesq buoyancy (SourceTerm.cpp:29-58)."""
        self.cfg.update(source=_abi.SOURCE_BOUSSINESQ, thermal_expansion=thermal_expansion_coefficient,
                        reference_temperature=reference_temperature)

    def setArtificialViscosity(self, empirical_tolerance, artificial_viscosity_factor=1.0):
        """Shock capturing (SystemControl.cpp:105-108)."""
        self.cfg.update(shock_capturing=_abi.ARTIFICIAL_VISCOSITY, empirical_tolerance=empirical_tolerance,
                        artificial_viscosity_factor=artificial_viscosity_factor)

    def addInitialCondition(self, raw_binary_path, lower_order=False):
        """InitialConditionEnum::SpecificFile (SystemControl.cpp:70-74): the state of a raw-binary file (of the
        order below with lower_order, InitialCondition.cpp:58-80)."""
        self.initial_condition_kind = INITIAL_SPECIFIC_FILE
        self.initial_condition_file = raw_binary_path
        self.initial_condition_lower_order = lower_order

    def setTimeIntegration(self, cfl, iteration_range):
        self.cfl = cfl
        self.iteration_start, self.iteration_end = iteration_range

    def setViewConfig(self, output_directory, output_file_name_prefix, io_interval=-1):
        """Output directory, file prefix and raw-binary interval (SystemControl.cpp:124-140; -1 or 0: the last
        step only, where the reference asks on stdin for 0)."""
        self.output_directory = os.fspath(output_directory)
        self.output_file_name_prefix = output_file_name_prefix
        self.io_interval = self.iteration_end if io_interval in (0, -1) else int(io_interval)

    def setDeltaTime(self, dt):
        self.delta_time = dt

    def synchronize(self):
        self.solver = GpuSolver(self.mesh, make_config(**self.cfg), self.device)

    def _boundary_primitive(self, pts, physical, time):
        if self.boundary_time == BOUNDARY_TIME_VARYING:
            return self.boundary_condition(pts, time, physical)
        return self.boundary_condition(pts, physical)

    def _raw_path(self, step):
        return os.path.join(self.output_directory, "raw", f"{self.output_file_name_prefix}_{step}.zst")

    def _variable_list(self):
        """error.txt header (View/CommandLine.cpp:70-93)."""
        d = self.dimension
        incomp = self.cfg["equation"] in (_abi.INCOMPRESSIBLE_EULER, _abi.INCOMPRESSIBLE_NAVIER_STOKES)
        names = ["Time", "rho"] + ["rho*" + c for c in "uvw"[:d]] + ["rho*e" if incomp else "rho*E"]
        return "".join(f"|{n:^13}" for n in names) + "|"

    @staticmethod
    def _line(time_value, error):
        """One error.txt line (View/CommandLine.cpp:95-106): {:^13.5e} fields."""
        return "".join(f"|{x:^13.5e}" for x in [time_value, *error]) + "|"

    def solve(self, delete_dir=True):
        s = self.solver
        last_step = self.initial_condition_kind == INITIAL_LAST_STEP
        error_lines = None
        if self.output_directory is not None:  # View::initializeSolverFinout (IOControl.cpp:318-335)
            raw = os.path.join(self.output_directory, "raw")
            if delete_dir and not last_step and os.path.isdir(raw):
                shutil.rmtree(raw)
            os.makedirs(raw, exist_ok=True)
            error_path = os.path.join(self.output_directory, "error.txt")
            if last_step and os.path.exists(error_path):  # keep the header, the zero line and the steps done
                with open(error_path) as f:
                    error_lines = f.read().splitlines()[: self.iteration_start + 2]
            else:
                error_lines = []
        if self.initial_condition_kind == INITIAL_SPECIFIC_FILE:
            s.read_raw_binary(self.initial_condition_file, lower_order=self.initial_condition_lower_order)
        elif last_step:
            s.read_raw_binary(self._raw_path(self.iteration_start))
        else:
            pts = s.volume_points()
            s.initialize_primitive(self.initial_condition(pts[:, : self.dimension]))
        bpts = bphys = None
        if s.counts.boundary_face_count:
            bpts, phys = s.boundary_points()
            bpts, bphys = bpts[:, : self.dimension], np.repeat(phys, s.counts.face_point_count)
            s.set_boundary_primitive(self._boundary_primitive(bpts, bphys, 0.0))
        if self.delta_time == 0.0:
            self.delta_time = s.calculateDeltaTime(self.cfl)
        error_file = None
        if error_lines is not None:  # error.txt is written line by line as the reference's error_finout is
            error_file = open(os.path.join(self.output_directory, "error.txt"), "w")
            for line in error_lines:
                error_file.write(line + "\n")
            if not last_step:
                s.writeRawBinary(self._raw_path(0))
                error_file.write(self._variable_list() + "\n" + self._line(0.0, np.zeros(s.nv)) + "\n")
        io_interval = self.io_interval or self.iteration_end
        iteration = 0  # TimeIntegration::iteration_ (TimeIntegration.cpp:37): 0 until a step has been taken
        try:
            for i in range(self.iteration_start + 1, self.iteration_end + 1):
                if self.boundary_time == BOUNDARY_TIME_VARYING and bpts is not None:
                    # Solver::updateBoundaryVariable at the start of each step, at time iteration_ * dt
                    # (TimeIntegration.cpp:333-335, BoundaryCondition.cpp:29-74)
                    s.set_boundary_primitive(self._boundary_primitive(bpts, bphys, iteration * self.delta_time))
                err = s.stepSolver(self.delta_time).copy()
                iteration = i
                self.error_history.append((i * self.delta_time, err))
                if error_file is not None:
                    if i % io_interval == 0:
                        s.writeRawBinary(self._raw_path(i))
                    error_file.write(self._line(i * self.delta_time, err) + "\n")
                    error_file.flush()
                if np.isnan(err).all():  # src/Utils/SystemControl.cpp:185-191
                    if io_interval == self.iteration_end:
                        io_interval = i
                    self.iteration_end = i
                    break
        finally:
            if error_file is not None:
                error_file.close()
        self.io_interval = io_interval
        return self.error_history
