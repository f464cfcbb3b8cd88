"""ctypes wrapper of the oracle (oracle/liborc.so) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker / the timed CPU baseline.  The product path
(subrosadg_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, byref, c_double, c_int, c_int32, c_int64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBS = {"double": os.path.join(HERE, "liborc.so"), "extended": os.path.join(HERE, "liborc_ext.so")}
_pd = POINTER(c_double)
_pi = POINTER(c_int32)
_libs = {}


def load(precision="double"):
    if precision not in _libs:
        path = LIBS[precision]
        if not os.path.exists(path):
            from . import build as _build
            _build.build()
        lib = ctypes.CDLL(path)
        lib.orc_create.restype = c_void_p
        lib.orc_create.argtypes = [c_void_p, c_void_p, c_int]
        lib.orc_create_sampled.restype = c_void_p
        lib.orc_create_sampled.argtypes = [c_void_p, c_void_p, c_int, c_int64, POINTER(c_int64)]
        lib.orc_last_error.restype = ctypes.c_char_p
        lib.orc_destroy.argtypes = [c_void_p]
        for name in ("orc_volume_point_coordinate", "orc_set_initial_primitive", "orc_set_state_point",
                     "orc_set_boundary_primitive", "orc_get_state_point", "orc_get_state_modal",
                     "orc_relative_error", "orc_residual_point", "orc_interior_face_geometry"):
            getattr(lib, name).argtypes = [c_void_p, _pd]
            getattr(lib, name).restype = c_int
        lib.orc_node_artificial_viscosity.argtypes = [c_void_p, _pd]
        lib.orc_node_artificial_viscosity.restype = c_int
        lib.orc_boundary_point_coordinate.argtypes = [c_void_p, _pd, _pi]
        lib.orc_counts.argtypes = [c_void_p, POINTER(c_int64)]
        lib.orc_calculate_delta_time.argtypes = [c_void_p, c_double, _pd]
        lib.orc_step.argtypes = [c_void_p, c_int, c_double]
        lib.orc_stage.argtypes = [c_void_p, c_int, c_double]
        lib.orc_adjacency.argtypes = [c_void_p, _pi, _pi]
        lib.orc_raw_gradient.argtypes = [c_void_p, _pd, _pd]
        lib.orc_set_threads.argtypes = [c_int]
        lib.orc_max_threads.restype = c_int
        lib.orc_real_digits.restype = c_int
        _libs[precision] = lib
    return _libs[precision]


class Oracle:
    """CPU restatement of the reference solver on the same mesh/config structs as sdg_create.

    faithful=True : the reference's arithmetic -- gradient pass also for Euler, plain explicit inverses
                    (the reference-faithful timed CPU baseline);
    faithful=False: the checker -- no unused gradient pass, solves refined by one correction step.
    lean=True     : the lean timed CPU baseline -- no unused Euler gradient pass, plain inverses, one shared
                    reference inverse scaled by 1/|J| on blocks of affine elements (overrides faithful).
    precision     : "double" (the reference's Real) or "extended" (long double truth).
    sample        : global element indices (block order): evaluate the residual of these elements only (the
                    element-sample mode for meshes too large for the extended build; residual_point is zero
                    elsewhere; stepping is refused).
    """

    def __init__(self, mesh, config, faithful=True, precision="double", lean=False, sample=None):
        self.lib = load(precision)
        self._m = mesh.struct()
        self._c = config
        flags = 6 if lean else (3 if faithful else 0)
        if sample is None:
            self.h = self.lib.orc_create(ctypes.addressof(self._m), ctypes.addressof(self._c), flags)
        else:
            self._sample = np.ascontiguousarray(sample, np.int64)
            self.h = self.lib.orc_create_sampled(ctypes.addressof(self._m), ctypes.addressof(self._c), flags,
                                                 len(self._sample), self._sample.ctypes.data_as(POINTER(c_int64)))
        if not self.h:
            raise RuntimeError("oracle: " + self.lib.orc_last_error().decode())
        c = (c_int64 * 6)()
        self.lib.orc_counts(self.h, c)
        self.elements, self.volume_points_count, self.interior, self.boundary, self.nfq, self.dof = list(c)
        self.nv = mesh.dimension + 2
        self.node_count = len(mesh.nodes)

    def node_artificial_viscosity(self):
        """Artificial viscosity of the current state at the mesh nodes (zeros without shock capturing)."""
        out = np.zeros(self.node_count)
        self.lib.orc_node_artificial_viscosity(self.h, out.ctypes.data_as(_pd))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def volume_points(self):
        out = np.zeros((self.volume_points_count, 3))
        self.lib.orc_volume_point_coordinate(self.h, out.ctypes.data_as(_pd))
        return out

    def boundary_points(self):
        out = np.zeros((self.boundary * self.nfq, 3))
        phys = np.zeros(self.boundary, np.int32)
        self.lib.orc_boundary_point_coordinate(self.h, out.ctypes.data_as(_pd), phys.ctypes.data_as(_pi))
        return out, phys

    def initialize_primitive(self, prim):
        p = np.ascontiguousarray(prim, np.float64)
        self.lib.orc_set_initial_primitive(self.h, p.ctypes.data_as(_pd))

    def set_state_point(self, cons):
        p = np.ascontiguousarray(cons, np.float64)
        self.lib.orc_set_state_point(self.h, p.ctypes.data_as(_pd))

    def set_boundary_primitive(self, prim):
        p = np.ascontiguousarray(prim, np.float64)
        self.lib.orc_set_boundary_primitive(self.h, p.ctypes.data_as(_pd))

    def state_point(self):
        out = np.zeros((self.volume_points_count, self.nv))
        self.lib.orc_get_state_point(self.h, out.ctypes.data_as(_pd))
        return out

    def state_modal(self):
        out = np.zeros(self.dof)
        self.lib.orc_get_state_modal(self.h, out.ctypes.data_as(_pd))
        return out

    def residual_point(self):
        out = np.zeros((self.volume_points_count, self.nv))
        self.lib.orc_residual_point(self.h, out.ctypes.data_as(_pd))
        return out

    def step(self, dt, n=1):
        self.lib.orc_step(self.h, n, dt)

    def stage(self, stage, dt):
        """One RK stage (stage 0 also saves U^n as the step's base state, as a step does first)."""
        self.lib.orc_stage(self.h, stage, dt)

    def relative_error(self):
        out = np.zeros(self.nv)
        self.lib.orc_relative_error(self.h, out.ctypes.data_as(_pd))
        return out

    def delta_time(self, cfl):
        dt = c_double()
        self.lib.orc_calculate_delta_time(self.h, cfl, byref(dt))
        return dt.value

    def adjacency(self):
        a = np.zeros((self.interior, 7), np.int32)
        b = np.zeros((self.boundary, 5), np.int32)
        self.lib.orc_adjacency(self.h, a.ctypes.data_as(_pi), b.ctypes.data_as(_pi))
        return a, b

    def raw_gradient(self, element_values, boundary_values):
        """Navier-Stokes gradient records of the reference's raw-binary file: per element (block order) and per
        boundary face (sorted adjacency order) -- BR2: the volume gradient plus that face's lift."""
        e = np.zeros(element_values)
        b = np.zeros(boundary_values)
        if self.lib.orc_raw_gradient(self.h, e.ctypes.data_as(_pd), b.ctypes.data_as(_pd)) != 0:
            raise RuntimeError("oracle: raw gradients need a Navier-Stokes problem")
        return e, b

    def interior_face_geometry(self):
        out = np.zeros((self.interior, self.nfq, 4))
        self.lib.orc_interior_face_geometry(self.h, out.ctypes.data_as(_pd))
        return out


def set_threads(n, precision="double"):
    load(precision).orc_set_threads(int(n))


def max_threads():
    return load().orc_max_threads()
