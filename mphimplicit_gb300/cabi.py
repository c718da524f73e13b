"""ctypes mirror of the C ABI structs in include/mph_gb300.h.

The structs carry the `.data` keyword parameters (reference source/main.cpp:
523-563) and the `.grid` particle set (source/main.cpp:565-669)."""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from . import casegen

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)

MPH_OK = 0
ERR_NAMES = {
    0: "MPH_OK", 1: "MPH_ERR_ARG", 2: "MPH_ERR_IO", 3: "MPH_ERR_INPUT", 4: "MPH_ERR_CUDA",
    5: "MPH_ERR_NOMEM", 6: "MPH_ERR_CAPACITY", 7: "MPH_ERR_NOT_CONVERGED", 8: "MPH_ERR_NAN",
    9: "MPH_ERR_STATE",
}
PRECISION_FP64 = 0
PRECISION_MIXED = 1


class MphParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("output_interval", ctypes.c_double),
        ("vtk_output_interval", ctypes.c_double),
        ("end_time", ctypes.c_double),
        ("radius_ratio_a", ctypes.c_double),
        ("radius_ratio_p", ctypes.c_double),
        ("radius_ratio_v", ctypes.c_double),
        ("density", ctypes.c_double * 4),
        ("bulk_modulus", ctypes.c_double * 4),
        ("bulk_viscosity", ctypes.c_double * 4),
        ("shear_viscosity", ctypes.c_double * 4),
        ("surface_tension", ctypes.c_double * 4),
        ("interaction_ratio", (ctypes.c_double * 4) * 4),
        ("gravity", ctypes.c_double * 3),
        ("wall_center", (ctypes.c_double * 3) * 4),
        ("wall_velocity", (ctypes.c_double * 3) * 4),
        ("wall_omega", (ctypes.c_double * 3) * 4),
    ]


class MphParticles(ctypes.Structure):
    _fields_ = [
        ("count", ctypes.c_int),
        ("time", ctypes.c_double),
        ("spacing", ctypes.c_double),
        ("domain_min", ctypes.c_double * 3),
        ("domain_max", ctypes.c_double * 3),
        ("type", c_int_p),
        ("pos", c_double_p),
        ("vel", c_double_p),
        ("id", c_int_p),
    ]


class MphFields(ctypes.Structure):
    _fields_ = [
        ("id", c_int_p), ("type", c_int_p), ("pos", c_double_p), ("vel", c_double_p),
        ("force", c_double_p), ("vol_strain_p", c_double_p), ("divergence_p", c_double_p),
        ("pressure_p", c_double_p), ("virial_p", c_double_p), ("neighbor_count", c_int_p),
    ]


class MphSolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("rr0", ctypes.c_double), ("rr", ctypes.c_double),
                ("rs0", ctypes.c_double), ("rs", ctypes.c_double), ("status", ctypes.c_int),
                ("outer_iterations", ctypes.c_int), ("inner_form", ctypes.c_int),
                ("inner_local_blocks", ctypes.c_int), ("inner_gather_blocks", ctypes.c_int),
                ("inner_local_cols", ctypes.c_longlong), ("inner_ct_local_blocks", ctypes.c_int),
                ("inner_reserved", ctypes.c_int)]


def params_to_c(p: casegen.Params) -> MphParams:
    c = MphParams()
    c.dt, c.output_interval, c.vtk_output_interval, c.end_time = p.dt, p.output_interval, p.vtk_output_interval, p.end_time
    c.radius_ratio_a, c.radius_ratio_p, c.radius_ratio_v = p.radius_ratio_a, p.radius_ratio_p, p.radius_ratio_v
    for t in range(4):
        c.density[t] = p.density[t]
        c.bulk_modulus[t] = p.bulk_modulus[t]
        c.bulk_viscosity[t] = p.bulk_viscosity[t]
        c.shear_viscosity[t] = p.shear_viscosity[t]
        c.surface_tension[t] = p.surface_tension[t]
        for u in range(4):
            c.interaction_ratio[t][u] = p.interaction_ratio[t][u]
    for d in range(3):
        c.gravity[d] = p.gravity[d]
    for t, w in ((2, p.wall2), (3, p.wall3)):
        for d in range(3):
            c.wall_center[t][d] = w[d]
            c.wall_velocity[t][d] = w[3 + d]
            c.wall_omega[t][d] = w[6 + d]
    return c


def params_from_c(c: MphParams) -> casegen.Params:
    w = lambda t: tuple(list(c.wall_center[t]) + list(c.wall_velocity[t]) + list(c.wall_omega[t]))
    return casegen.Params(
        dt=c.dt, output_interval=c.output_interval, vtk_output_interval=c.vtk_output_interval,
        end_time=c.end_time, radius_ratio_a=c.radius_ratio_a, radius_ratio_p=c.radius_ratio_p,
        radius_ratio_v=c.radius_ratio_v, density=tuple(c.density), bulk_modulus=tuple(c.bulk_modulus),
        bulk_viscosity=tuple(c.bulk_viscosity), shear_viscosity=tuple(c.shear_viscosity),
        surface_tension=tuple(c.surface_tension),
        interaction_ratio=tuple(tuple(c.interaction_ratio[t]) for t in range(4)),
        gravity=tuple(c.gravity), wall2=w(2), wall3=w(3))


class ParticlesC:
    """Holds numpy buffers alive behind an MphParticles struct."""

    def __init__(self, parts: casegen.Particles, ids: Optional[np.ndarray] = None):
        self.types = np.ascontiguousarray(parts.types, dtype=np.int32)
        self.pos = np.ascontiguousarray(parts.pos, dtype=np.float64)
        self.vel = np.ascontiguousarray(parts.vel, dtype=np.float64)
        self.ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        s = MphParticles()
        s.count = parts.count
        s.time = parts.time
        s.spacing = parts.spacing
        for d in range(3):
            s.domain_min[d] = parts.domain_min[d]
            s.domain_max[d] = parts.domain_max[d]
        s.type = self.types.ctypes.data_as(c_int_p)
        s.pos = self.pos.ctypes.data_as(c_double_p)
        s.vel = self.vel.ctypes.data_as(c_double_p)
        s.id = self.ids.ctypes.data_as(c_int_p) if self.ids is not None else None
        self.struct = s


def np_ptr(a: np.ndarray, ctype=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ctype))
