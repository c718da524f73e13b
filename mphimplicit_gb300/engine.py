"""Python access to the GB300 engine through its C ABI (include/mph_gb300.h).

``Case`` mirrors the reference solver's run: create from a `.data` parameter
set and a `.grid` particle set (source/main.cpp:347-375), advance with
``step`` (the body of main.cpp:386-474) or stage by stage, and write `.vtk` /
`.prof` frames.  The CUDA library is required: there is no CPU fallback, and
loading fails loudly when libmph_gb300.so has not been built.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional

import numpy as np

from . import casegen
from .cabi import (MphFields, MphParams, MphParticles, MphSolveStats, ParticlesC, ERR_NAMES, PRECISION_FP64,
                   PRECISION_MIXED, np_ptr, params_from_c, params_to_c)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmph_gb300.so")

_lib = None


class MphError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(status, status)}: {msg}")
        self.status = status


def load_library(path: str = LIB_PATH):
    """Load libmph_gb300.so and declare the C ABI."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"GB300 engine library not built: {path} (run mphimplicit_gb300.build.build())")
    lib = ctypes.CDLL(path)
    vp, ip, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p
    sig = {
        "mph_read_data": ([cp, vp], ip),
        "mph_read_grid": ([cp, vp], ip),
        "mph_write_prof": ([cp, vp], ip),
        "mph_case_write_vtk": ([vp, cp], ip),
        "mph_case_write_prof": ([vp, cp], ip),
        "mph_write_checkpoint": ([cp, vp, vp], ip),
        "mph_read_checkpoint": ([cp, vp, vp], ip),
        "mph_case_checkpoint": ([vp, cp], ip),
        "mph_case_create": ([vp, vp, ip, ip, vp, ctypes.POINTER(vp)], ip),
        "mph_case_destroy": ([vp], ip),
        "mph_case_set_stream": ([vp, vp], ip),
        "mph_step": ([vp, ip], ip),
        "mph_batch_step": ([ctypes.POINTER(vp), ip, ip], ip),
        "mph_case_count": ([vp, ctypes.POINTER(ip), ctypes.POINTER(ip)], ip),
        "mph_case_time": ([vp, ctypes.POINTER(ctypes.c_double)], ip),
        "mph_get_fields": ([vp, vp], ip),
        "mph_get_solve_stats": ([vp, vp], ip),
        "mph_case_set_state": ([vp, vp, vp], ip),
        "mph_export": ([vp, cp, vp, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ip)], ip),
        "mph_scalars": ([vp, ctypes.POINTER(ctypes.c_double), ip], ip),
        "mph_scalar_names": ([], cp),
        "mph_case_profile": ([vp, ip], ip),
        "mph_case_set_solver": ([vp, ctypes.c_double, ctypes.c_double, ip], ip),
        "mph_case_set_option": ([vp, cp, ctypes.c_double], ip),
        "mph_case_profile_read": ([vp, ctypes.POINTER(ctypes.c_double), ip], ip),
        "mph_launch_count": ([], ctypes.c_longlong),
        "mph_last_error": ([], cp),
        "mph_version": ([], cp),
    }
    for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build", "solve", "step_end", "output_fields"):
        sig["mph_stage_" + st] = ([vp], ip)
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _check(status: int):
    if status != 0:
        raise MphError(status, load_library().mph_last_error().decode())


_KIND = {0: np.int32, 1: np.int64, 2: np.float64}


def read_data(path: str) -> casegen.Params:
    p = MphParams()
    _check(load_library().mph_read_data(path.encode(), ctypes.byref(p)))
    return params_from_c(p)


def read_grid(path: str) -> casegen.Particles:
    lib = load_library()
    s = MphParticles()
    _check(lib.mph_read_grid(path.encode(), ctypes.byref(s)))
    n = s.count
    types = np.zeros(n, np.int32)
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    s.type = np_ptr(types, ctypes.c_int)
    s.pos = np_ptr(pos)
    s.vel = np_ptr(vel)
    _check(lib.mph_read_grid(path.encode(), ctypes.byref(s)))
    return casegen.Particles(s.time, s.spacing, np.array(s.domain_min[:]), np.array(s.domain_max[:]), types, pos, vel)


def write_checkpoint(path: str, parts: casegen.Particles, ids: Optional[np.ndarray] = None,
                     wall_center: Optional[np.ndarray] = None):
    """Full-precision checkpoint sidecar of a particle state."""
    ps = ParticlesC(parts, ids)
    wc = None if wall_center is None else np.ascontiguousarray(wall_center, dtype=np.float64).reshape(-1)
    _check(load_library().mph_write_checkpoint(path.encode(), ctypes.byref(ps.struct),
                                               None if wc is None else wc.ctypes.data_as(ctypes.c_void_p)))


def read_checkpoint(path: str):
    """(particles, ids, wall_center[4][3]) of a checkpoint file."""
    lib = load_library()
    s = MphParticles()
    _check(lib.mph_read_checkpoint(path.encode(), ctypes.byref(s), None))
    n = s.count
    types = np.zeros(n, np.int32)
    ids = np.zeros(n, np.int32)
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    wc = np.zeros((4, 3))
    s.type = np_ptr(types, ctypes.c_int)
    s.id = np_ptr(ids, ctypes.c_int)
    s.pos = np_ptr(pos)
    s.vel = np_ptr(vel)
    _check(lib.mph_read_checkpoint(path.encode(), ctypes.byref(s), wc.ctypes.data_as(ctypes.c_void_p)))
    parts = casegen.Particles(s.time, s.spacing, np.array(s.domain_min[:]), np.array(s.domain_max[:]), types, pos, vel)
    return parts, ids, wc


class Case:
    """One simulation case resident on the GPU."""

    def __init__(self, params: casegen.Params, parts: casegen.Particles, dim: int,
                 precision: int = PRECISION_FP64, stream: Optional[int] = None, ids: Optional[np.ndarray] = None):
        self.lib = load_library()
        self.dim = dim
        self._p = params_to_c(params)
        self._parts = ParticlesC(parts, ids)
        h = ctypes.c_void_p()
        _check(self.lib.mph_case_create(ctypes.byref(self._p), ctypes.byref(self._parts.struct), dim, precision,
                                        ctypes.c_void_p(stream or 0), ctypes.byref(h)))
        self.h = h
        n, nf = ctypes.c_int(), ctypes.c_int()
        self.lib.mph_case_count(self.h, ctypes.byref(n), ctypes.byref(nf))
        self.count, self.fluid_count = n.value, nf.value

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.mph_case_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # whole steps and stages -------------------------------------------------
    def step(self, n: int = 1) -> int:
        st = self.lib.mph_step(self.h, n)
        if st not in (0, 7):
            _check(st)
        return st

    def stage(self, name: str):
        _check(getattr(self.lib, "mph_stage_" + name)(self.h))

    def set_stream(self, stream: int):
        _check(self.lib.mph_case_set_stream(self.h, ctypes.c_void_p(stream)))

    # state ----------------------------------------------------------------------
    def export(self, name: str) -> np.ndarray:
        cnt, kind = ctypes.c_long(), ctypes.c_int()
        _check(self.lib.mph_export(self.h, name.encode(), None, ctypes.byref(cnt), ctypes.byref(kind)))
        out = np.empty(cnt.value, dtype=_KIND[kind.value])
        _check(self.lib.mph_export(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(cnt), ctypes.byref(kind)))
        return out

    def scalars(self) -> Dict[str, float]:
        buf = (ctypes.c_double * 64)()
        _check(self.lib.mph_scalars(self.h, buf, 64))
        names = self.lib.mph_scalar_names().decode().split(",")
        return dict(zip(names, list(buf)[:len(names)]))

    def solve_stats(self) -> Dict[str, float]:
        s = MphSolveStats()
        _check(self.lib.mph_get_solve_stats(self.h, ctypes.byref(s)))
        return {"iter": s.iterations, "rr0": s.rr0, "rr": s.rr, "rs0": s.rs0, "rs": s.rs, "status": s.status,
                "outer": s.outer_iterations, "inner_form": s.inner_form,
                "inner_local_blocks": s.inner_local_blocks, "inner_gather_blocks": s.inner_gather_blocks,
                "inner_local_cols": s.inner_local_cols, "inner_ct_local_blocks": s.inner_ct_local_blocks}

    def set_solver(self, outer_rel_residual: float = 1e-6, inner_rel_residual: float = 1e-3, max_outer: int = 50):
        _check(self.lib.mph_case_set_solver(self.h, outer_rel_residual, inner_rel_residual, max_outer))

    def set_option(self, name: str, value: float):
        _check(self.lib.mph_case_set_option(self.h, name.encode(), float(value)))

    def time(self) -> float:
        t = ctypes.c_double()
        _check(self.lib.mph_case_time(self.h, ctypes.byref(t)))
        return t.value

    def fields(self, which=None, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        """Per-particle fields (cell order) copied to host; `which` selects a
        subset of id, type, pos, vel, force, vol_strain_p, divergence_p,
        pressure_p, virial_p, neighbor_count.  `out` supplies the buffers
        (contiguous, int32 / float64 of the field's shape; pinned host memory
        takes the copies at link speed)."""
        n = self.count
        if out is None:
            out = {"id": np.empty(n, np.int32), "type": np.empty(n, np.int32), "pos": np.empty((n, 3)), "vel": np.empty((n, 3)),
                   "force": np.empty((n, 3)), "vol_strain_p": np.empty(n), "divergence_p": np.empty(n),
                   "pressure_p": np.empty(n), "virial_p": np.empty(n), "neighbor_count": np.empty(n, np.int32)}
            if which is not None:
                out = {k: v for k, v in out.items() if k in which}
        else:
            for k, a in out.items():
                want = (n,) if k in ("id", "type", "neighbor_count", "vol_strain_p", "divergence_p", "pressure_p", "virial_p") else (n, 3)
                dt = np.int32 if k in ("id", "type", "neighbor_count") else np.float64
                if a.shape != want or a.dtype != dt or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"fields: buffer {k} must be a contiguous {np.dtype(dt).name} array of shape {want}")
        f = MphFields()
        for k, a in out.items():
            setattr(f, k, np_ptr(a, ctypes.c_int if a.dtype == np.int32 else ctypes.c_double))
        _check(self.lib.mph_get_fields(self.h, ctypes.byref(f)))
        return out

    def set_state(self, parts: casegen.Particles, ids: Optional[np.ndarray] = None,
                  wall_center: Optional[np.ndarray] = None):
        ps = ParticlesC(parts, ids)
        wc = None if wall_center is None else np.ascontiguousarray(wall_center, dtype=np.float64).reshape(-1)
        _check(self.lib.mph_case_set_state(self.h, ctypes.byref(ps.struct),
                                           None if wc is None else wc.ctypes.data_as(ctypes.c_void_p)))

    def profile(self, enable: bool = True):
        _check(self.lib.mph_case_profile(self.h, 1 if enable else 0))

    def profile_read(self) -> Dict[str, float]:
        buf = (ctypes.c_double * 32)()
        n = self.lib.mph_case_profile_read(self.h, buf, 32)
        if n < 0 or n > 32:
            _check(n)
        v = list(buf)
        stages = ["step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build", "solve"]
        kern = ["spmv", "precond", "assemble_a", "neighbors"]
        out = {f"stage_ms_{s}": v[k] for k, s in enumerate(stages)}
        out.update({f"kern_ms_{s}": v[7 + k] for k, s in enumerate(kern)})
        out.update({f"kern_n_{s}": int(v[11 + k]) for k, s in enumerate(kern)})
        out.update({"slots": int(v[15]), "nnb": int(v[16]), "nnbP": int(v[17])})
        return out

    def checkpoint(self, path: str):
        _check(self.lib.mph_case_checkpoint(self.h, path.encode()))

    @classmethod
    def restore(cls, params: casegen.Params, path: str, dim: int, precision: int = PRECISION_FP64,
                stream: Optional[int] = None) -> "Case":
        """A case continuing from a checkpoint: created from the stored
        particles (ids included), then given the stored order, wall centres
        and time."""
        parts, ids, wc = read_checkpoint(path)
        c = cls(params, parts, dim, precision=precision, stream=stream, ids=ids)
        c.set_state(parts, ids, wc)
        return c

    def write_vtk(self, path: str):
        _check(self.lib.mph_case_write_vtk(self.h, path.encode()))

    def write_prof(self, path: str):
        _check(self.lib.mph_case_write_prof(self.h, path.encode()))


def launch_count() -> int:
    return int(load_library().mph_launch_count())


def batch_step(cases, nsteps: int = 1) -> int:
    lib = load_library()
    arr = (ctypes.c_void_p * len(cases))(*[c.h.value for c in cases])
    st = lib.mph_batch_step(arr, len(cases), nsteps)
    if st not in (0, 7):
        _check(st)
    return st
