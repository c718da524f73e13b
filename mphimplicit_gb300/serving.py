"""Serving loop and batched stepping through the C ABI.

``Server`` wraps mph_server_*: cases are submitted as they arrive, admitted
in arrival order while their device-memory footprint (mph_case_footprint)
fits the budget, kept resident, and stepped concurrently with every other
admitted case, each on its own stream; a finished case frees its memory for
the next waiting one.  Results carry the final fields, every step's latency
and the submit / admit / completion times.  The reference has no serving or
batching layer (it runs one case per process, source/main.cpp:313-474).
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional

import numpy as np

from . import casegen
from .cabi import MphFields, ParticlesC, PRECISION_FP64, params_to_c, np_ptr
from .engine import _check, load_library


class MphServerResult(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_longlong), ("status", ctypes.c_int), ("steps", ctypes.c_int),
                ("particles", ctypes.c_int), ("pad", ctypes.c_int), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double), ("footprint_bytes", ctypes.c_longlong),
                ("error", ctypes.c_char * 128)]


class MphServerStats(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_longlong), ("used_bytes", ctypes.c_longlong), ("pending", ctypes.c_int),
                ("active", ctypes.c_int), ("finished", ctypes.c_int), ("pad", ctypes.c_int), ("steps", ctypes.c_longlong),
                ("particle_steps", ctypes.c_double), ("elapsed_s", ctypes.c_double)]


def _lib():
    lib = load_library()
    if not getattr(lib, "_mph_serving_declared", False):
        vp, ip = ctypes.c_void_p, ctypes.c_int
        decl = {
            "mph_case_footprint": ([vp, vp, ip, ip, ctypes.POINTER(ctypes.c_longlong)], ip),
            "mph_batch_step_workers": ([ctypes.POINTER(vp), ip, ip, ip], ip),
            "mph_server_create": ([ctypes.c_longlong, ip, ip, ctypes.POINTER(vp)], ip),
            "mph_server_submit": ([vp, vp, vp, ip, ip, ip, vp, vp, ctypes.POINTER(ctypes.c_longlong)], ip),
            "mph_server_poll": ([vp, ctypes.POINTER(MphServerResult), ip, ip, ctypes.POINTER(ip)], ip),
            "mph_server_stats_get": ([vp, ctypes.POINTER(MphServerStats)], ip),
            "mph_server_set_solver": ([vp, ctypes.c_double, ctypes.c_double, ip], ip),
            "mph_server_set_option": ([vp, ctypes.c_char_p, ctypes.c_double], ip),
            "mph_server_destroy": ([vp], ip),
        }
        for name, (args, res) in decl.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        lib._mph_serving_declared = True
    return lib


def footprint(params: casegen.Params, parts: casegen.Particles, dim: int, precision: int = PRECISION_FP64) -> int:
    """Upper bound of the device bytes one case takes (the admission unit)."""
    p = params_to_c(params)
    pc = ParticlesC(parts)
    out = ctypes.c_longlong()
    _check(_lib().mph_case_footprint(ctypes.byref(p), ctypes.byref(pc.struct), dim, precision, ctypes.byref(out)))
    return out.value


def batch_step(cases, nsteps: int = 1, workers: int = 0) -> int:
    """Step independent cases concurrently (one host worker and one stream
    per case at a time); returns 0 or 7 (a solve reached its cap)."""
    lib = _lib()
    arr = (ctypes.c_void_p * len(cases))(*[c.h.value for c in cases])
    st = lib.mph_batch_step_workers(arr, len(cases), nsteps, workers)
    if st not in (0, 7):
        _check(st)
    return st


class Server:
    """Continuous-batching server on the current CUDA device."""

    def __init__(self, budget_bytes: int, workers: int = 16, device: int = -1):
        self.lib = _lib()
        h = ctypes.c_void_p()
        _check(self.lib.mph_server_create(int(budget_bytes), workers, device, ctypes.byref(h)))
        self.h = h
        self._live: Dict[int, tuple] = {}

    def set_solver(self, outer_rel_residual: float = 1e-6, inner_rel_residual: float = 1e-3, max_outer: int = 50):
        """Solver tolerances of the cases of later submissions."""
        _check(self.lib.mph_server_set_solver(self.h, outer_rel_residual, inner_rel_residual, max_outer))

    def set_option(self, name: str, value: float):
        """An engine option of the cases of later submissions."""
        _check(self.lib.mph_server_set_option(self.h, name.encode(), float(value)))

    def submit(self, params: casegen.Params, parts: casegen.Particles, dim: int, steps: int,
               precision: int = PRECISION_FP64, fields=("id", "pos", "vel")) -> int:
        n = parts.count
        out = {}
        if "id" in fields:
            out["id"] = np.empty(n, np.int32)
        if "type" in fields:
            out["type"] = np.empty(n, np.int32)
        for k in ("pos", "vel", "force"):
            if k in fields:
                out[k] = np.empty((n, 3))
        f = MphFields()
        for k, a in out.items():
            setattr(f, k, np_ptr(a, ctypes.c_int if a.dtype == np.int32 else ctypes.c_double))
        step_ms = np.zeros(steps, np.float32)
        p = params_to_c(params)
        pc = ParticlesC(parts)
        t = ctypes.c_longlong()
        _check(self.lib.mph_server_submit(self.h, ctypes.byref(p), ctypes.byref(pc.struct), dim, precision, steps,
                                          ctypes.byref(f), step_ms.ctypes.data_as(ctypes.c_void_p), ctypes.byref(t)))
        self._live[t.value] = (out, step_ms, f)
        return t.value

    def poll(self, wait_ms: int = 0, max_results: int = 64) -> List[dict]:
        buf = (MphServerResult * max_results)()
        n = ctypes.c_int()
        _check(self.lib.mph_server_poll(self.h, buf, max_results, wait_ms, ctypes.byref(n)))
        res = []
        for k in range(n.value):
            r = buf[k]
            out, step_ms, _ = self._live.pop(r.ticket)
            res.append({"ticket": r.ticket, "status": r.status, "steps": r.steps, "particles": r.particles,
                        "submit_s": r.submit_s, "admit_s": r.admit_s, "done_s": r.done_s,
                        "footprint": r.footprint_bytes, "error": r.error.decode(errors="replace"),
                        "fields": out, "step_ms": step_ms[:r.steps].copy()})
        return res

    def stats(self) -> dict:
        s = MphServerStats()
        _check(self.lib.mph_server_stats_get(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in MphServerStats._fields_ if k != "pad"}

    def outstanding(self) -> int:
        return len(self._live)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.mph_server_destroy(self.h)
            self.h = ctypes.c_void_p()
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ReplicaDispatcher:
    """Serving on several GPUs of one node: one Server per device, each
    request sent to the device with the most uncommitted budget (the
    footprints of its requests not yet finished), results gathered from all
    of them.  Host-side only: replicas share nothing and need no collective.
    `server_factory(device)` makes a server (tests pass fakes)."""

    def __init__(self, devices, budget_bytes: int, workers: int = 16, server_factory=None):
        make = server_factory or (lambda d: Server(budget_bytes, workers, device=d))
        self.devices = list(devices)
        self.servers = [make(d) for d in self.devices]
        self.budget = int(budget_bytes)
        self.queued = [0] * len(self.servers)      # footprints submitted and not yet finished
        self.route = {}                            # dispatcher ticket -> (replica, local ticket, footprint)
        self.back = {}                             # (replica, local ticket) -> dispatcher ticket
        self.next_ticket = 1

    def submit(self, params, parts, dim: int, steps: int, precision: int = PRECISION_FP64, fields=("id", "pos", "vel"),
               footprint_bytes: Optional[int] = None) -> int:
        fp = footprint_bytes if footprint_bytes is not None else footprint(params, parts, dim, precision)
        k = min(range(len(self.servers)), key=lambda r: (self.queued[r], r))
        local = self.servers[k].submit(params, parts, dim, steps, precision=precision, fields=fields)
        t = self.next_ticket
        self.next_ticket += 1
        self.queued[k] += fp
        self.route[t] = (k, local, fp)
        self.back[(k, local)] = t
        return t

    def poll(self, wait_ms: int = 0) -> List[dict]:
        out = []
        for k, srv in enumerate(self.servers):
            for r in srv.poll(wait_ms=wait_ms if not out else 0):
                t = self.back.pop((k, r["ticket"]))
                self.queued[k] -= self.route.pop(t)[2]
                r = dict(r)
                r["ticket"], r["device"] = t, self.devices[k]
                out.append(r)
        return out

    def outstanding(self) -> int:
        return len(self.route)

    def close(self):
        for srv in self.servers:
            srv.close()
