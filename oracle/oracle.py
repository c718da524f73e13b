"""Python access to the CPU oracle (TEST INFRASTRUCTURE).

* ``Oracle``   wraps _build/libmph_oracle.so, the C++ restatement of the
               reference algorithm (mph_oracle.cpp).
* ``Reference`` wraps _ref/libmphref{2d,3d}.so, the reference solver's own
               sources compiled with ref_harness.cpp (development container only;
               never present on the GPU hosts).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs use this module, as the checker.  The shipped engine never imports it.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import sys
import tempfile
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from mphimplicit_gb300 import casegen  # noqa: E402
from mphimplicit_gb300.cabi import MphParticles, ParticlesC, params_to_c  # noqa: E402

ORACLE_SO = os.path.join(HERE, "_build", "libmph_oracle.so")
REF_SO = {2: os.path.join(HERE, "_ref", "libmphref2d.so"), 3: os.path.join(HERE, "_ref", "libmphref3d.so")}
_KIND = {0: np.int32, 1: np.int64, 2: np.float64}


def build_oracle(ref=False) -> None:
    """Build the oracle; ref=True also the reference harness (needs the
    reference checkout), ref="if-present" only where the checkout exists."""
    targets = ["oracle"] + (["ref-if-present"] if ref == "if-present" else ["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


_lib = None


def oracle_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        lib = ctypes.CDLL(ORACLE_SO)
        lib.mpho_create.restype = ctypes.c_void_p
        lib.mpho_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        for fn in ("mpho_destroy", "mpho_init", "mpho_step_begin", "mpho_cellsort", "mpho_neighbors",
                   "mpho_explicit", "mpho_assemble", "mpho_mg_build", "mpho_step_end", "mpho_output_fields"):
            getattr(lib, fn).argtypes = [ctypes.c_void_p]
            getattr(lib, fn).restype = None
        lib.mpho_solve.argtypes = [ctypes.c_void_p]
        lib.mpho_solve.restype = ctypes.c_int
        lib.mpho_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.mpho_step.restype = ctypes.c_int
        lib.mpho_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int)]
        lib.mpho_array.restype = ctypes.c_long
        lib.mpho_scalars.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        lib.mpho_scalar_names.restype = ctypes.c_char_p
        lib.mpho_solve_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        lib.mpho_mg_level_geom.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        lib.mpho_mg_level_matrix.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                             ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int)]
        lib.mpho_set_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.mpho_set_threads.argtypes = [ctypes.c_int]
        lib.mpho_set_tolerance.argtypes = [ctypes.c_void_p, ctypes.c_double]
        lib.mpho_set_tolerance.restype = None
        _lib = lib
    return _lib


def _copy(ptr, n, kind):
    if n <= 0:
        return np.zeros(0, dtype=_KIND[kind])
    ct = {0: ctypes.c_int32, 1: ctypes.c_int64, 2: ctypes.c_double}[kind]
    buf = ctypes.cast(ptr, ctypes.POINTER(ct * n)).contents
    return np.frombuffer(buf, dtype=_KIND[kind]).copy()


class Oracle:
    """The C++ restatement, stage by stage."""

    def __init__(self, params: casegen.Params, parts: casegen.Particles, dim: int, threads: int = 1):
        self.lib = oracle_lib()
        self.lib.mpho_set_threads(threads)
        self.dim = dim
        self._p = params_to_c(params)
        self._parts = ParticlesC(parts)
        self.h = self.lib.mpho_create(ctypes.byref(self._p), ctypes.byref(self._parts.struct), dim)
        if not self.h:
            raise ValueError("oracle rejected the case")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.mpho_destroy(self.h)
            self.h = None

    def init(self): self.lib.mpho_init(self.h)
    def step_begin(self): self.lib.mpho_step_begin(self.h)
    def cellsort(self): self.lib.mpho_cellsort(self.h)
    def neighbors(self): self.lib.mpho_neighbors(self.h)
    def explicit(self): self.lib.mpho_explicit(self.h)
    def assemble(self): self.lib.mpho_assemble(self.h)
    def mg_build(self): self.lib.mpho_mg_build(self.h)
    def solve(self): return self.lib.mpho_solve(self.h)
    def step_end(self): self.lib.mpho_step_end(self.h)
    def output_fields(self): self.lib.mpho_output_fields(self.h)
    def step(self, n=1): return self.lib.mpho_step(self.h, n)

    def set_tolerance(self, rel: float):
        """CR stop test ||r||/||b|| < rel; the reference's constant is 1e-6."""
        self.lib.mpho_set_tolerance(self.h, rel)

    def array(self, name: str) -> np.ndarray:
        p = ctypes.c_void_p()
        k = ctypes.c_int()
        n = self.lib.mpho_array(self.h, name.encode(), ctypes.byref(p), ctypes.byref(k))
        if n < 0:
            raise KeyError(name)
        return _copy(p, n, k.value)

    def scalars(self) -> Dict[str, float]:
        buf = (ctypes.c_double * 64)()
        n = self.lib.mpho_scalars(self.h, buf)
        return dict(zip(self.lib.mpho_scalar_names().decode().split(","), list(buf)[:n]))

    def solve_stats(self):
        buf = (ctypes.c_double * 5)()
        self.lib.mpho_solve_stats(self.h, buf)
        return {"iter": int(buf[0]), "rr0": buf[1], "rr": buf[2], "rs0": buf[3], "rs": buf[4]}

    def mg_levels(self):
        depth = int(self.scalars()["MultiGridDepth"])
        out = []
        for L in range(depth):
            g = (ctypes.c_int * 9)()
            self.lib.mpho_mg_level_geom(self.h, L, g)
            cof = ctypes.POINTER(ctypes.c_double)()
            inv = ctypes.POINTER(ctypes.c_double)()
            rows, width = ctypes.c_int(), ctypes.c_int()
            self.lib.mpho_mg_level_matrix(self.h, L, ctypes.byref(cof), ctypes.byref(inv), ctypes.byref(rows), ctypes.byref(width))
            out.append({"min": list(g[0:3]), "max": list(g[3:6]), "count": list(g[6:9]),
                        "cof": _copy(cof, rows.value * width.value, 2).reshape(rows.value, width.value),
                        "invd": _copy(inv, rows.value, 2)})
        return out

    def set_state(self, parts: casegen.Particles, ids: np.ndarray, wall_center: Optional[np.ndarray] = None):
        self._state = ParticlesC(parts, ids)
        wc = None if wall_center is None else np.ascontiguousarray(wall_center, dtype=np.float64)
        self._wc = wc
        self.lib.mpho_set_state(self.h, ctypes.byref(self._state.struct), None if wc is None else wc.ctypes.data)


class Reference:
    """The reference solver's own code, compiled with ref_harness.cpp."""

    def __init__(self, params: casegen.Params, parts: casegen.Particles, dim: int, workdir: Optional[str] = None):
        so = REF_SO[dim]
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        # one process-wide copy of the reference globals per library: load a
        # private copy per instance
        self.tmp = tempfile.mkdtemp(prefix="mphref_", dir=workdir)
        priv = os.path.join(self.tmp, os.path.basename(so))
        with open(so, "rb") as fi, open(priv, "wb") as fo:
            fo.write(fi.read())
        self.lib = lib = ctypes.CDLL(priv)
        lib.ref_init.argtypes = [ctypes.c_char_p] * 3
        lib.ref_array.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int)]
        lib.ref_array.restype = ctypes.c_long
        lib.ref_scalars.argtypes = [ctypes.POINTER(ctypes.c_double)]
        lib.ref_scalar_names.restype = ctypes.c_char_p
        lib.ref_mg_level_geom.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        lib.ref_mg_level_matrix.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 5
        lib.ref_write_vtk.argtypes = [ctypes.c_char_p]
        lib.ref_write_prof.argtypes = [ctypes.c_char_p]
        self.dim = dim
        self.data, self.grid = casegen.write_case(os.path.join(self.tmp, "case"), params, parts)
        self.log = os.path.join(self.tmp, "case.log")
        self.n = lib.ref_init(self.data.encode(), self.grid.encode(), self.log.encode())

    def init(self): pass
    def step_begin(self): self.lib.ref_step_begin()
    def cellsort(self): self.lib.ref_cellsort()
    def neighbors(self): self.lib.ref_neighbor()
    def explicit(self): self.lib.ref_explicit()

    def assemble(self):
        self.lib.ref_assemble_ac()
        self.lib.ref_multiply_c()

    def free_c(self): self.lib.ref_free_c()
    def mg_build(self): self.lib.ref_mg_build()
    def solve(self): self.lib.ref_solve()
    def output_fields(self): self.lib.ref_output_fields()

    def step_end(self):
        self.lib.ref_free_mg()
        self.lib.ref_free_a()
        self.lib.ref_free_neighbor()
        self.lib.ref_advance_time()

    def step(self, n=1):
        for _ in range(n):
            self.step_begin(); self.cellsort(); self.neighbors(); self.explicit(); self.assemble()
            self.free_c(); self.mg_build(); self.solve(); self.step_end()

    def array(self, name: str) -> np.ndarray:
        p = ctypes.c_void_p()
        k = ctypes.c_int()
        n = self.lib.ref_array(name.encode(), ctypes.byref(p), ctypes.byref(k))
        if n < 0:
            raise KeyError(name)
        return _copy(p, n, k.value)

    def scalars(self) -> Dict[str, float]:
        buf = (ctypes.c_double * 64)()
        n = self.lib.ref_scalars(buf)
        return dict(zip(self.lib.ref_scalar_names().decode().split(","), list(buf)[:n]))

    def solve_log(self):
        """(iter, rr0, rr, rs0, rs) of every solve so far, parsed from the
        reference's log line (source/main.cpp:4381)."""
        out = []
        with open(self.log) as f:
            for line in f:
                if "iter,=" in line:
                    it = int(re.search(r"iter,=\s*(-?\d+)", line).group(1))
                    nums = [float(x) for x in re.findall(r"=,\s*([-+0-9.eE]+)", line)]
                    out.append((it, *nums))
        return out

    def mg_levels(self):
        depth = int(self.scalars()["MultiGridDepth"])
        out = []
        for L in range(depth):
            g = (ctypes.c_int * 9)()
            self.lib.ref_mg_level_geom(L, g)
            ptr = ctypes.POINTER(ctypes.c_int)()
            ind = ctypes.POINTER(ctypes.c_int)()
            cof = ctypes.POINTER(ctypes.c_double)()
            inv = ctypes.POINTER(ctypes.c_double)()
            rows = ctypes.c_int()
            self.lib.ref_mg_level_matrix(L, ctypes.byref(ptr), ctypes.byref(ind), ctypes.byref(cof), ctypes.byref(inv), ctypes.byref(rows))
            nr = rows.value
            p = _copy(ptr, nr + 1, 0)
            nnz = int(p[-1])
            out.append({"min": list(g[0:3]), "max": list(g[3:6]), "count": list(g[6:9]), "ptr": p,
                        "ind": _copy(ind, nnz, 0), "cof": _copy(cof, nnz, 2), "invd": _copy(inv, nr, 2)})
        return out
