"""mph_residual_noalloc, the allocation-free residual check, against an
independent residual and against the solver's own report.

Servers whose device memory is committed to resident cases call this check
where a per-call allocation could fail.  The entry point recomputes ||b - A
x||^2 and ||b||^2 of the solved system with its fixed scratch array.  Each
result is checked against numpy on the exported system (CsrPtrA / CsrIndA /
CsrCofA, VectorB and the solved Velocity), and two calls in a row must give
the same bits.  The mixed solver's last outer step also reports the same two
norms (its FP64 residual kernel has the same arithmetic).  One test runs in a
fresh process: it creates a case and calls the check with no earlier lookup
of the array.  This file is collected last, so it runs after every other GPU
test as well as alone."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from mphimplicit_gb300 import casegen, engine
from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]
ERR_CAPACITY, ERR_STATE = 6, 9
TOL = 1e-12


def _entry():
    fn = engine.load_library().mph_residual_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    fn.restype = ctypes.c_int
    return fn


def _noalloc(case):
    out = (ctypes.c_double * 2)()
    st = _entry()(case.h, out)
    return st, (out[0], out[1])


def _solved(params, parts, dim, precision, factored=0):
    g = engine.Case(params, parts, dim, precision=precision)
    g.set_option("factored", factored)   # the factored mixed form has no FP64 blocks
    for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build", "solve"):
        g.stage(st)
    return g


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def _numpy_norms(g, dim):
    """||b - A x||^2 and ||b||^2 from the exported system, in numpy."""
    ptr, ind, val = g.export("CsrPtrA"), g.export("CsrIndA"), g.export("CsrCofA")
    b = g.export("VectorB")
    nf = g.fluid_count
    x = g.export("Velocity").reshape(-1, 3)[:nf, :dim].ravel()
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    ax = np.bincount(rows, weights=val * x[ind], minlength=len(ptr) - 1)
    r = b - ax
    return float(r @ r), float(b @ b)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_noalloc_matches_solver_report(engine_lib, case):
    name, dim, params, parts = case
    g = _solved(params, parts, dim, PRECISION_MIXED)
    s = g.solve_stats()
    st1, (rr1, bb1) = _noalloc(g)
    st2, (rr2, bb2) = _noalloc(g)
    assert st1 == 0 and st2 == 0, engine.load_library().mph_last_error()
    assert (rr1, bb1) == (rr2, bb2)
    rr_np, bb_np = _numpy_norms(g, dim)
    assert _rel(bb1, bb_np) <= TOL
    assert _rel(rr1, rr_np) <= 1e-6   # r = b - A x is ~1e-6 of b: cancellation
    assert _rel(rr1, s["rr"]) <= TOL
    assert _rel(bb1, s["rr0"]) <= TOL
    assert rr1 / bb1 < 1e-12   # the solve's stopping test, ||r|| < 1e-6 ||b||
    g.close()


def test_noalloc_fp64_case(engine_lib):
    name, dim, params, parts = CASES[0]
    g = _solved(params, parts, dim, PRECISION_FP64)
    s = g.solve_stats()
    st1, (rr1, bb1) = _noalloc(g)
    st2, out2 = _noalloc(g)
    assert st1 == 0 and st2 == 0
    assert (rr1, bb1) == out2
    rr_np, bb_np = _numpy_norms(g, dim)
    assert _rel(bb1, bb_np) <= TOL
    assert _rel(rr1, rr_np) <= 1e-6
    assert _rel(bb1, s["rr0"]) <= TOL
    # the FP64 form stops on its recursive residual; the true one stays close
    assert np.isfinite(rr1) and rr1 / bb1 < 1e-10
    g.close()


FRESH = r"""
import ctypes, sys
sys.path[:0] = [{repo!r}, {tests!r}]
from mphimplicit_gb300 import engine
from mphimplicit_gb300.cabi import PRECISION_MIXED
from parity_util import small_cases
name, dim, params, parts = small_cases()[0]
g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
g.set_option("factored", 0)
for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build", "solve"):
    g.stage(st)
fn = engine.load_library().mph_residual_noalloc
fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
out = (ctypes.c_double * 2)()
st = fn(g.h, out)
s = g.solve_stats()
print(st, out[0], out[1], s["rr"], s["rr0"])
"""


def test_noalloc_first_call_after_case_creation(engine_lib):
    """In a fresh process the first check comes right after case creation,
    with no earlier lookup of the array: creation reserved it."""
    here = os.path.dirname(os.path.abspath(__file__))
    code = FRESH.format(repo=os.path.dirname(here), tests=here)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    st, rr, bb, srr, srr0 = r.stdout.split()[-5:]
    assert int(st) == 0
    assert _rel(float(rr), float(srr)) <= TOL and _rel(float(bb), float(srr0)) <= TOL


def test_noalloc_rejects_calls_out_of_order(engine_lib):
    name, dim, params, parts = CASES[0]
    g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    g.set_option("factored", 0)
    assert _noalloc(g)[0] == ERR_STATE          # nothing solved yet
    for st in ("step_begin", "cellsort", "neighbors", "explicit", "assemble", "mg_build"):
        g.stage(st)
    assert _noalloc(g)[0] == ERR_STATE          # assembled, not solved
    g.stage("solve")
    assert _noalloc(g)[0] == 0
    g.stage("step_end")
    assert _noalloc(g)[0] == ERR_STATE          # the step has ended
    assert _entry()(g.h, None) != 0             # null output
    g.close()
    f = _solved(params, parts, dim, PRECISION_MIXED, factored=1)
    assert _noalloc(f)[0] == ERR_STATE          # no FP64 blocks in this form
    f.close()


def test_noalloc_rejects_cases_beyond_its_limit(engine_lib):
    # 1449 x 1449 = 2,099,601 fluid particles > 2,097,152
    parts = casegen.dam_case(2, (1449, 1449), (1460, 1452), 0.001, seed=1)
    params = casegen.baseline_params(2, 0.001, 1.0e-5)
    g = engine.Case(params, parts, 2, precision=PRECISION_MIXED)
    assert g.fluid_count > 2_097_152
    st, _ = _noalloc(g)
    assert st == ERR_CAPACITY
    assert b"limit" in engine.load_library().mph_last_error()
    g.close()
