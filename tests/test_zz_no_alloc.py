"""mph_residual_noalloc, the allocation-free residual check, against the
solver's own residual report.

The mixed solver's last outer step ends with the FP64 residual kernel, so
mph_get_solve_stats then holds rr = ||b - A x||^2 of the returned solution and
rr0 = ||b||^2; the allocation-free entry point recomputes both from the
resident system with its fixed scratch array.  Two calls in a row must agree
with the report and with each other.  This file is collected last, so it runs
after every other GPU test as well as alone."""
import ctypes

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


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_noalloc_matches_solver_report(engine_lib, case):
    name, dim, params, parts = case
    g = _solved(params, parts, dim, PRECISION_MIXED)
    s = g.solve_stats()
    st1, (rr1, bb1) = _noalloc(g)
    st2, (rr2, bb2) = _noalloc(g)
    assert st1 == 0 and st2 == 0, engine.load_library().mph_last_error()
    assert (rr1, bb1) == (rr2, bb2)
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
    assert _rel(bb1, s["rr0"]) <= TOL
    assert np.isfinite(rr1) and rr1 / bb1 < 1e-10
    g.close()


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
