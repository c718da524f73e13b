"""The mixed form's CR start from extrapolated velocities (option
"extrapolate"; the reference starts from v_n, main.cpp:4299-4308).

The start value changes only where the CR iteration begins: the solution is
still refined to the outer tolerance, so a step from a state with velocity
history lies within 1e-6 of the FP64 form solved to 1e-12 from the same
state.  A state set from outside has no history, so the next step starts
from v_n again, bit for bit as a fresh case."""
import numpy as np
import pytest

from mphimplicit_gb300 import casegen, engine
from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]


def _state(g, parts):
    f = g.fields(("id", "type", "pos", "vel"))
    p = casegen.Particles(g.time(), parts.spacing, parts.domain_min, parts.domain_max, f["type"], f["pos"], f["vel"])
    return p, f["id"], g.export("WallCenter")


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_extrapolated_start_keeps_accuracy(engine_lib, case, order):
    name, dim, params, parts = case
    m = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    m.set_solver(1e-10, 1e-3, 50)
    m.set_option("extrapolate", order)
    m.step(4)
    st, ids, wc = _state(m, parts)
    f = engine.Case(params, parts, dim, precision=PRECISION_FP64)
    f.set_state(st, ids, wc)
    f.set_solver(1e-12, 1e-3, 50)
    f.step(1)
    m.step(1)
    s = m.solve_stats()
    assert s["status"] == 0 and s["rr"] / s["rr0"] < 1e-20
    a, b = m.fields(("id", "type", "vel")), f.fields(("id", "type", "vel"))
    assert np.array_equal(a["id"], b["id"])
    fl = b["type"] < 2
    err = float(np.linalg.norm(a["vel"][fl] - b["vel"][fl]) / np.linalg.norm(b["vel"][fl]))
    print(f"{name} order {order}: {s['iter']} FP32 iterations, velocity vs FP64 at 1e-12: {err:.2e}")
    assert err <= 1e-6


def test_set_state_clears_the_history(engine_lib):
    name, dim, params, parts = CASES[2]
    m = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    m.set_option("extrapolate", 2)
    m.step(3)
    st, ids, wc = _state(m, parts)
    m.set_state(st, ids, wc)
    m.step(1)
    fresh = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    fresh.set_option("extrapolate", 2)
    fresh.set_state(st, ids, wc)
    fresh.step(1)
    assert np.array_equal(m.export("Velocity"), fresh.export("Velocity"))
    assert m.solve_stats()["iter"] == fresh.solve_stats()["iter"]


def test_extrapolate_is_mixed_form_only(engine_lib):
    name, dim, params, parts = CASES[0]
    f = engine.Case(params, parts, dim, precision=PRECISION_FP64)
    with pytest.raises(engine.MphError):
        f.set_option("extrapolate", 1)
    m = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    with pytest.raises(engine.MphError):
        m.set_option("extrapolate", 3)


def test_keep_history_continues_bit_for_bit(engine_lib):
    """With option keep_history, uploading the state a case just read back
    changes nothing: the next steps give the bits of the case stepped on."""
    name, dim, params, parts = CASES[2]
    runs = []
    for upload in (False, True):
        m = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        m.set_option("extrapolate", 2)
        m.set_option("keep_history", 1)
        m.step(3)
        if upload:
            st, ids, wc = _state(m, parts)
            m.set_state(st, ids, wc)
        m.step(2)
        runs.append((m.export("Velocity"), m.solve_stats()["iter"]))
    assert np.array_equal(runs[0][0], runs[1][0]) and runs[0][1] == runs[1][1]
