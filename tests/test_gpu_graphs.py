"""Graph replay of the solver's iteration chunks changes nothing: the same
kernels run in the same order whether they are launched one by one or
replayed from a captured CUDA graph, so both give bit-identical steps."""
import numpy as np
import pytest

from mphimplicit_gb300 import engine
from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]


def _run(params, parts, dim, precision, graphs, steps=2):
    g = engine.Case(params, parts, dim, precision=precision)
    g.set_option("graphs", 1 if graphs else 0)
    iters = []
    for _ in range(steps):
        g.step(1)
        s = g.solve_stats()
        iters.append((s["iter"], s["outer"]))
    f = g.fields(("id", "pos", "vel"))
    g.close()
    return f, iters


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_graph_replay_is_bit_identical(engine_lib, case, precision):
    name, dim, params, parts = case
    fa, ia = _run(params, parts, dim, precision, True)
    fb, ib = _run(params, parts, dim, precision, False)
    assert ia == ib
    assert np.array_equal(fa["id"], fb["id"])
    assert np.array_equal(fa["pos"], fb["pos"])
    assert np.array_equal(fa["vel"], fb["vel"])


@pytest.mark.parametrize("case", CASES[:2], ids=IDS[:2])
def test_profiled_mixed_steps_keep_graphs_and_bits(engine_lib, case):
    """With kernel profiling on, the mixed form still replays its CR chunks as
    graphs (each chunk records an event pair around every iteration's
    operator): the operator timings cover exactly the iterations that ran,
    and the step gives the same bits as an unprofiled one."""
    name, dim, params, parts = case
    a = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    a.profile(True)
    a.step(2)
    p = a.profile_read()
    b = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    iters = 0
    for _ in range(2):
        b.step(1)
        iters += b.solve_stats()["iter"]
    assert p["kern_n_spmv"] == iters
    assert p["kern_ms_spmv"] > 0.0
    fa, fb = a.fields(("id", "pos", "vel")), b.fields(("id", "pos", "vel"))
    for k in ("id", "pos", "vel"):
        assert np.array_equal(fa[k], fb[k]), k


def _run_mixed(params, parts, dim, device_loop, factored, steps=3):
    g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    g.set_solver(1e-10, 1e-3, 50)
    g.set_option("extrapolate", 2)
    g.set_option("factored", factored)
    g.set_option("device_loop", device_loop)
    stats = []
    for _ in range(steps):
        g.step(1)
        s = g.solve_stats()
        stats.append((s["iter"], s["outer"], s["status"], s["rr"], s["rr0"]))
    f = g.fields(("id", "pos", "vel"))
    g.close()
    return f, stats


@pytest.mark.parametrize("factored", [1, 0], ids=["factored", "assembled"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_device_driven_solve_is_bit_identical(engine_lib, case, factored):
    """The whole mixed solve as one graph with device-side loops (conditional
    while nodes for the refinement phases and the CR iterations) runs the
    kernels of the host-driven solve in the same order: the same bits, the
    same iteration and phase counts, with refinement to 1e-10 and the
    extrapolated start (several phases a solve)."""
    name, dim, params, parts = case
    fa, sa = _run_mixed(params, parts, dim, 1, factored)
    fb, sb = _run_mixed(params, parts, dim, 0, factored)
    assert sa == sb
    assert all(s[1] >= 2 for s in sa)
    for k in ("id", "pos", "vel"):
        assert np.array_equal(fa[k], fb[k]), k


def test_device_driven_solve_stops_at_its_caps(engine_lib):
    """A refinement bound of one phase ends the device-side loops at once:
    the solve reports one phase and its unmet tolerance."""
    name, dim, params, parts = CASES[0]
    g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    g.set_solver(1e-12, 1e-3, 1)
    g.set_option("device_loop", 1)
    g.step(1)
    s = g.solve_stats()
    assert s["outer"] == 1 and s["status"] == 7
