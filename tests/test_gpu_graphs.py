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
