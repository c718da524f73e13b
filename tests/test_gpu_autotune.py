"""The mixed form's launch-shape options and the autotuner on a GB300.

The graph chunk only decides how often the host reads the solver's flags:
every chunk length gives the same bits.  The operator block widths change
the order in which block partial sums of the dot products add up: results
stay within the solver's band of the defaults, and refined to 1e-10 within
1e-9.  The autotuner returns settings among its candidates."""
import numpy as np
import pytest

from mphimplicit_gb300 import autotune, engine
from mphimplicit_gb300.cabi import PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]


def _run(case, opts, steps=2):
    name, dim, params, parts = case
    g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
    g.set_solver(1e-10, 1e-3, 50)
    for k, v in opts.items():
        g.set_option(k, v)
    g.step(steps)
    out = g.fields(("id", "vel")), g.solve_stats()
    g.close()
    return out


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_chunk_length_keeps_the_bits(engine_lib, case):
    (fa, sa), (fb, sb) = _run(case, {"chunk": 8}), _run(case, {"chunk": 32})
    assert sa["iter"] == sb["iter"]
    assert np.array_equal(fa["vel"], fb["vel"])


@pytest.mark.parametrize("opts", [{"pair_block": 128}, {"pair_block": 256, "ct_block": 128}], ids=["pb128", "pb256-ct128"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_block_widths_within_tolerance(engine_lib, case, opts):
    (fa, sa), (fb, sb) = _run(case, {}), _run(case, opts)
    assert np.array_equal(fa["id"], fb["id"])
    assert sb["status"] == 0 and sb["rr"] / sb["rr0"] < 1e-20
    err = float(np.linalg.norm(fb["vel"] - fa["vel"]) / np.linalg.norm(fa["vel"]))
    assert err <= 1e-9, err


def test_autotuner_picks_candidates(engine_lib):
    name, dim, params, parts = CASES[2]

    def make():
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        g.set_solver(1e-10, 1e-3, 50)
        return g
    out = autotune.tune(make, steps=1, warmup=1)
    for k, values in autotune.CANDIDATES:
        assert out["settings"][k] in values
    with pytest.raises(engine.MphError):
        make().set_option("pair_block", 384)
