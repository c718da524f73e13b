"""Restart from the full-precision checkpoint sidecar continues bit for bit
(the .prof frames keep 7 digits, so a restart from them would not)."""
import numpy as np
import pytest

from mphimplicit_gb300 import engine
from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_restart_from_checkpoint_is_bit_exact(engine_lib, tmp_path, case, precision):
    name, dim, params, parts = case
    a = engine.Case(params, parts, dim, precision=precision)
    a.step(2)
    path = str(tmp_path / f"{name}.ckpt")
    a.checkpoint(path)
    a.step(2)
    b = engine.Case.restore(params, path, dim, precision=precision)
    b.step(2)
    assert a.time() == b.time()
    fa, fb = a.fields(("id", "pos", "vel")), b.fields(("id", "pos", "vel"))
    for k in ("id", "pos", "vel"):
        assert np.array_equal(fa[k], fb[k]), k
    assert np.array_equal(a.export("WallCenter"), b.export("WallCenter"))
