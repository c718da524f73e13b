"""The state upload and field download of the public API: fields read into
caller buffers (pinned host memory here) equal the library-allocated ones,
and a case given that state continues bit for bit like the case it came
from."""
import numpy as np
import pytest

from mphimplicit_gb300 import casegen, engine
from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
IDS = [c[0] for c in CASES]


def _pinned_like(fields):
    torch = pytest.importorskip("torch")
    out = {}
    for k, v in fields.items():
        dt = torch.int32 if v.dtype == np.int32 else torch.float64
        out[k] = torch.empty(v.shape, dtype=dt, pin_memory=True).numpy()
    return out


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_pinned_fields_and_state_upload(engine_lib, case, precision):
    name, dim, params, parts = case
    a = engine.Case(params, parts, dim, precision=precision)
    a.step(2)
    which = ("id", "type", "pos", "vel", "force", "neighbor_count")
    f = a.fields(which)
    pin = _pinned_like(f)
    a.fields(out=pin)
    for k in which:
        assert np.array_equal(f[k], pin[k]), k
    with pytest.raises(ValueError):
        a.fields(out={"pos": np.empty((a.count, 2))})
    # a fresh case given this state continues exactly as the original
    b = engine.Case(params, parts, dim, precision=precision)
    host = casegen.Particles(a.time(), parts.spacing, parts.domain_min, parts.domain_max, pin["type"], pin["pos"], pin["vel"])
    b.set_state(host, pin["id"], a.export("WallCenter"))
    a.step(1)
    b.step(1)
    fa, fb = a.fields(("id", "pos", "vel")), b.fields(("id", "pos", "vel"))
    for k in ("id", "pos", "vel"):
        assert np.array_equal(fa[k], fb[k]), k
