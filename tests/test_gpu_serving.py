"""Batched stepping and the serving loop.

Each case's arithmetic is independent of the others (own buffers, own
stream, deterministic reductions), so a case stepped in a batch or served in
a mix of cases must give the same bits as the same case stepped alone: the
stated tolerance of these tests is exact equality."""
import numpy as np
import pytest

from mphimplicit_gb300 import casegen, engine, serving
from mphimplicit_gb300.cabi import PRECISION_FP64, PRECISION_MIXED
from parity_util import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()


def _alone(params, parts, dim, precision, steps):
    g = engine.Case(params, parts, dim, precision=precision)
    g.step(steps)
    f = g.fields(("id", "pos", "vel"))
    g.close()
    return f


def _mix():
    """Small cases of both dimensions and precisions, uneven sizes."""
    out = []
    for k, (name, dim, params, parts) in enumerate(CASES):
        out.append((f"{name}-fp64", dim, params, parts, PRECISION_FP64, 2 + k % 2))
        out.append((f"{name}-mixed", dim, params, parts, PRECISION_MIXED, 3 - k % 2))
    p, parts = casegen.square_drop_2d(scale=0.2, seed=5)
    out.append(("dam2d_20-mixed", 2, p, parts, PRECISION_MIXED, 2))
    return out


def test_batch_step_matches_alone(engine_lib):
    mix = _mix()
    cases = [engine.Case(params, parts, dim, precision=prec) for _, dim, params, parts, prec, _ in mix]
    assert serving.batch_step(cases, 2) in (0, 7)
    for (name, dim, params, parts, prec, _), g in zip(mix, cases):
        ref = _alone(params, parts, dim, prec, 2)
        got = g.fields(("id", "pos", "vel"))
        for k in ("id", "pos", "vel"):
            assert np.array_equal(got[k], ref[k]), (name, k)
        g.close()


def test_batched_solve_matches_per_case_solve(engine_lib):
    """With option batch_solve, mph_batch_step solves its point-Jacobi mixed
    cases together (the CR iterations of all of them in one launch per
    kernel, each block on its case with the case's own block decomposition),
    so every case gets the bits and the iteration counts of its own solve:
    the batch with the option off is the reference.  Cases of
    several sizes and both dimensions, so the batch forms groups and its
    cases finish their refinement phases at different times."""
    ens = casegen.ensemble_2d(10, seed=3)
    picked = [(2, params, parts) for params, parts in ens if parts.count < 20000][:6]
    for name, dim, params, parts in CASES:
        picked.append((dim, params, parts))
    runs = {}
    for on in (0, 1):
        cases = []
        for dim, params, parts in picked:
            g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
            g.set_solver(1e-8, 1e-3, 50)
            g.set_option("extrapolate", 2)
            g.set_option("batch_solve", on)
            cases.append(g)
        assert serving.batch_step(cases, 3) in (0, 7)
        runs[on] = [(g.fields(("id", "pos", "vel")), g.solve_stats()) for g in cases]
        for g in cases:
            g.close()
    for (fa, sa), (fb, sb) in zip(runs[0], runs[1]):
        assert sa["iter"] == sb["iter"] and sa["outer"] == sb["outer"] and sa["status"] == sb["status"]
        for k in ("id", "pos", "vel"):
            assert np.array_equal(fa[k], fb[k]), k


def test_batch_rejects_duplicates(engine_lib):
    name, dim, params, parts = CASES[0]
    g = engine.Case(params, parts, dim)
    with pytest.raises(engine.MphError):
        serving.batch_step([g, g], 1)
    g.close()


def test_server_results_equal_alone_and_admission_by_footprint(engine_lib):
    mix = _mix()
    fps = [serving.footprint(params, parts, dim, prec) for _, dim, params, parts, prec, _ in mix]
    budget = sorted(fps)[-1] + sorted(fps)[-2]          # at most about two cases resident at once
    srv = serving.Server(budget, workers=4)
    tickets = {}
    for (name, dim, params, parts, prec, steps) in mix:
        tickets[srv.submit(params, parts, dim, steps, precision=prec)] = (name, dim, params, parts, prec, steps)
    results = []
    for _ in range(600):
        results += srv.poll(wait_ms=200)
        if len(results) == len(mix):
            break
    st = srv.stats()
    srv.close()
    assert len(results) == len(mix)
    assert st["used_bytes"] == 0 and st["pending"] == 0
    assert st["steps"] == sum(m[5] for m in mix)
    by_ticket = sorted(results, key=lambda r: r["ticket"])
    admits = [r["admit_s"] for r in by_ticket]
    assert admits == sorted(admits)                     # admitted in arrival order
    for r in results:
        name, dim, params, parts, prec, steps = tickets[r["ticket"]]
        assert r["status"] in (0, 7), (name, r["error"])
        assert r["steps"] == steps and len(r["step_ms"]) == steps and (r["step_ms"] > 0).all()
        assert r["submit_s"] <= r["admit_s"] <= r["done_s"]
        ref = _alone(params, parts, dim, prec, steps)
        for k in ("id", "pos", "vel"):
            assert np.array_equal(r["fields"][k], ref[k]), (name, k)


def test_footprint_bounds_device_memory(engine_lib):
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    p, parts = casegen.square_drop_2d(scale=0.5, seed=3)
    for prec in (PRECISION_FP64, PRECISION_MIXED):
        fp = serving.footprint(p, parts, 2, prec)
        free0, _ = torch.cuda.mem_get_info()
        g = engine.Case(p, parts, 2, precision=prec)
        g.step(2)
        free1, _ = torch.cuda.mem_get_info()
        g.close()
        assert free0 - free1 <= fp, (prec, free0 - free1, fp)


def test_server_settings_apply_to_its_cases(engine_lib):
    """mph_server_set_solver / mph_server_set_option reach every case the
    server creates afterwards: served mixed cases refined to 1e-10 with the
    extrapolated start give the bits of the same settings stepped alone, and
    an invalid option fails the request, not the server."""
    mix = [m for m in _mix() if m[4] == PRECISION_MIXED]
    srv = serving.Server(int(20e9), workers=4)
    srv.set_solver(1e-10, 1e-3, 50)
    srv.set_option("extrapolate", 2)
    tickets = {srv.submit(params, parts, dim, 4, precision=prec): (name, dim, params, parts)
               for name, dim, params, parts, prec, _ in mix}
    results = []
    while len(results) < len(tickets):
        results += srv.poll(wait_ms=100)
    for r in results:
        assert r["status"] == 0, r["error"]
        name, dim, params, parts = tickets[r["ticket"]]
        g = engine.Case(params, parts, dim, precision=PRECISION_MIXED)
        g.set_solver(1e-10, 1e-3, 50)
        g.set_option("extrapolate", 2)
        g.step(4)
        ref = g.fields(("id", "pos", "vel"))
        g.close()
        for k in ("id", "pos", "vel"):
            assert np.array_equal(r["fields"][k], ref[k]), (name, k)
    srv.set_option("no_such_option", 1)
    name, dim, params, parts = CASES[0]
    t = srv.submit(params, parts, dim, 1, precision=PRECISION_MIXED)
    res = []
    while not res:
        res = srv.poll(wait_ms=100)
    assert res[0]["ticket"] == t and res[0]["status"] == 1
    srv.close()
