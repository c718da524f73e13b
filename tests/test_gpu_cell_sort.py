"""The production cell sort (option cell_sort 1: a counting sort of the cell
keys with scan-derived bucket offsets) against the oracle, which runs the
reference's bitonic network (main.cpp:1190-1211).

That network is not stable, so the two give different orders inside a cell;
what must agree is everything the order does not decide: the sorted keys and
the cell ranges bit for bit, the set of particles of every cell, every
particle's neighbour and P-neighbour sets (by particle id), and the step's
result by particle id within the band of the FP64 parity tests (the sums
then run in another order).  The counting sort itself is deterministic:
two runs give the same permutation."""
import numpy as np
import pytest

from mphimplicit_gb300 import casegen, engine
from parity_util import small_cases, vec_proj

pytestmark = pytest.mark.gpu

CASES = small_cases()
CASES.append(("dam2d_full", 2) + casegen.square_drop_2d(1.0, seed=0))
IDS = [c[0] for c in CASES]
RANGES = ["CellIndex", "CellFluidParticleBegin", "CellFluidParticleEnd", "CellWallParticleBegin", "CellWallParticleEnd"]


def _cell_sets(ids, begin, end):
    return [tuple(sorted(ids[b:e])) for b, e in zip(begin, end)]


def _neighbour_sets(ids, ptr, ind):
    out = {}
    for p in range(len(ids)):
        out[int(ids[p])] = tuple(sorted(ids[ind[ptr[p]:ptr[p + 1]]]))
    return out


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_counting_sort_against_bitonic_oracle(engine_lib, oracle_built, case):
    name, dim, params, parts = case
    o = oracle_built.Oracle(params, parts, dim, threads=4)
    o.init()
    g = engine.Case(params, parts, dim)
    g.set_option("cell_sort", 1)
    o.step_begin(); g.stage("step_begin")
    o.cellsort(); g.stage("cellsort")
    for n in RANGES:
        assert np.array_equal(g.export(n), o.array(n)), n
    gi, oi = g.export("ParticleIndex"), o.array("ParticleIndex")
    for b, e in (("CellFluidParticleBegin", "CellFluidParticleEnd"), ("CellWallParticleBegin", "CellWallParticleEnd")):
        assert _cell_sets(gi, g.export(b), g.export(e)) == _cell_sets(oi, o.array(b), o.array(e))
    o.neighbors(); g.stage("neighbors")
    for ptr, ind in (("NeighborPtr", "NeighborInd"), ("NeighborPtrP", "NeighborIndP")):
        assert _neighbour_sets(gi, g.export(ptr), g.export(ind)) == _neighbour_sets(oi, o.array(ptr), o.array(ind)), ind
    o.explicit(); o.assemble(); o.mg_build(); o.solve()
    for st in ("explicit", "assemble", "mg_build", "solve"):
        g.stage(st)
    nf = g.fluid_count
    vg = np.empty((len(gi), dim)); vg[gi] = vec_proj(g.export("Velocity"), dim)
    vo = np.empty((len(oi), dim)); vo[oi] = vec_proj(o.array("Velocity"), dim)
    fl = np.empty(len(oi), bool); fl[oi] = o.array("Property") < 2
    err = float(np.linalg.norm(vg[fl] - vo[fl]) / np.linalg.norm(vo[fl]))
    print(f"{name}: cells and neighbour sets equal; velocity by id {err:.2e}; "
          f"{int(np.sum(gi != oi))} of {len(gi)} positions ordered differently")
    assert abs(g.solve_stats()["iter"] - o.solve_stats()["iter"]) <= 2
    assert err <= 2e-5
    assert nf == int(np.sum(fl))


def test_counting_sort_is_deterministic(engine_lib):
    name, dim, params, parts = CASES[2]
    runs = []
    for _ in range(2):
        g = engine.Case(params, parts, dim)
        g.set_option("cell_sort", 1)
        g.step(3)
        runs.append((g.export("ParticleIndex"), g.export("Velocity"), g.export("NeighborInd")))
    for a, b in zip(*runs):
        assert np.array_equal(a, b)
