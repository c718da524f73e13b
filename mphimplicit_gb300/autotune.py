"""Autotuner of the mixed form's launch shapes (block and chunk widths).

Three launch shapes of the mixed form are runtime options of a case:

* ``pair_block``: threads a block of the pair-term operator (k_visc_pen32,
  k_resid_pairs), which is also the row block whose distinct neighbours'
  values it stages in shared memory (128, 256, 512);
* ``ct_block``: threads a block of the transposed P-list apply
  (k_ct_apply32) and its staged particle block (128, 256);
* ``chunk``: CR iterations in one captured CUDA-graph chunk, i.e. how often
  the host reads the solver's flags (4, 8, 16, 32).

``tune`` times whole steps of fresh copies of a case for each candidate by
coordinate descent (one option at a time, the others at their best so far)
and returns the fastest settings with every timing.  ``tune_table`` does this
for one case of each size class (dimension and octave of the fluid count) of
a workload and ``choose`` picks a case's settings from such a table, so that
cases run measured settings deterministically: the block widths set the
order in which the dot products' block partial sums add up, so the settings
(not the timings of the moment) decide a case's bits.
"""
from __future__ import annotations

import json
import math
import time
from typing import Callable, Dict, Iterable, Optional

DEFAULTS = {"pair_block": 512, "ct_block": 256, "chunk": 8}
CANDIDATES = (("pair_block", (512, 256, 128)), ("ct_block", (256, 128)), ("chunk", (8, 4, 16, 32)))


def apply(case, settings: Dict[str, int]) -> None:
    for k, v in settings.items():
        case.set_option(k, v)


def _ms_per_step(make_case: Callable, settings: Dict[str, int], steps: int, warmup: int) -> float:
    c = make_case()
    try:
        apply(c, settings)
        c.step(warmup)
        t0 = time.perf_counter()
        c.step(steps)   # a step ends with the host reading its solve's results
        return (time.perf_counter() - t0) * 1000.0 / steps
    finally:
        c.close()


MARGIN = 0.03   # a candidate replaces the current setting only when this much faster (timing noise)


def tune(make_case: Callable, steps: int = 3, warmup: int = 2, candidates=CANDIDATES, margin: float = MARGIN) -> Dict:
    """Coordinate descent over `candidates` on fresh cases from make_case()
    (every trial starts from the same state): the fastest settings and the
    milliseconds per step of every trial.  A setting leaves its current value
    only for a candidate at least `margin` faster."""
    best = dict(DEFAULTS)
    timings: Dict[tuple, float] = {}
    for name, values in candidates:
        res = {}
        for v in values:
            trial = dict(best)
            trial[name] = v
            key = tuple(sorted(trial.items()))
            if key not in timings:
                timings[key] = _ms_per_step(make_case, trial, steps, warmup)
            res[v] = timings[key]
        fastest = min(res, key=res.get)
        if res[fastest] < (1.0 - margin) * res[best[name]]:
            best[name] = fastest
    return {"settings": best,
            "ms_per_step": {",".join(f"{k}={v}" for k, v in key): round(ms, 3) for key, ms in timings.items()},
            "steps": steps, "warmup": warmup}


def size_class(dim: int, fluid: int) -> str:
    return f"{dim}d:{int(round(math.log2(max(fluid, 1))))}"


def tune_table(cases: Iterable, make: Callable, steps: int = 3, warmup: int = 2) -> Dict[str, Dict]:
    """One tuning per size class: `cases` yields (dim, fluid count, key) and
    make(key) builds a fresh case of that key."""
    table: Dict[str, Dict] = {}
    for dim, fluid, key in cases:
        cls = size_class(dim, fluid)
        if cls in table:
            continue
        table[cls] = tune(lambda: make(key), steps, warmup)
    return table


def choose(table: Optional[Dict[str, Dict]], dim: int, fluid: int) -> Dict[str, int]:
    """The settings of the case's size class, else of the nearest class of the
    same dimension, else the defaults."""
    if not table:
        return dict(DEFAULTS)
    cls = size_class(dim, fluid)
    if cls in table:
        return dict(table[cls]["settings"])
    same = [k for k in table if k.startswith(f"{dim}d:")]
    if not same:
        return dict(DEFAULTS)
    octave = int(cls.split(":")[1])
    near = min(same, key=lambda k: abs(int(k.split(":")[1]) - octave))
    return dict(table[near]["settings"])


def save(table: Dict, path: str) -> None:
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)


def load(path: str) -> Dict:
    with open(path) as f:
        return json.load(f)
