"""Autotuner for the mixed-precision pool.

Two kinds of choices are made by measurement rather than fixed in code:

* the cell ordering (Hilbert or Morton curve) of every mesh, by the halo
  cost of the order (extra reconstructions per tile; tables.best_order);
* the fused flux kernel variant (register cap 80 with 3 blocks/SM, or 64 with
  4 blocks/SM and spills) and the grid mode (persistent grid of #SMs x blocks,
  or one block per tile), by timing a few real steps of the pool's own
  scenarios.  The pool state is snapshotted before and restored after, so
  tuning leaves the simulation untouched.
"""
from __future__ import annotations

import time

VARIANTS = [(0, 0), (0, 1), (1, 0), (1, 1)]
NAMES = {(0, 0): "r80-persistent", (0, 1): "r80-per-tile", (1, 0): "r64-persistent", (1, 1): "r64-per-tile"}


def _time_steps(pool, steps, reps):
    sids = pool.scenarios()
    best = float("inf")
    for _ in range(reps):
        pool.restore()
        for s in sids:
            st = pool.stats(s)
            pool.set_clock(s, st.time, 1e300, -1.0, steps)
        t0 = time.perf_counter()
        pool.advance()          # synchronous: returns after the graph completes
        best = min(best, time.perf_counter() - t0)
    return best


def tune_pool(pool, steps=10, reps=2, variants=VARIANTS):
    """Time each kernel variant on the pool's scenarios and keep the fastest.
    Returns {name: seconds per step} and the chosen name."""
    pool.snapshot()
    res = {}
    for v in variants:
        pool.set_variant(*v)
        _time_steps(pool, 1, 1)                       # build the graph once
        res[NAMES[v]] = _time_steps(pool, steps, reps) / steps
    best = min(res, key=res.get)
    v = [k for k, n in NAMES.items() if n == best][0]
    pool.set_variant(*v)
    pool.restore()
    return res, best
