"""Autotuner for the mixed-precision pool.

Choices made by measurement rather than fixed in code:

* the kernel form of the step, by timing real steps of the pool's own
  scenarios: the separate flux, update, timestep, rate and clock kernels
  captured in the step graph with a persistent grid (at most 6 or at most 8
  blocks of 128 threads per SM: 80 or 64 registers per thread), the same with
  one block per tile, or the whole step as one cooperative kernel (grid
  barriers between its phases) at either register budget;
* whether the work records the flux kernels gather are kept resident in L2
  (an access policy window), timed with the chosen form;
* the cell ordering of every mesh (Hilbert or Morton curve), by the halo
  cost of the order (extra reconstructions per tile; tables.best_order), and,
  for a Batch, by timing steps of the pool built with each ordering
  (batch.Batch.tune_order).

The pool state is snapshotted before and restored after, so tuning leaves
the simulation untouched.
"""
from __future__ import annotations

import time

# (variant, grid mode): variant 0 = at most 6 blocks per SM, 1 = at most 8;
# grid mode 0 = persistent grid, 1 = one block per tile, 2 = one-kernel step
VARIANTS = [(0, 0), (0, 1), (1, 0), (1, 1), (0, 2), (1, 2)]
NAMES = {(0, 0): "b6-persistent", (0, 1): "b6-per-tile", (1, 0): "b8-persistent", (1, 1): "b8-per-tile",
         (0, 2): "b6-one-kernel", (1, 2): "b8-one-kernel"}


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


def tune_pool(pool, steps=10, reps=2, variants=VARIANTS, l2=True):
    """Time each kernel form on the pool's scenarios and keep the fastest;
    then the same form with the work records kept in L2 (l2=True).
    Returns {name: seconds per step} and the chosen name."""
    pool.snapshot()
    res = {}
    pool.set_l2_window(False)
    for v in variants:
        pool.set_variant(*v)
        _time_steps(pool, 1, 1)                       # build the graph once
        res[NAMES[v]] = _time_steps(pool, steps, reps) / steps
    best = min(res, key=res.get)
    v = [k for k, n in NAMES.items() if n == best][0]
    pool.set_variant(*v)
    if l2:
        try:
            pool.set_l2_window(True)
        except Exception:                             # no persisting L2 on this device
            pool.set_l2_window(False)
        else:
            _time_steps(pool, 1, 1)
            name = best + "+l2"
            res[name] = _time_steps(pool, steps, reps) / steps
            if res[name] < res[best]:
                best = name
            else:
                pool.set_l2_window(False)
    pool.restore()
    return res, best
