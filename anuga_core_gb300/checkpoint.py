"""Restart from a checkpoint (shallow_water/checkpoint.py).

``Domain.set_checkpointing(checkpoint_dir=..., checkpoint_step=...)`` pickles
the domain at yieldsteps as ``<dir>/<name>_<time>.pickle``;
``load_checkpoint_file(domain_name, checkpoint_dir, time=None)`` loads the
latest one (or the one at ``time``) that opens, and the next ``evolve`` call
continues from its time on the device.
"""
from __future__ import annotations

import os
import pickle
import time as _time


def _checkpoint_times(domain_name, checkpoint_dir):
    times = set()
    for path, dirs, files in os.walk(checkpoint_dir):
        for fn in files:
            base, ext = os.path.splitext(fn)
            if ext != ".pickle":
                continue
            name, _, t = base.rpartition("_")
            if name == domain_name:
                try:
                    times.add(float(t))
                except ValueError:
                    pass
        break
    return sorted(times)


def load_checkpoint_file(domain_name="domain", checkpoint_dir=".", time=None):
    times = [float(time)] if time is not None else _checkpoint_times(domain_name, checkpoint_dir)
    for t in reversed(times):
        name = os.path.join(checkpoint_dir, domain_name) + "_" + str(t) + ".pickle"
        try:
            with open(name, "rb") as fh:
                domain = pickle.load(fh)
        except Exception:
            continue
        domain.last_walltime = _time.time()
        return domain
    raise Exception("Unable to open checkpoint file")
