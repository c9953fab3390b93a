"""Measured choice of the psi sweep's launch shape, persisted per problem.

The psi sweep kernel is compiled for the strip heights in ``STRIP_ROWS`` and,
in FP32, as two kernels (register strip, bulk-copy ring).  By default a handle
takes the height an item-count model picks.  ``tune(handle)`` measures instead:
it times one sweep launch (``glgpu_time_sweeps``: CUDA events, L2 flushed
before each launch) for every (kernel, height) pair, applies the fastest, and
stores it in a JSON cache keyed by (dtype, Nx, Ny, kappa finite), so that later
handles with the same key take the stored choice without measuring.  Results
do not depend on the choice: every pair computes the same values bitwise
(tests/test_gpu_strip_rows.py, tests/test_gpu_psi_kernels.py).

The cache file is ``$SVIRL_GB300_TUNE_CACHE`` or ``~/.cache/svirl_gb300/psi_sweep.json``.
No counterpart in the reference, whose kernels have one fixed launch shape
(128-thread blocks, svirl/parallel/startup.py:65).
"""
import json
import os

import numpy as np

STRIP_ROWS = (8, 12, 17)  # the heights libglgpu compiles the sweep for
KERNELS_FP32 = (0, 1)     # 0 register strip, 1 bulk-copy ring (glgpu_set_psi_sweep_kernel)


def cache_path():
    p = os.environ.get("SVIRL_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "svirl_gb300", "psi_sweep.json")


def key_of(handle):
    return "%s:%dx%d:%s" % (np.dtype(handle.dtype).name, handle.Nx, handle.Ny,
                            "finite" if handle.kappa_finite() else "inf")


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(handle, choice):
    handle.set_psi_sweep_kernel(int(choice["kernel"]))
    handle.set_psi_strip_rows(int(choice["rows"]))


def tune(handle, reps=5, path=None, force=False):
    """Measure (or look up) and apply the fastest psi sweep launch shape for
    `handle`; returns the choice {"kernel", "rows", "us", "measured": {...}}."""
    path = path or cache_path()
    table = _load(path)
    key = key_of(handle)
    if not force and key in table:
        apply(handle, table[key])
        return dict(table[key], cached=True)
    kernels = KERNELS_FP32 if np.dtype(handle.dtype) == np.float32 else (0,)
    measured = {}
    for kern in kernels:
        for rows in STRIP_ROWS:
            handle.set_psi_sweep_kernel(kern)
            handle.set_psi_strip_rows(rows)
            handle.time_sweeps(0, 1)  # warm-up launch
            measured["%d/%d" % (kern, rows)] = 1e3 * handle.time_sweeps(0, reps)
    best = min(measured, key=measured.get)
    kern, rows = (int(x) for x in best.split("/"))
    choice = {"kernel": kern, "rows": rows, "us": measured[best], "measured": measured}
    apply(handle, choice)
    table[key] = choice
    _store(path, table)
    return dict(choice, cached=False)
