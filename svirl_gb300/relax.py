"""Relaxation engine: sampled GL instances of mixed sizes relaxed together by
the batched device CG (and, optionally, batched TDGL first), with library
handles reused across batches.  Used by the states/s benchmark, the learned
warm start's dataset generation and evaluation, and the serving loop.  No
counterpart in the reference (one solver per process, svirl/config.py).
"""
import numpy as np

from . import _lib
from .batch import HandleBatch


class HandleCache:
    """Library handles kept per (n, dtype) and handed out again after release."""

    def __init__(self, device=0, dx=0.5):
        self.device, self.dx = device, dx
        self.free = {}
        self.all = []

    def get(self, n, dtype):
        key = (int(n), np.dtype(dtype).str)
        lst = self.free.setdefault(key, [])
        if lst:
            return lst.pop()
        h = _lib.Handle(n, n, self.dx, self.dx, dtype, device=self.device)
        self.all.append(h)
        return h

    def put(self, h):
        self.free.setdefault((h.Nx, h.dtype.str), []).append(h)

    def close(self):
        for h in self.all:
            h.close()
        self.all, self.free = [], {}


def relax(insts, cache, dtype=np.float32, starts=None, n_iter=4000, gtol=1e-4, gtol_abs=True, rtol=0.0,
          td_steps=0, td_dt=0.1, fetch=True, timed=True, targets=None, target_tol=1e-6, window=0, window_tol=0.0,
          graphs=True):
    """Load `insts` (learned.Instance, any sizes) into handles, optionally run
    `td_steps` TDGL steps, then the device CG (exact boundary gradient) of all of
    them in one batch; with `targets`, an instance also stops once its energy is
    within `target_tol` of its target; with `window` > 0, once its energy fell by
    no more than `window_tol` |E| over `window` iterations; graphs=False runs the
    host-driven loop (the same kernels).  Returns (cg dict with per-instance arrays
    and 'ms', [(psi, ab)] if fetch, td_ms)."""
    hs = [cache.get(it.n, dtype) for it in insts]
    try:
        for q, (it, h) in enumerate(zip(insts, hs)):
            if starts is None:
                it.load_into(h)
            else:
                it.load_into(h, psi=starts[q][0], ab=starts[q][1])
        batch = HandleBatch(hs)
        try:
            td_ms = 0.0
            if targets is not None:
                batch.set_energy_targets(targets, target_tol)
            if window > 0:
                batch.set_cg_window(window, window_tol)
            if not graphs:
                batch.set_use_graphs(False)
            if td_steps > 0:
                _, td_ms = batch.td_raw(td_dt, td_steps, 0, timed=True)
            out = batch.cg_device(n_iter=n_iter, rtol=rtol, gtol=gtol, exact_boundary=True, gtol_abs=gtol_abs,
                                  timed=timed)
        finally:
            batch.close()
        states = [(h.get_psi(), h.get_ab()) for h in hs] if fetch else None
        return out, states, td_ms
    finally:
        for h in hs:
            cache.put(h)


def polish_fp64(insts, states, cache, n_iter, gtol, window=0, window_tol=0.0):
    """Finish FP32-relaxed states in float64: each (psi, ab) state goes into a
    float64 handle and one batched device CG (exact-boundary gradient, absolute
    gradient tolerance gtol, at most n_iter iterations) runs from it.  A state
    stored in FP32 cannot meet an absolute gradient tolerance below the gradient
    of its own rounding; the FP64 iterations remove that.  Returns (cg dict with
    'ms', [(psi, ab)] in float64)."""
    hs = [cache.get(it.n, np.float64) for it in insts]
    try:
        for it, h, (psi, ab) in zip(insts, hs, states):
            it.load_into(h, psi=np.asarray(psi, np.complex128), ab=np.asarray(ab, np.float64))
        batch = HandleBatch(hs)
        try:
            if window > 0:
                batch.set_cg_window(window, window_tol)
            out = batch.cg_device(n_iter=n_iter, rtol=0.0, gtol=gtol, exact_boundary=True, gtol_abs=True,
                                  timed=True)
        finally:
            batch.close()
        return out, [(h.get_psi(), h.get_ab()) for h in hs]
    finally:
        for h in hs:
            cache.put(h)


def energies_fp64(insts, states, cache):
    """Free energy of each (psi, ab) state evaluated in float64."""
    E = np.empty(len(insts))
    for q, (it, (psi, ab)) in enumerate(zip(insts, states)):
        h = cache.get(it.n, np.float64)
        try:
            it.load_into(h, psi=np.asarray(psi, np.complex128), ab=np.asarray(ab, np.float64))
            E[q] = h.free_energy()
        finally:
            cache.put(h)
    return E


def gradient_ok_fp64(insts, states, cache, gtol):
    """Whether each (psi, ab) state meets the device CG's absolute gradient
    tolerance |grad F| <= gtol (exact-boundary gradient), evaluated in float64:
    the state is loaded into a float64 handle and a one-iteration CG stops at
    iteration 0 with status 1 exactly when the tolerance holds."""
    ok = np.zeros(len(insts), dtype=bool)
    for q, (it, (psi, ab)) in enumerate(zip(insts, states)):
        h = cache.get(it.n, np.float64)
        try:
            it.load_into(h, psi=np.asarray(psi, np.complex128), ab=np.asarray(ab, np.float64))
            b = HandleBatch([h])
            try:
                out = b.cg_device(n_iter=1, rtol=0.0, gtol=gtol, exact_boundary=True, gtol_abs=True)
            finally:
                b.close()
            ok[q] = int(out["status"][0]) == 1 and int(out["iters"][0]) == 0
        finally:
            cache.put(h)
    return ok
