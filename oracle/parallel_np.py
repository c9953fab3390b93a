"""The oracle's TD time loop at kappa = inf on all host cores: one domain split into
row blocks, one process per block, shared memory between them.

TEST INFRASTRUCTURE ONLY: the reference arm of ``bench.py`` times the reference's
arithmetic on the host with it, and ``tests/test_oracle_parallel.py`` checks it
against the single-process oracle.  Nothing in the product imports it.

The reference has no CPU implementation of this path; its arithmetic on the host
is the oracle's (``oracle/kernels_np.py``, a restatement of
``svirl/cuda/td.h:4-133``), here with the host loop of
``svirl/solvers/td.py:157-200,342-377`` (right-hand side = psi at the start of
the step, Jacobi sweeps until ``1e-4*code < 1`` or 1024 sweeps).  Process k owns
node rows [j0, j1) and reads one halo row on each side from the shared psi
buffer; a sweep writes only owned rows into the other buffer, so every node gets
exactly the single-domain value (a psi sweep reads only a node's four
neighbours).  Each process publishes the residual code of its rows; after one
barrier per sweep all processes take the same maximum and the same stop
decision.  The codes are double-buffered by sweep parity, so one barrier per
sweep suffices: a process writes a psi buffer only after every process has
finished reading it in the previous sweep.
"""
import multiprocessing as mp
import os
import time
from multiprocessing import shared_memory

import numpy as np

from oracle import kernels_np as K

MAX_SWEEPS = 1024  # svirl/solvers/td.py:164


def _rows(Ny, P, k):
    edges = [round(q * Ny / P) for q in range(P + 1)]
    j0, j1 = edges[k], edges[k + 1]
    return j0, j1, max(0, j0 - 1), min(Ny, j1 + 1)


def _attach(name, shape, dtype):
    shm = shared_memory.SharedMemory(name=name)
    return shm, np.ndarray(shape, dtype=dtype, buffer=shm.buf)


def _worker(k, P, spec, names, bar_sweep, bar_step, nsteps, out_q):
    os.environ["OMP_NUM_THREADS"] = "1"
    Nx, Ny, dx, dy, dt, stop, has_mt = spec
    N, Nab = Nx * Ny, (Nx - 1) * Ny + Nx * (Ny - 1)
    handles = []

    def att(key, shape, dtype):
        shm, a = _attach(names[key], shape, dtype)
        handles.append(shm)
        return a

    psi = [att("psi0", (Ny, Nx), np.complex128), att("psi1", (Ny, Nx), np.complex128)]
    rhs = att("rhs", (Ny, Nx), np.complex128)
    ab = att("ab", (Nab,), np.float64)
    codes = att("codes", (2, P), np.int64)
    mt = att("mt", (Ny - 1, Nx - 1), np.bool_) if has_mt else None
    j0, j1, lo, hi = _rows(Ny, P, k)
    g = K.Grid(Nx, hi - lo, dx, dy)
    Na = (Nx - 1) * Ny
    a2 = ab[:Na].reshape(Ny, Nx - 1)
    b2 = ab[Na:].reshape(Ny - 1, Nx)
    ab_loc = np.concatenate([a2[lo:hi].reshape(-1), b2[lo:hi - 1].reshape(-1)])
    mt_loc = None if mt is None else np.ascontiguousarray(mt[lo:hi - 1]).reshape(-1)
    own = slice(j0 - lo, j1 - lo)
    dtype = np.float64
    cur, par = 0, 0
    sweeps = []
    with np.errstate(all="ignore"):
        for _ in range(nsteps):
            rhs[j0:j1] = psi[cur][j0:j1]  # a sweep reads the right-hand side at its own node only
            n = 0
            while True:
                P_loc = psi[cur][lo:hi].reshape(-1)
                nxt, _ = K.iterate_order_parameter_jacobi_step(g, dt, 1.0, None, mt_loc, ab_loc,
                                                               rhs[lo:hi].reshape(-1).copy(), P_loc, 0.0, n, 1, stop)
                nxt = nxt.reshape(hi - lo, Nx)[own]
                old = psi[cur][j0:j1]
                r = np.fmax(np.abs(nxt.real - old.real), np.abs(nxt.imag - old.imag))
                psi[1 - cur][j0:j1] = nxt
                codes[par, k] = int(K.residual_code(r, stop).max()) if r.size else 0
                bar_sweep.wait()
                code = int(codes[par].max())
                cur, par, n = 1 - cur, 1 - par, n + 1
                if 1.0e-4 * dtype(code) < 1.0 or n >= MAX_SWEEPS:
                    break
            sweeps.append(n)
            bar_step.wait()
    if k == 0:
        out_q.put((sweeps, cur))
    for h in handles:
        h.close()


class SharedTD:
    """One kappa = inf TD trajectory of an (Nx, Ny) domain on P processes.

    ``run(nsteps, on_step)`` advances ``nsteps`` steps; ``on_step(s)`` is called by
    the parent after each step's barrier (the timing hook).  ``psi()`` returns the
    state as the oracle's flat complex array."""

    def __init__(self, Nx, Ny, dx, dy, psi0, ab, mt=None, dt=0.1, stop=1e-6, processes=None):
        self.Nx, self.Ny, self.dx, self.dy, self.dt, self.stop = Nx, Ny, float(dx), float(dy), float(dt), float(stop)
        self.P = max(1, min(processes or len(os.sched_getaffinity(0)), Ny // 2))
        self._shm, self.names, self.arrays = [], {}, {}
        N, Nab = Nx * Ny, (Nx - 1) * Ny + Nx * (Ny - 1)
        self._new("psi0", (Ny, Nx), np.complex128)[:] = np.asarray(psi0, dtype=np.complex128).reshape(Ny, Nx)
        self._new("psi1", (Ny, Nx), np.complex128)[:] = 0.0
        self._new("rhs", (Ny, Nx), np.complex128)[:] = 0.0
        self._new("ab", (Nab,), np.float64)[:] = np.asarray(ab, dtype=np.float64).reshape(-1)
        self._new("codes", (2, self.P), np.int64)[:] = 0
        self.has_mt = mt is not None
        if self.has_mt:
            self._new("mt", (Ny - 1, Nx - 1), np.bool_)[:] = np.asarray(mt, dtype=bool).reshape(Ny - 1, Nx - 1)
        self.cur = 0
        self.sweeps = []
        del N

    def _new(self, key, shape, dtype):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        shm = shared_memory.SharedMemory(create=True, size=max(nbytes, 1))
        self._shm.append(shm)
        self.names[key] = shm.name
        a = np.ndarray(shape, dtype=dtype, buffer=shm.buf)
        self.arrays[key] = a
        return a

    def run(self, nsteps, on_step=None, timeout_s=900.0):
        ctx = mp.get_context("spawn")
        bar_sweep = ctx.Barrier(self.P, timeout=timeout_s)
        bar_step = ctx.Barrier(self.P + 1, timeout=timeout_s)
        q = ctx.Queue()
        if self.cur == 1:  # keep the state in psi0 between runs
            self.arrays["psi0"][:] = self.arrays["psi1"]
            self.cur = 0
        spec = (self.Nx, self.Ny, self.dx, self.dy, self.dt, self.stop, self.has_mt)
        procs = [ctx.Process(target=_worker, args=(k, self.P, spec, self.names, bar_sweep, bar_step, nsteps, q))
                 for k in range(self.P)]
        for p in procs:
            p.start()
        try:
            for s in range(nsteps):
                bar_step.wait()
                if on_step is not None:
                    on_step(s)
            sweeps, cur = q.get(timeout=timeout_s)
        finally:
            for p in procs:
                p.join(timeout=60)
                if p.is_alive():
                    p.terminate()
        self.sweeps.extend(sweeps)
        self.cur = cur
        return sweeps

    def psi(self):
        return self.arrays["psi%d" % self.cur].reshape(-1).copy()

    def close(self):
        for shm in self._shm:
            shm.close()
            shm.unlink()
        self._shm = []


def timed_steps(td, warmup, steps):
    """Advance ``warmup`` untimed then ``steps`` timed steps in one run of the
    processes; returns the wall seconds of the timed steps."""
    marks = {}

    def on_step(s):
        if s == warmup - 1:
            marks["t0"] = time.perf_counter()
        if s == warmup + steps - 1:
            marks["t1"] = time.perf_counter()

    t_start = time.perf_counter()
    td.run(warmup + steps, on_step)
    return marks["t1"] - marks.get("t0", t_start)
