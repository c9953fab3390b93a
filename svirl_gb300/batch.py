"""Batched engine: many GL instances of uneven sizes advanced together on one GPU.

    from svirl_gb300 import GLSolver
    from svirl_gb300.batch import GLBatch
    solvers = [GLSolver(...), GLSolver(...), ...]      # any sizes / parameters, one dtype
    batch = GLBatch(solvers)
    stats = batch.td(dt=0.1, Nt=2000)                  # one device-side loop for all
    batch.cg(n_iter=1000, gtol=1e-6)                   # device CG, every instance at once

The TD call runs every instance's time loop and Jacobi loops inside one CUDA
graph launch: one sweep launch covers all instances (concatenated item tables,
per-instance descriptors), each instance keeps the reference's own Jacobi stop
rule and buffer bookkeeping, so each ends in exactly the state it reaches when
run alone.  The device CG runs the minimisation of every instance in one graph
launch, with beta, the step lengths and the stop test decided on the device.
The reference has no batched mode (one solver per process).

``HandleBatch`` is the same engine over raw library handles (``_lib.Handle``),
for code that manages instances itself (dataset generation, serving).
"""
import ctypes as C

import numpy as np

from . import _lib

CG_EXACT_BOUNDARY = 1
CG_GTOL_ABS = 2


class HandleBatch:
    """A batch over ``_lib.Handle`` objects (one dtype, one device)."""

    def __init__(self, handles):
        self.handles = list(handles)
        if not self.handles:
            raise ValueError("a batch needs at least one instance")
        if len({h.dtype for h in self.handles}) != 1:
            raise ValueError("all instances of a batch must have the same dtype")
        self.lib = _lib.load()
        n = len(self.handles)
        arr = (C.c_void_p * n)(*[h.h.value for h in self.handles])
        b = C.c_void_p()
        rc = self.lib.glgpu_batch_create(arr, n, C.byref(b))
        if rc != 0:
            raise _lib.GLGPUError("glgpu_batch_create failed (%d): %s" % (rc, self.lib.glgpu_last_error(None).decode()))
        self.b = b
        self.last_stats = None

    def close(self):
        if getattr(self, "b", None):
            self.lib.glgpu_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc == 0:
            return
        msg = self.lib.glgpu_batch_last_error(self.b)
        msg = msg.decode() if msg else ""
        if rc == _lib.GLGPU_E_NAN:
            import warnings
            warnings.warn("glgpu: %s: %s" % (what, msg), RuntimeWarning, stacklevel=3)
            return
        raise _lib.GLGPUError("glgpu error %d in %s: %s" % (rc, what, msg))

    def set_use_graphs(self, enable):
        self._check(self.lib.glgpu_batch_set_use_graphs(self.b, 1 if enable else 0), "set_use_graphs")

    def set_loop_guard(self, launches):
        """Jacobi loop guard in sweep launches (0: the default of 1088)."""
        self._check(self.lib.glgpu_batch_set_loop_guard(self.b, int(launches)), "set_loop_guard")

    def td_raw(self, dt, Nt, eqn=0, timed=False):
        """``glgpu_batch_td``: eqn 0 = both equations, 1 = psi only, 2 = A only."""
        st = _lib.TDStats()
        ms = C.c_double()
        self._check(self.lib.glgpu_batch_td(self.b, float(dt), int(Nt), int(eqn), C.byref(st), C.byref(ms)), "batch_td")
        self.last_stats = st
        return (st, ms.value) if timed else st

    def set_energy_targets(self, targets, rel_tol=1e-6):
        """Per-instance energy targets for the next device CG calls (None clears):
        an instance also stops, with status 4, once E <= target + rel_tol |target|."""
        if targets is None:
            self._check(self.lib.glgpu_batch_set_energy_targets(self.b, None, 0.0), "set_energy_targets")
            return
        t = np.ascontiguousarray(targets, dtype=np.float64)
        assert t.size == len(self.handles)
        self._check(self.lib.glgpu_batch_set_energy_targets(self.b, t.ctypes.data_as(C.c_void_p), float(rel_tol)),
                    "set_energy_targets")

    def set_cg_window(self, window, rel_tol=0.0):
        """Energy-window stop for the next device CG calls: every `window`
        iterations an instance stops, with status 5, unless its energy fell by more
        than rel_tol |E| since `window` iterations before (window 0: off)."""
        self._check(self.lib.glgpu_batch_set_cg_window(self.b, int(window), float(rel_tol)), "set_cg_window")

    def cg_device(self, n_iter=1000, rtol=1e-6, gtol=0.0, exact_boundary=False, gtol_abs=False, timed=False):
        """``glgpu_batch_cg``; returns per-instance arrays (see ``GLBatch.cg``)."""
        n = len(self.handles)
        iters = (C.c_int32 * n)()
        energy = (C.c_double * n)()
        grad_rel = (C.c_double * n)()
        status = (C.c_int32 * n)()
        ms = C.c_double()
        flags = (CG_EXACT_BOUNDARY if exact_boundary else 0) | (CG_GTOL_ABS if gtol_abs else 0)
        rc = self.lib.glgpu_batch_cg(self.b, int(n_iter), float(rtol), float(gtol), flags, iters, energy, grad_rel,
                                     status, C.byref(ms))
        self._check(rc, "batch_cg")
        out = {"iters": np.array(iters[:], dtype=np.int32), "energy": np.array(energy[:]),
               "grad_rel": np.array(grad_rel[:]), "status": np.array(status[:], dtype=np.int32)}
        if timed:
            out["ms"] = ms.value
        return out


class GLBatch(HandleBatch):
    """A batch of ``GLSolver`` instances."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        if not self.solvers:
            raise ValueError("GLBatch needs at least one solver")
        if len({s.cfg.dtype for s in self.solvers}) != 1:
            raise ValueError("all solvers of a batch must have the same dtype")
        super().__init__([s._h for s in self.solvers])

    def td(self, dt=0.1, Nt=1000, eqn=None, timed=False):
        """``solve.td(dt, Nt, eqn=eqn)`` of every solver, in one device loop."""
        code = {None: 0, "order_parameter": 1, "vector_potential": 2}[eqn]
        for s in self.solvers:
            s.solve._init_td()
            td = s.solve._td
            if eqn in (None, "order_parameter"):
                td._set_iterator_options("order_parameter", Nt, dt, None)
            if eqn in (None, "vector_potential"):
                td._set_iterator_options("vector_potential", Nt, dt, None)
            if eqn == "vector_potential" and td.dt is None:
                raise TypeError("vector-potential steps use the order-parameter dt, which is not set yet")
        dt_used = self.solvers[0].solve._td.dt
        out = self.td_raw(dt_used, Nt, code, timed=timed)
        for s in self.solvers:
            s.solve.vortices_detected = False
        return out

    def free_energies(self):
        return np.array([s.observables.free_energy for s in self.solvers])

    def cg(self, n_iter=1000, rtol=None, gtol=0.0, mode="device", exact_boundary=False, gtol_abs=False, timed=False):
        """Free-energy minimisation of every solver.

        ``mode="device"``: one graph launch runs the CG of all instances; beta,
        the step lengths and the stop test are decided on the device (see
        ``glgpu_batch_cg``).  Stops per instance after ``n_iter`` updates, on the
        reference's energy-ratio test with ``rtol`` (default: the first
        solver's ``convergence_rtol``) or when the gradient norm falls below
        ``gtol`` times its first value (``gtol_abs``: below ``gtol``).  Returns
        a dict of per-instance arrays ``iters``, ``energy``, ``grad_rel``,
        ``status`` (and ``ms`` if ``timed``).  ``exact_boundary``: use the exact
        dF/dA on the boundary links (the reference's formula doubles it there,
        so at finite kappa its gradient norm stalls above zero at the energy
        minimum).

        ``mode="reference"``: ``solve.cg(n_iter)`` of each solver in turn, the
        reference's decisions taken on the host."""
        if mode == "reference":
            for s in self.solvers:
                s.solve.cg(n_iter=n_iter)
            return None
        if mode != "device":
            raise ValueError("mode must be 'device' or 'reference'")
        if rtol is None:
            rtol = self.solvers[0].cfg.convergence_rtol
        try:
            return self.cg_device(n_iter, rtol, gtol, exact_boundary=exact_boundary, gtol_abs=gtol_abs, timed=timed)
        finally:
            for s in self.solvers:
                s.solve.vortices_detected = False
