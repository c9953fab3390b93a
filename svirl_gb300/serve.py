"""Serving loop: GL solve requests arriving over time are admitted while device
memory allows, advanced together in batches (one batched TDGL chunk and one
batched device-CG chunk per engine step, one batch per dtype), and answered
when their CG has converged.  Device-resident state throughout; a request's
data crosses the host link once in each direction.  No counterpart in the
reference (one solver per process, no request handling).

Request: grid n x n nodes (dx = 0.5), kappa in [2, 10] or inf, float32 or
float64, H, a hole mask and a random start; TDGL for `td_steps` steps (dt
0.1), then the CG from the TDGL state until the reference's energy-ratio stop
(|E_k/E_{k-1} - 1| < rtol) or the iteration cap.
"""
import collections
import time

import numpy as np

from .batch import HandleBatch
from .learned import Instance
from .relax import HandleCache

Request = collections.namedtuple("Request", "rid arrival n kappa dtype inst")


def poisson_requests(count, rate_hz, seed=0, sizes=(64, 512), kappa_inf_prob=0.5):
    """`count` requests with exponential inter-arrival times (mean 1/rate), n ~ U{sizes},
    kappa ~ U[2, 10] or inf (50/50), float32 or float64 (50/50)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for r in range(count):
        t += rng.exponential(1.0 / rate_hz)
        n = int(rng.integers(sizes[0], sizes[1] + 1))
        dtype = np.float32 if rng.random() < 0.5 else np.float64
        inst = Instance.sample(n, rng, H_range=(0.02, 0.5), kappa_range=(2.0, 10.0), hole_frac=(0.0, 0.05),
                               radius=(2.0, 6.0), kappa_inf_prob=kappa_inf_prob)
        out.append(Request(r, t, n, inst.kappa, dtype, inst))
    return out


def instance_bytes(n, dtype):
    """Device bytes of one instance (TD buffers, link tables, CG buffers), with margin."""
    rs = np.dtype(dtype).itemsize
    N = n * n
    return int(1.25 * N * (6 * 2 * rs + 3 * rs * 2 + 2 * rs * 2 + 1 + 1 + 8 * 2 * rs * 2)) + (1 << 20)


class Engine:
    """Continuous batching of TDGL + CG requests."""

    def __init__(self, td_steps=500, td_chunk=50, cg_chunk=200, cg_cap=4000, rtol=1e-6, dt=0.1, reserve_bytes=8 << 30,
                 max_active_nodes=6_000_000, device=0):
        self.td_steps, self.td_chunk, self.cg_chunk, self.cg_cap = td_steps, td_chunk, cg_chunk, cg_cap
        self.max_active_nodes = max_active_nodes  # bounds a step's duration, hence latency
        self.rtol, self.dt, self.reserve = rtol, dt, reserve_bytes
        self.cache = HandleCache(device=device)
        self.active = []   # dicts: req, h, phase ('td' | 'cg'), td_left, cg_done, admitted
        self.done = []

    def _free_bytes(self):
        """Free device memory as the CUDA runtime reports it through torch.  Where
        torch cannot report it, admission rests on the active-node budget alone."""
        try:
            import torch
            free, _ = torch.cuda.mem_get_info()
            return free
        except Exception:  # noqa: BLE001
            return 1 << 40

    def admit(self, req, now):
        """Admit a waiting request if device memory (with a reserve) and the
        active-node budget allow it; first come, first served."""
        need = instance_bytes(req.n, req.dtype)
        active_nodes = sum(a["req"].n ** 2 for a in self.active)
        if self.active and active_nodes + req.n ** 2 > self.max_active_nodes:
            return False
        if self._free_bytes() - need < self.reserve:
            return False
        h = self.cache.get(req.n, req.dtype)
        req.inst.load_into(h)
        self.active.append({"req": req, "h": h, "phase": "td", "td_left": self.td_steps, "cg_iters": 0,
                            "admitted": now})
        return True

    def step(self):
        """One engine step: a TDGL chunk for the instances in TDGL, a CG chunk for
        those in CG, per dtype; returns the requests finished in this step."""
        finished = []
        for dt_ in (np.float32, np.float64):
            td = [a for a in self.active if a["phase"] == "td" and a["h"].dtype == np.dtype(dt_)]
            if td:
                nt = min(self.td_chunk, min(a["td_left"] for a in td))
                b = HandleBatch([a["h"] for a in td])
                try:
                    b.td_raw(self.dt, nt, 0)
                finally:
                    b.close()
                for a in td:
                    a["td_left"] -= nt
                    if a["td_left"] <= 0:
                        a["phase"] = "cg"
            cg = [a for a in self.active if a["phase"] == "cg" and a["h"].dtype == np.dtype(dt_)]
            if cg:
                b = HandleBatch([a["h"] for a in cg])
                try:
                    out = b.cg_device(n_iter=self.cg_chunk, rtol=self.rtol, gtol=0.0, exact_boundary=True)
                finally:
                    b.close()
                for a, it, st in zip(cg, out["iters"], out["status"]):
                    a["cg_iters"] += int(it)
                    if st in (1, 2) or a["cg_iters"] >= self.cg_cap:
                        a["phase"] = "done"
                        a["energy"] = float(out["energy"][cg.index(a)])
                        finished.append(a)
        for a in finished:
            a["psi"] = a["h"].get_psi()  # the answer leaves the device
            self.active.remove(a)
            self.cache.put(a["h"])
        return finished

    def run(self, requests, max_wall_s=60.0):
        """Serve `requests` in real time (arrival offsets from the start); returns the
        finished records (with 'latency') and the wall time."""
        t0 = time.perf_counter()
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting = collections.deque()
        while True:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            while waiting and self.admit(waiting[0], now):
                waiting.popleft()
            if not self.active:
                if not pending and not waiting:
                    break
                if pending and not waiting:
                    time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)))
                if now > max_wall_s:
                    break
                continue
            for a in self.step():
                a["finished"] = time.perf_counter() - t0
                a["latency"] = a["finished"] - a["req"].arrival
                self.done.append(a)
            if time.perf_counter() - t0 > max_wall_s:
                break
        return self.done, time.perf_counter() - t0

    def close(self):
        self.cache.close()


def summarize(done, wall):
    lat = np.array([a["latency"] for a in done]) if done else np.zeros(1)
    return {"completed": len(done), "wall_s": wall, "throughput_per_s": len(done) / wall if wall > 0 else 0.0,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                          "p99": float(np.percentile(lat, 99))},
            "mean_cg_iters": float(np.mean([a["cg_iters"] for a in done])) if done else 0.0}
