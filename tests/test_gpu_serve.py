"""The serving loop (continuous batching of TDGL + CG requests) on a short seeded
Poisson trace: every request completes, and each answer is bitwise the answer
of the same request run alone (one instance, the same TDGL length and the same
CG chunks), whatever else shared its batches.  Mixed kappa (finite and inf) and
mixed FP32 / FP64 requests, handles reused between requests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(req, td_steps, cg_chunk, cg_cap, rtol, dt):
    from svirl_gb300.batch import HandleBatch
    from svirl_gb300.relax import HandleCache
    cache = HandleCache()
    try:
        h = cache.get(req.n, req.dtype)
        req.inst.load_into(h)
        b = HandleBatch([h])
        b.td_raw(dt, td_steps, 0)
        iters = 0
        while True:
            out = b.cg_device(n_iter=cg_chunk, rtol=rtol, gtol=0.0, exact_boundary=True)
            iters += int(out["iters"][0])
            if out["status"][0] in (1, 2) or iters >= cg_cap:
                break
        b.close()
        return h.get_psi(), float(out["energy"][0]), iters
    finally:
        cache.close()


def test_poisson_trace_completes_and_matches_requests_run_alone():
    from svirl_gb300 import serve as S
    reqs = S.poisson_requests(10, 500.0, seed=11, sizes=(24, 56))
    assert {r.dtype for r in reqs} == {np.float32, np.float64}
    assert any(np.isinf(r.kappa) for r in reqs) and any(np.isfinite(r.kappa) for r in reqs)
    kw = dict(td_steps=24, td_chunk=10, cg_chunk=40, cg_cap=200, rtol=1e-6)
    eng = S.Engine(max_active_nodes=3 * 56 * 56, **kw)  # a small node budget: admission waits, handles are reused
    try:
        done, wall = eng.run(reqs, max_wall_s=300.0)
    finally:
        eng.close()
    assert sorted(a["req"].rid for a in done) == list(range(len(reqs)))
    summ = S.summarize(done, wall)
    assert summ["completed"] == len(reqs) and summ["latency_s"]["p99"] >= summ["latency_s"]["p50"] > 0
    for a in done:
        r = a["req"]
        psi, energy, iters = _alone(r, kw["td_steps"], kw["cg_chunk"], kw["cg_cap"], kw["rtol"], 0.1)
        assert iters == a["cg_iters"], r.rid
        assert np.array_equal(psi, a["psi"]), r.rid
        assert energy == a["energy"], r.rid
