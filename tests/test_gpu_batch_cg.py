"""Batched device CG: the whole minimisation of every instance in one graph
launch, beta / step lengths / stop test decided on the device.

Checks: an instance's run does not depend on the rest of the batch (bitwise),
the graph and the host-driven loop agree (bitwise), the first iterations
follow the oracle's CG (kappa = inf: the same quartic roots, 1e-9; finite
kappa: BFGS on the host vs. Newton on the device, 1e-5), every update lowers
the energy, and the minimisation reaches the oracle CG's converged energy."""
import numpy as np
import pytest

from tests._pairs import gpu_state, make_pair, oracle_of, rel_err

pytestmark = pytest.mark.gpu

CONFIGS = [
    dict(Nx=33, Ny=17, kappa=np.inf, H=0.2, mask="holes", seed=1),
    dict(Nx=20, Ny=25, kappa=5.0, sigma=200.0, H=0.1, mask="random30", seed=2),
    dict(Nx=65, Ny=40, kappa=2.0, sigma=100.0, H=0.15, mask="none", seed=3),
    dict(Nx=9, Ny=9, kappa=np.inf, H=0.3, mask="q1", seed=4),
    dict(Nx=41, Ny=41, kappa=4.0, sigma=150.0, H=0.2, mask="holes", seed=5),
]


def _solvers(dtype=np.float64, configs=CONFIGS):
    pairs = [make_pair(dtype=dtype, **c) for c in configs]
    return [p[0] for p in pairs], [p[1] for p in pairs]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_cg_instance_independent_of_batch(dtype):
    from svirl_gb300.batch import GLBatch
    together, _ = _solvers(dtype)
    alone, _ = _solvers(dtype)
    out = GLBatch(together).cg(n_iter=25, rtol=0.0)
    for q, gl in enumerate(alone):
        o = GLBatch([gl]).cg(n_iter=25, rtol=0.0)
        assert o["iters"][0] == out["iters"][q]
        assert o["energy"][0] == out["energy"][q]
        pa, aa = gpu_state(gl)
        pb, ab = gpu_state(together[q])
        assert np.array_equal(pa, pb) and np.array_equal(aa, ab)


def test_batch_cg_graph_equals_host_loop():
    from svirl_gb300.batch import GLBatch
    a, _ = _solvers()
    b, _ = _solvers()
    ba, bb = GLBatch(a), GLBatch(b)
    bb.set_use_graphs(False)
    oa = ba.cg(n_iter=30, rtol=1e-9)
    ob = bb.cg(n_iter=30, rtol=1e-9)
    assert np.array_equal(oa["iters"], ob["iters"]) and np.array_equal(oa["energy"], ob["energy"])
    for ga, gb in zip(a, b):
        assert np.array_equal(gpu_state(ga)[0], gpu_state(gb)[0])
        assert np.array_equal(gpu_state(ga)[1], gpu_state(gb)[1])


def test_batch_cg_first_iterations_follow_oracle():
    from svirl_gb300.batch import GLBatch
    sol, orcs = _solvers()
    n = 4
    out = GLBatch(sol).cg(n_iter=n, rtol=0.0)
    assert np.all(out["iters"] == n) and np.all(out["status"] == 3)
    for q, (gl, orc) in enumerate(zip(sol, orcs)):
        orc.convergence_rtol = 0.0
        orc.cg(n_iter=n)
        tol = 1e-9 if np.isinf(CONFIGS[q]["kappa"]) else 1e-5
        p, a = gpu_state(gl)
        assert rel_err(p, orc.psi) < tol, q
        if orc.solveA:
            assert rel_err(a, orc.ab) < tol, q
        assert abs(out["energy"][q] / orc.cg_energies[-1] - 1.0) < tol, q


def test_batch_cg_spatial_linear_coefficient_follows_oracle():
    """A per-node linear coefficient reaches the batched CG (each instance's
    own field): first iterations against the oracle, and batch independence."""
    from svirl_gb300.batch import GLBatch
    cfgs = [CONFIGS[0], CONFIGS[1]]

    def build():
        sol, _ = _solvers(np.float64, cfgs)
        for q, gl in enumerate(sol):
            c = gl.cfg
            gl.params.linear_coefficient = 1.0 + 0.2 * np.random.default_rng(20 + q).random((int(c.Nx), int(c.Ny)))
        return sol

    sol = build()
    orcs = [oracle_of(gl, rand_t=1) for gl in sol]
    n = 4
    out = GLBatch(sol).cg(n_iter=n, rtol=0.0)
    for q, (gl, orc) in enumerate(zip(sol, orcs)):
        assert orc.epsilon_spatial is not None
        orc.convergence_rtol = 0.0
        orc.cg(n_iter=n)
        tol = 1e-9 if np.isinf(cfgs[q]["kappa"]) else 1e-5
        p, _ = gpu_state(gl)
        assert rel_err(p, orc.psi) < tol, q
        assert abs(out["energy"][q] / orc.cg_energies[-1] - 1.0) < tol, q
    alone = build()
    for q, gl in enumerate(alone):
        o = GLBatch([gl]).cg(n_iter=n, rtol=0.0)
        assert o["energy"][0] == out["energy"][q]


def test_batch_cg_monotone_energy():
    from svirl_gb300.batch import GLBatch
    sol, _ = _solvers()
    b = GLBatch(sol)
    E = np.array([gl.observables.free_energy for gl in sol])
    for _ in range(6):
        out = b.cg(n_iter=3, rtol=0.0)
        assert np.all(out["energy"] <= E + 1e-12 * np.abs(E)), (out["energy"], E)
        assert np.allclose(out["energy"], [gl.observables.free_energy for gl in sol], rtol=1e-12, atol=0)
        E = out["energy"]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_cg_converges_to_oracle_minimum(dtype):
    from svirl_gb300.batch import GLBatch
    cfgs = [CONFIGS[0], CONFIGS[1], CONFIGS[3]]
    sol, orcs = _solvers(dtype, cfgs)
    out = GLBatch(sol).cg(n_iter=3000, rtol=1e-12 if dtype == np.float64 else 1e-7)
    assert np.all(out["status"] > 0)
    for q, orc in enumerate(orcs):
        orc.convergence_rtol = 1e-12
        orc.dtype = np.float64
        orc.cg(n_iter=3000)
        tol = 1e-7 if dtype == np.float64 else 2e-4
        assert abs(out["energy"][q] / orc.cg_energies[-1] - 1.0) < tol, (q, out["energy"][q], orc.cg_energies[-1])


def test_batch_cg_gradient_stop_and_zero_iterations():
    from svirl_gb300.batch import GLBatch
    sol, _ = _solvers(configs=CONFIGS[:2])
    b = GLBatch(sol)
    E0 = np.array([gl.observables.free_energy for gl in sol])
    out = b.cg(n_iter=0)
    assert np.all(out["iters"] == 0)
    assert np.allclose(out["energy"], E0, rtol=1e-13, atol=0)
    # the reference's dF/dA doubles the magnetic terms on boundary links, so at
    # finite kappa its gradient norm stalls (energy-ratio stop only); with the
    # exact boundary derivative the gradient-norm stop is met
    ref, _ = _solvers(configs=CONFIGS[1:2])
    o_ref = GLBatch(ref).cg(n_iter=3000, rtol=0.0, gtol=1e-6)
    assert o_ref["status"][0] == 3 and o_ref["grad_rel"][0] > 1e-5
    out = b.cg(n_iter=5000, rtol=0.0, gtol=1e-6, exact_boundary=True)
    assert np.all(out["status"] == 1) and np.all(out["grad_rel"] <= 1e-6)
    assert np.all(out["iters"] < 5000)
    assert out["energy"][1] <= o_ref["energy"][0] + 1e-9 * abs(o_ref["energy"][0])


def test_batch_cg_independent_of_batch_at_every_tile_depth():
    """Instances large enough for each CG tile depth (2, 4, 8 nodes per thread),
    in one batch and alone: the same iterations bitwise."""
    from svirl_gb300 import learned as L
    from svirl_gb300.relax import HandleCache
    from svirl_gb300.batch import HandleBatch
    rng = np.random.default_rng(11)
    insts = [L.Instance.sample(n, rng, kappa_range=(4.0, 4.0)) for n in (129, 257, 385)]
    cache = HandleCache()
    try:
        hs = [cache.get(it.n, np.float32) for it in insts]
        for it, h in zip(insts, hs):
            it.load_into(h)
        together = HandleBatch(hs).cg_device(n_iter=20, rtol=0.0, gtol=0.0, exact_boundary=True)
        states = [(h.get_psi(), h.get_ab()) for h in hs]
        for q, it in enumerate(insts):
            h = cache.get(it.n, np.float32)  # a second handle of the size (the first is still held)
            it.load_into(h)
            alone = HandleBatch([h]).cg_device(n_iter=20, rtol=0.0, gtol=0.0, exact_boundary=True)
            assert alone["energy"][0] == together["energy"][q]
            assert np.array_equal(h.get_psi(), states[q][0]) and np.array_equal(h.get_ab(), states[q][1])
    finally:
        cache.close()


def test_batch_cg_energy_window_stop():
    """FP32 instances with an unreachable gradient tolerance: the energy-window
    stop ends each run at a multiple of the window (status 5) before the cap, and
    the state it returns is the state of a run capped at the same iteration count
    (bitwise); with the window off the runs reach the cap (status 3)."""
    from svirl_gb300 import learned as L
    from svirl_gb300.batch import HandleBatch
    from svirl_gb300.relax import HandleCache
    rng = np.random.default_rng(3)
    insts = [L.Instance.sample(n, rng, kappa_range=(4.0, 4.0)) for n in (48, 64)]
    cache = HandleCache()
    try:
        def run(n_iter, window):
            hs = [cache.get(it.n, np.float32) for it in insts]
            try:
                for it, h in zip(insts, hs):
                    it.load_into(h)
                b = HandleBatch(hs)
                b.set_cg_window(window, 1e-7)
                o = b.cg_device(n_iter=n_iter, rtol=0.0, gtol=1e-12, exact_boundary=True)
                st = [(h.get_psi(), h.get_ab()) for h in hs]
                b.close()
                return o, st
            finally:
                for h in hs:
                    cache.put(h)
        cap = 20000
        ow, sw = run(cap, 100)
        assert np.all(ow["status"] == 5), ow["status"]
        assert np.all(ow["iters"] % 100 == 0) and np.all(ow["iters"] < cap)
        for q in range(len(insts)):
            oc, sc = run(int(ow["iters"][q]), 0)
            assert oc["status"][q] == 3 and oc["iters"][q] == ow["iters"][q]
            assert oc["energy"][q] == ow["energy"][q]
            assert np.array_equal(sc[q][0], sw[q][0]) and np.array_equal(sc[q][1], sw[q][1])
        o0, _ = run(300, 0)
        assert np.all(o0["status"] == 3) and np.all(o0["iters"] == 300)
    finally:
        cache.close()
