"""The learned warm start end to end on a small problem: relaxed states made by
the batched device CG, the network trained by the library's kernels (its loss
must fall), then what it gains, in CG iterations from the random start and from
the prediction: (1) to the energy level of the random start's minimum F*
(within 1e-6): the median from the prediction must be below 0.8 of that from the
random start; (2) to the minimum of the run's own start (F* of a tight FP64
relaxation from that start, reached within 1e-6): the prediction must not be
slower (measured: about the same; the predicted amplitude keeps the random
phase, whose vortices the CG still has to move).  Whether the predictions relax
to the random start's own minimum is reported, as are the states/s of both arms."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_trained_network_gain_is_measured():
    from svirl_gb300 import learned as L
    from svirl_gb300.relax import HandleCache
    x, y, _ = L.generate(384, n=64, seed=1, pool_size=128, n_iter=1500, gtol=1e-4)
    net = L.WarmStartNet(seed=0, levels=(16, 32, 64, 64))
    hist = L.train(net, x, y, epochs=8, batch=32, lr=2e-3)
    assert hist[-1] < 0.7 * hist[0], hist
    rng = np.random.default_rng(99)
    ev = [L.Instance.sample(64, rng) for _ in range(16)]
    cache = HandleCache()
    try:
        Estar = L.reference_energies(ev, cache, n_iter=8000)
        res = L.evaluate(net, ev, n_iter=8000, cache=cache, Estar=Estar)
        thr = L.states_throughput(net, ev, Estar, cache, cap=1500, plain_sample=4)
    finally:
        cache.close()
    print("learned warm start (64^2):", res)
    assert res["reached_random_own"] >= 8 and res["reached_warm_own"] >= 8, res
    assert 0 <= res["reached_warm"] <= res["n"]
    # the gain: the prediction reaches the random start's minimum energy level in
    # fewer CG iterations, and its own minimum no later than the random start its own
    assert res["reached_level_both"] >= 4, res
    assert res["iters_warm_level_median"] < 0.8 * res["iters_random_level_median"], res
    assert res["iters_warm_own_median"] <= 1.05 * res["iters_random_own_median"], res
    # the throughput comparison counts states by the same criterion on both arms
    assert 0 <= thr["ok"] <= thr["n"] and 0 <= thr["plain"]["ok"] <= thr["plain"]["sample"]
    assert thr["wall_s"] > 0 and thr["plain"]["wall_s"] > 0
    # the FP64 arm follows the arithmetic of F* (FP64 from the same predicted start)
    assert thr["by_dtype"]["float64"]["ok"] >= thr["n"] // 2, thr["by_dtype"]["float64"]
    print("learned + batched states/s (64^2):", thr)
