"""The learned warm start end to end on a small problem: relaxed states made by
the batched device CG, the network trained by the library's kernels, then the
gain it brings: its predicted states start the CG at a lower energy than the
random start does (the measured iteration counts to F* are reported)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_trained_network_beats_random_start():
    from svirl_gb300 import learned as L
    from svirl_gb300.relax import HandleCache, relax
    x, y, _ = L.generate(384, n=64, seed=1, pool_size=128, n_iter=1500, gtol=1e-4)
    net = L.WarmStartNet(seed=0, levels=(16, 32, 64, 64))
    hist = L.train(net, x, y, epochs=8, batch=32, lr=2e-3)
    assert hist[-1] < 0.7 * hist[0], hist
    rng = np.random.default_rng(99)
    ev = [L.Instance.sample(64, rng) for _ in range(16)]
    cache = HandleCache()
    try:
        r0, _, _ = relax(ev, cache, np.float64, n_iter=0, gtol=0.0, fetch=False)
        starts = L.decode(ev, net.predict(L.features(ev)))
        w0, _, _ = relax(ev, cache, np.float64, starts=starts, n_iter=0, gtol=0.0, fetch=False)
        res = L.evaluate(net, ev, n_iter=8000, cache=cache)
    finally:
        cache.close()
    # the prediction is a far better starting point than the random state
    assert np.median(w0["energy"] - r0["energy"]) < 0, (w0["energy"], r0["energy"])
    assert res["reached_random"] >= 8
    print("learned warm start (64^2):", res)
