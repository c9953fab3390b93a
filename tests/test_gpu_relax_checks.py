"""The FP64 checks and the FP64 finish of the relaxation engine (svirl_gb300/relax.py)
used by the states/s measurement: the gradient-tolerance test agrees with the
batched CG's own gradient stop, and the FP64 finish of an FP32-relaxed state keeps
lowering its energy in float64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(k=3, n=33):
    from svirl_gb300 import learned as L
    out = []
    for s in range(k):
        rng = np.random.default_rng(500 + s)
        out.append(L.Instance.sample(n, rng, H_range=(0.05, 0.3), kappa_range=(4.0, 4.0), hole_frac=(0.0, 0.05),
                                     radius=(2.0, 3.0)))
    return out


def test_gradient_check_matches_the_cg_stop():
    from svirl_gb300 import relax as RX
    insts = _instances()
    cache = RX.HandleCache()
    try:
        # random starts are far from any minimum; FP64 states relaxed to 1e-6 meet 1e-4
        starts = [(it.psi0, it.ab0) for it in insts]
        assert not RX.gradient_ok_fp64(insts, starts, cache, 1e-4).any()
        out, states, _ = RX.relax(insts, cache, np.float64, n_iter=20000, gtol=1e-6)
        assert (out["status"] == 1).all()
        assert RX.gradient_ok_fp64(insts, states, cache, 1e-4).all()
        # the check leaves the state alone: the energy is unchanged
        E0 = RX.energies_fp64(insts, states, cache)
        RX.gradient_ok_fp64(insts, states, cache, 1e-4)
        assert np.array_equal(E0, RX.energies_fp64(insts, states, cache))
    finally:
        cache.close()


def test_fp64_finish_lowers_the_energy_of_fp32_states():
    from svirl_gb300 import relax as RX
    insts = _instances()
    cache = RX.HandleCache()
    try:
        _, s32, _ = RX.relax(insts, cache, np.float32, n_iter=300, gtol=0.0)
        E32 = RX.energies_fp64(insts, s32, cache)
        out, s64 = RX.polish_fp64(insts, s32, cache, n_iter=200, gtol=0.0)
        assert out["ms"] > 0 and (out["iters"] == 200).all()
        assert all(p.dtype == np.complex128 and a.dtype == np.float64 for p, a in s64)
        E64 = RX.energies_fp64(insts, s64, cache)
        assert (E64 <= E32).all() and (E64 < E32).any()
    finally:
        cache.close()
