"""Batched engine: one device loop over instances of uneven sizes and mixed
parameters gives, for every instance, exactly the state it reaches alone, and
the oracle's state to 1e-12."""
import numpy as np
import pytest

from tests._pairs import gpu_state, make_pair, rel_err

pytestmark = pytest.mark.gpu

CONFIGS = [
    dict(Nx=33, Ny=17, kappa=np.inf, H=0.2, mask="holes", seed=1),
    dict(Nx=20, Ny=25, kappa=5.0, sigma=200.0, H=0.1, mask="random30", seed=2),
    dict(Nx=65, Ny=40, kappa=2.0, sigma=100.0, H=0.15, mask="none", seed=3),
    dict(Nx=9, Ny=9, kappa=np.inf, H=0.3, mask="q1", seed=4, langevin=(0.03, 0.0)),
    dict(Nx=41, Ny=41, kappa=4.0, sigma=150.0, H=0.2, mask="holes", seed=5, langevin=(0.02, 0.01)),
]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("graphs", [True, False])
def test_batch_td_equals_individual_runs(dtype, graphs):
    from svirl_gb300.batch import GLBatch
    batched, alone, oracles = [], [], []
    for cfg in CONFIGS:
        gl_b, orc = make_pair(dtype=dtype, **cfg)
        gl_a, _ = make_pair(dtype=dtype, **cfg)
        batched.append(gl_b)
        alone.append(gl_a)
        oracles.append(orc)
    batch = GLBatch(batched)
    batch.set_use_graphs(graphs)
    st = batch.td(dt=0.1, Nt=12)
    assert st.steps == 12 and st.used_graph == (1 if graphs else 0)
    total = 0
    for gl in alone:
        gl.solve.td(dt=0.1, Nt=12)
        total += gl.solve._td.last_stats.total_sweeps_psi
    assert st.total_sweeps_psi == total
    for gb, ga in zip(batched, alone):
        pb, ab = gpu_state(gb)
        pa, aa = gpu_state(ga)
        assert np.array_equal(pb, pa) and np.array_equal(ab, aa)
        assert int(gb.solve._td._random_t) == int(ga.solve._td._random_t)
    if dtype == np.float64:
        for gb, orc in zip(batched, oracles):
            orc.td(dt=0.1, Nt=12)
            pb, ab = gpu_state(gb)
            assert rel_err(pb, orc.psi) < 1e-12 and rel_err(ab, orc.ab) < 1e-12
    batch.close()


def test_batch_eqn_modes_and_repeated_calls():
    from svirl_gb300.batch import GLBatch
    batched = [make_pair(**c)[0] for c in CONFIGS[:3]]
    alone = [make_pair(**c)[0] for c in CONFIGS[:3]]
    batch = GLBatch(batched)
    for eqn, nt in (("order_parameter", 3), ("vector_potential", 2), (None, 4), (None, 1)):
        batch.td(dt=0.1, Nt=nt, eqn=eqn)
        for gl in alone:
            gl.solve.td(dt=0.1, Nt=nt, eqn=eqn)
    for gb, ga in zip(batched, alone):
        assert np.array_equal(gpu_state(gb)[0], gpu_state(ga)[0])
        assert np.array_equal(gpu_state(gb)[1], gpu_state(ga)[1])
