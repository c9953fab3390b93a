"""Checkpoint / resume: a TDGL run with Langevin noise restored from a
checkpoint continues bit for bit as the uninterrupted run; the dataset file
round-trips instances and states."""
import numpy as np
import pytest


def _solver(dtype, seed=3):
    from svirl_gb300 import GLSolver
    rng = np.random.default_rng(seed)
    mt = rng.random((16, 12)) > 0.1
    gl = GLSolver(Nx=17, Ny=13, dx=0.5, dy=0.5, dtype=dtype, random_seed=seed, gl_parameter=3.0,
                  normal_conductivity=50.0, homogeneous_external_field=0.2, material_tiling=mt,
                  order_parameter_Langevin_coefficient=0.05, vector_potential_Langevin_coefficient=0.02)
    gl.params.linear_coefficient = 1.0 + 0.1 * rng.random((17, 13))
    return gl


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_resume_continues_bitwise(tmp_path, dtype):
    from svirl_gb300 import checkpoint
    a = _solver(dtype)
    a.solve.td(dt=0.05, Nt=20)
    b = _solver(dtype)
    b.solve.td(dt=0.05, Nt=10)
    path = str(tmp_path / "state.npz")
    checkpoint.save(b, path)
    b.close()
    c = checkpoint.load(path)
    c.solve.td(dt=0.05, Nt=10)
    assert np.array_equal(a.vars.order_parameter, c.vars.order_parameter)
    for x, y in zip(a.vars.vector_potential, c.vars.vector_potential):
        assert np.array_equal(x, y)
    # restore into an existing solver of the same grid
    d = _solver(dtype, seed=9)
    checkpoint.restore(d, path)
    d.solve.td(dt=0.05, Nt=10)
    assert np.array_equal(a.vars.order_parameter, d.vars.order_parameter)


@pytest.mark.gpu
def test_restore_rejects_other_grid(tmp_path):
    from svirl_gb300 import GLSolver, checkpoint
    a = _solver(np.float64)
    path = str(tmp_path / "s.npz")
    checkpoint.save(a, path)
    other = GLSolver(Nx=9, Ny=9, dx=0.5, dy=0.5, dtype=np.float64)
    with pytest.raises(ValueError):
        checkpoint.restore(other, path)


def test_dataset_roundtrip(tmp_path):
    from svirl_gb300 import checkpoint
    from svirl_gb300.learned import Instance
    rng = np.random.default_rng(0)
    insts = [Instance.sample(16, rng) for _ in range(3)]
    states = [(rng.random(256) + 1j * rng.random(256), rng.random(2 * 15 * 16)) for _ in insts]
    path = str(tmp_path / "d.npz")
    checkpoint.save_dataset(path, insts, states)
    i2, s2 = checkpoint.load_dataset(path)
    for a, b in zip(insts, i2):
        assert (a.n, a.dx, a.H, a.kappa, a.sigma) == (b.n, b.dx, b.H, b.kappa, b.sigma)
        assert np.array_equal(a.mt, b.mt) and np.array_equal(a.psi0, b.psi0) and np.array_equal(a.nm, b.nm)
    for (p, q), (p2, q2) in zip(states, s2):
        assert np.array_equal(p, p2) and np.array_equal(q, q2)
