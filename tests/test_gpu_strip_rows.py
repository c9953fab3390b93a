"""The psi sweep's strip height (chosen per handle / batch from the compiled
heights) does not change results: every node gets the same arithmetic and the
residual is a maximum, so TD states and Jacobi sweep counts are bitwise equal
for every height."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HEIGHTS = (8, 12, 17)


def _solver(dtype, kappa):
    from svirl_gb300 import GLSolver
    rng = np.random.default_rng(5)
    mt = rng.random((140, 96)) > 0.05
    return GLSolver(Nx=141, Ny=97, dx=0.5, dy=0.5, dtype=dtype, random_seed=2, gl_parameter=kappa,
                    normal_conductivity=100.0, homogeneous_external_field=0.1, material_tiling=mt)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("kappa", [np.inf, 3.0])
def test_td_independent_of_strip_height(dtype, kappa):
    out = []
    for R in HEIGHTS:
        gl = _solver(dtype, kappa)
        gl._h.set_psi_strip_rows(R)
        assert gl._h.psi_strip_rows() == R
        gl.solve.td(dt=0.1, Nt=6)
        st = gl.solve._td.last_stats
        out.append((gl.vars.order_parameter, gl.vars.vector_potential, int(st.total_sweeps_psi)))
        gl.close()
    for psi, ab, sw in out[1:]:
        assert np.array_equal(psi, out[0][0]) and sw == out[0][2]
        for x, y in zip(ab, out[0][1]):
            assert np.array_equal(x, y)


def test_model_choice_and_bad_height():
    from svirl_gb300 import _lib
    big = _lib.Handle(2049, 2049, 0.5, 0.5, np.float32)
    try:
        assert big.psi_strip_rows() == 17  # 79 strips x 121 row blocks over 2432 warps: 4 items each
    finally:
        big.close()
    small = _lib.Handle(33, 33, 0.5, 0.5, np.float32)
    try:
        assert small.psi_strip_rows() == 8  # fewer items than warps: the shortest strip
        with pytest.raises(_lib.GLGPUError):
            small.set_psi_strip_rows(13)
        small.set_psi_strip_rows(0)
        assert small.psi_strip_rows() == 8
    finally:
        small.close()
