"""Crank-Nicolson psi steps on the GPU (svirl/cuda/td.h:136-292, the reference's
commented-out kernel; ``gl.solve.td_scheme``) against the oracle, FP64:
"crank_nicolson" (explicit half of every link from the step's start) and
"crank_nicolson_as_written" (the kernel as written), single sweeps' arithmetic
and TD trajectories at 1e-12 with equal Jacobi sweep counts, with masks, finite
kappa, Langevin noise and a spatial linear coefficient; the graph and the
host-driven loop bitwise equal; the as-written variant also against the
reference's own compiled kernel (oracle/_ref).  FP32: max |dpsi| <= 1e-4 against
the FP64 oracle after 10 steps.  Batches reject Crank-Nicolson handles."""
import numpy as np
import pytest

from oracle import kernels_np as K
from svirl_gb300._lib import GLGPUError
from tests._pairs import flat, gpu_state, make_pair, oracle_of, rel_err

pytestmark = pytest.mark.gpu

SCHEMES = ["crank_nicolson", "crank_nicolson_as_written"]


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("mask", ["none", "random30", "holes"])
@pytest.mark.parametrize("kappa,sigma", [(np.inf, 1.0), (3.0, 50.0)])
def test_cn_td_matches_oracle(scheme, mask, kappa, sigma):
    gl, orc = make_pair(Nx=33, Ny=17, kappa=kappa, sigma=sigma, H=0.15, mask=mask, seed=4)
    gl.solve.td_scheme = scheme
    orc.scheme = scheme
    gl.solve.td(dt=0.1, Nt=8)
    orc.td(dt=0.1, Nt=8)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-12 and rel_err(ab, orc.ab) < 1e-12
    st = gl.solve._td.last_stats
    assert st.total_sweeps_psi == sum(orc.sweeps_psi) and st.total_sweeps_A == sum(orc.sweeps_A)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_cn_langevin_eps_field_and_host_loop(scheme):
    runs = []
    for graphs in (True, False):
        gl, _ = make_pair(Nx=20, Ny=23, kappa=np.inf, H=0.2, mask="holes", seed=6, langevin=(0.04, 0.0))
        gl.params.linear_coefficient = 1.0 - 0.3 * np.cos(0.7 * gl.mesh.xy_grid[0])
        orc = oracle_of(gl, rand_t=6)
        gl.solve.td_scheme = scheme
        orc.scheme = scheme
        gl._h.set_use_graphs(graphs)
        gl.solve.td(dt=0.08, Nt=6)
        orc.td(dt=0.08, Nt=6)
        psi, _ = gpu_state(gl)
        assert rel_err(psi, orc.psi) < 1e-12
        runs.append(psi)
    assert np.array_equal(runs[0], runs[1])


def test_cn_as_written_matches_reference_kernel():
    from oracle import ref_gpu
    if not ref_gpu.manifest():
        pytest.skip("reference kernels not built")
    R = ref_gpu.RefKernels(np.float64)
    gl, _ = make_pair(Nx=33, Ny=17, dx=0.5, dy=0.5, kappa=np.inf, H=0.15, mask="holes", seed=9)
    ref = oracle_of(gl, rand_t=9, kernels=R)
    ref.scheme = "crank_nicolson_as_written"
    gl.solve.td_scheme = "crank_nicolson_as_written"
    gl.solve.td(dt=0.1, Nt=8)
    ref.td(dt=0.1, Nt=8)
    psi, _ = gpu_state(gl)
    assert rel_err(psi, ref.psi) < 1e-12
    assert gl.solve._td.last_stats.total_sweeps_psi == sum(ref.sweeps_psi)
    # one sweep of arbitrary inputs: the oracle against the reference's kernel
    g = K.Grid(40, 37, 0.4, 0.55)
    rng = np.random.default_rng(1)
    psi0 = rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N)
    rhs = psi0 + 0.1 * rng.standard_normal(g.N)
    ab = 0.5 * rng.standard_normal(g.Nab)
    mt = flat(rng.random((g.Nxc, g.Nyc)) > 0.2)
    for jstep, lang in ((0, 0.05), (1, 0.0)):
        rr, ro = rhs.copy(), rhs.copy()
        n_r, c_r = R.iterate_order_parameter_jacobi_step_cn(g, 0.1, 1.0, None, mt, ab, rr, psi0, lang, jstep, 3, 1e-6)
        n_o, c_o = K.iterate_order_parameter_jacobi_step_cn(g, 0.1, 1.0, None, mt, ab, ro, psi0, lang, jstep, 3, 1e-6,
                                                            as_written=True)
        assert rel_err(n_o, n_r) < 1e-13 and abs(c_o - c_r) <= 1


def test_cn_fp32_against_fp64_oracle():
    gl, _ = make_pair(Nx=65, Ny=49, kappa=4.0, sigma=200.0, H=0.2, mask="holes", seed=3, dtype=np.float32)
    gl64, orc = make_pair(Nx=65, Ny=49, kappa=4.0, sigma=200.0, H=0.2, mask="holes", seed=3)
    gl.solve.td_scheme = "crank_nicolson"
    orc.scheme = "crank_nicolson"
    gl.solve.td(dt=0.1, Nt=10)
    orc.td(dt=0.1, Nt=10)
    psi, _ = gpu_state(gl)
    err = float(np.max(np.abs(psi - orc.psi)))
    print("Crank-Nicolson FP32 against the FP64 oracle after 10 steps: max |dpsi| %.2e" % err)
    assert err <= 1e-4


def test_batch_rejects_cn_handles():
    from svirl_gb300.batch import HandleBatch
    gl, _ = make_pair(Nx=12, Ny=11)
    gl.solve.td_scheme = "crank_nicolson"
    b = HandleBatch([gl._h])
    with pytest.raises(GLGPUError, match="Crank-Nicolson"):
        b.td_raw(0.1, 1, 0)
    b.close()
    with pytest.raises(ValueError):
        gl.solve.td_scheme = "leapfrog"
