"""GPU parity: the CUDA path (through libglgpu's C ABI) against the CPU oracle.

FP64 tolerances (relative to the max |value| of the field):
  one psi/A Jacobi step and short TD trajectories: 1e-12;
  observables, gradients: 1e-12; line-search coefficients: 1e-11 of max |c|;
  CG with kappa=inf (polyroots line search): energies 1e-10;
  CG with finite kappa: energies 1e-6 (scipy BFGS with tol=1e-8 amplifies
  1e-16 differences of the coefficients into 1e-10..1e-8 changes of the step).
Vortex lists: bit-exact for the same order parameter.
"""
import numpy as np
import pytest

from oracle import gl_oracle as O
from tests._pairs import flat, gpu_state, make_pair, oracle_of, rel_err

pytestmark = pytest.mark.gpu

MASKS = ["none", "full", "q1", "random30", "random90", "holes", "empty"]


@pytest.mark.parametrize("mask", MASKS)
@pytest.mark.parametrize("shape", [(8, 8), (11, 9), (33, 17)])
def test_psi_step_matches_oracle(mask, shape):
    gl, orc = make_pair(Nx=shape[0], Ny=shape[1], kappa=np.inf, H=0.2, mask=mask, seed=shape[0] + len(mask))
    gl.solve.td(dt=0.1, Nt=3, eqn="order_parameter")
    orc.td(dt=0.1, Nt=3, eqn="order_parameter")
    psi, ab = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-12
    assert gl.solve._td.last_stats.total_sweeps_psi == sum(orc.sweeps_psi)


@pytest.mark.parametrize("shape", [(4, 4), (5, 70), (70, 5), (27, 18), (53, 35), (25, 16)])
@pytest.mark.parametrize("mask", ["none", "random30"])
def test_psi_step_at_strip_edges_matches_oracle(mask, shape):
    """Domains at and around the psi sweep's strip width (26 columns) and heights
    (8, 12, 17 rows), down to the smallest grid, at every compiled strip height."""
    for rows in (8, 12, 17):
        gl, orc = make_pair(Nx=shape[0], Ny=shape[1], kappa=np.inf, H=0.2, mask=mask, seed=shape[0] + shape[1])
        gl._h.set_psi_strip_rows(rows)
        gl.solve.td(dt=0.1, Nt=3, eqn="order_parameter")
        orc.td(dt=0.1, Nt=3, eqn="order_parameter")
        psi, _ = gpu_state(gl)
        assert rel_err(psi, orc.psi) < 1e-12, rows
        assert gl.solve._td.last_stats.total_sweeps_psi == sum(orc.sweeps_psi), rows


@pytest.mark.parametrize("mask", ["none", "random30", "holes"])
@pytest.mark.parametrize("kappa,sigma", [(5.0, 200.0), (2.0, 10.0), (1.0, 4.0)])
def test_td_with_vector_potential_matches_oracle(mask, kappa, sigma):
    gl, orc = make_pair(Nx=13, Ny=10, kappa=kappa, sigma=sigma, H=0.15, mask=mask, seed=7)
    gl.solve.td(dt=0.1, Nt=10)
    orc.td(dt=0.1, Nt=10)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-12
    assert rel_err(ab, orc.ab) < 1e-12
    st = gl.solve._td.last_stats
    assert st.total_sweeps_psi == sum(orc.sweeps_psi) and st.total_sweeps_A == sum(orc.sweeps_A)


def test_td_eqn_variants_and_langevin_match_oracle():
    gl, orc = make_pair(Nx=9, Ny=11, kappa=3.0, sigma=20.0, H=0.15, seed=7, langevin=(0.05, 0.02))
    for eqn, nt in (("order_parameter", 4), ("vector_potential", 3), (None, 5)):
        gl.solve.td(dt=0.07, Nt=nt, eqn=eqn)
        orc.td(dt=0.07, Nt=nt, eqn=eqn)
        psi, ab = gpu_state(gl)
        assert rel_err(psi, orc.psi) < 1e-12 and rel_err(ab, orc.ab) < 1e-12
    assert int(gl.solve._td._random_t) == orc.rand_t


def _eps_field(x, y):
    return 1.0 - 0.3 * np.cos(0.7 * x) * np.sin(0.5 * y)


@pytest.mark.parametrize("kappa,sigma,mask,form", [(3.0, 20.0, "random30", "callable"),
                                                   (np.inf, 1.0, "holes", "array"),
                                                   (2.0, 50.0, "none", "array")])
def test_spatial_linear_coefficient_matches_oracle(kappa, sigma, mask, form):
    """epsilon(x, y) (svirl/vars/params.py:56-83): the TD step, the energy and
    the CG with a per-node linear coefficient."""
    gl, _ = make_pair(Nx=15, Ny=12, kappa=kappa, sigma=sigma, H=0.2, mask=mask, seed=5)
    if form == "callable":
        gl.params.linear_coefficient = _eps_field
    else:
        gl.params.linear_coefficient = _eps_field(*gl.mesh.xy_grid) + 0.1 * np.random.default_rng(5).random((15, 12))
    orc = oracle_of(gl, rand_t=5)
    assert orc.epsilon_spatial is not None and orc.epsilon == 0.0
    assert abs(gl.observables.free_energy - orc.free_energy()) <= 1e-12 * abs(orc.free_energy())
    gl.solve.td(dt=0.1, Nt=8)
    orc.td(dt=0.1, Nt=8)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-12 and rel_err(ab, orc.ab) < 1e-12
    st = gl.solve._td.last_stats
    assert st.total_sweeps_psi == sum(orc.sweeps_psi) and st.total_sweeps_A == sum(orc.sweeps_A)
    gl.solve.cg(n_iter=30)
    orc.cg(n_iter=30)
    e_gpu, e_orc = np.array(gl.solve._cg.cg_energies), np.array(orc.cg_energies)
    n = min(len(e_gpu), len(e_orc))
    assert abs(len(e_gpu) - len(e_orc)) <= (0 if np.isinf(kappa) else 2)
    assert np.max(np.abs(e_gpu[:n] - e_orc[:n]) / np.abs(e_orc[:n])) < (1e-10 if np.isinf(kappa) else 1e-6)


@pytest.mark.parametrize("mask", ["none", "random30", "q1"])
@pytest.mark.parametrize("kappa", [np.inf, 3.0])
def test_observables_match_oracle(mask, kappa):
    gl, orc = make_pair(Nx=14, Ny=12, kappa=kappa, H=0.3, mask=mask, seed=3, external_field=0.07)
    assert orc.abei is not None
    assert abs(gl.observables.free_energy - orc.free_energy()) <= 1e-12 * abs(orc.free_energy())
    assert rel_err(flat(gl.observables.magnetic_field), orc.magnetic_field()) < 1e-12
    jx, jy = gl.observables.current_density
    assert rel_err(np.concatenate([flat(jx), flat(jy)]), orc.current_density()) < 1e-12
    sx, sy = gl.observables.supercurrent_density
    assert rel_err(np.concatenate([flat(sx), flat(sy)]), orc.supercurrent_density()) < 1e-12


@pytest.mark.parametrize("mask", ["none", "random30", "holes"])
def test_jacobians_and_coefficients_match_oracle(mask):
    gl, orc = make_pair(Nx=12, Ny=13, kappa=2.5, H=0.2, mask=mask, seed=11, external_field=0.05)
    gl.solve._init_cg()
    gp = gl.solve._cg._free_energy_jacobian_psi.get()
    gA = gl.solve._cg._free_energy_jacobian_A.get()
    assert rel_err(gp, orc.jacobian_psi()) < 1e-12
    assert rel_err(gA, orc.jacobian_A()) < 1e-12
    rng = np.random.default_rng(1)
    dpsi = rng.standard_normal(orc.g.N) + 1j * rng.standard_normal(orc.g.N)
    dab = 0.1 * rng.standard_normal(orc.g.Nab)
    c17 = gl._h.conjgrad_coef(dpsi, dab)
    ref = orc.coef(dpsi, dab)
    assert np.max(np.abs(c17 - ref)) <= 1e-11 * np.max(np.abs(ref))
    orc.kappa = np.inf
    gl.params.gl_parameter = np.inf
    c5 = gl._h.conjgrad_coef(dpsi)
    ref5 = orc.coef_psi(dpsi)
    assert np.max(np.abs(c5 - ref5)) <= 1e-11 * np.max(np.abs(ref5))


def test_cg_kappa_inf_matches_oracle():
    gl, orc = make_pair(Nx=17, Ny=15, kappa=np.inf, H=0.1, mask="holes", seed=4)
    gl.solve.td(dt=0.1, Nt=5)
    orc.td(dt=0.1, Nt=5)
    gl.solve.cg(n_iter=60)
    orc.cg(n_iter=60)
    e_gpu = np.array(gl.solve._cg.cg_energies)
    e_orc = np.array(orc.cg_energies)
    assert len(e_gpu) == len(e_orc)
    assert np.max(np.abs(e_gpu - e_orc) / np.abs(e_orc)) < 1e-10
    psi, _ = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-8


def test_cg_finite_kappa_matches_oracle():
    gl, orc = make_pair(Nx=13, Ny=12, kappa=3.0, sigma=100.0, H=0.2, mask="random30", seed=5)
    gl.solve.td(dt=0.1, Nt=5)
    orc.td(dt=0.1, Nt=5)
    gl.solve.cg(n_iter=40)
    orc.cg(n_iter=40)
    e_gpu = np.array(gl.solve._cg.cg_energies)
    e_orc = np.array(orc.cg_energies)
    n = min(len(e_gpu), len(e_orc))
    assert abs(len(e_gpu) - len(e_orc)) <= 2
    assert np.max(np.abs(e_gpu[:n] - e_orc[:n]) / np.abs(e_orc[:n])) < 1e-6
    # second call: persistent direction / beta
    gl.solve.cg(n_iter=5)
    orc.cg(n_iter=5)
    assert abs(gl.observables.free_energy - orc.free_energy()) < 1e-6 * abs(orc.free_energy())


def test_vortices_bit_exact_for_same_state():
    gl, orc = make_pair(Nx=41, Ny=37, kappa=np.inf, H=0.4, seed=5)
    gl.solve.td(dt=0.1, Nt=3)
    psi, ab = gpu_state(gl)
    vx, vy, vv = gl.vortex_detector.vortices
    ox, oy, ov = O.detect_vortices(orc.g, psi, ab, 0.4)
    assert vx.size > 0
    assert np.array_equal(vx, ox) and np.array_equal(vy, oy) and np.array_equal(vv, ov)
    # alias from the reference README
    ax, ay, av = gl.params.fixed_vortices.vortices
    assert np.array_equal(ax, vx)


def test_graph_and_host_loop_give_identical_results():
    res = []
    for graphs in (True, False):
        gl, _ = make_pair(Nx=21, Ny=19, kappa=2.0, sigma=100.0, H=0.2, mask="holes", seed=9)
        gl._h.set_use_graphs(graphs)
        gl.solve.td(dt=0.1, Nt=7)
        assert gl.solve._td.last_stats.used_graph == (1 if graphs else 0)
        res.append(gpu_state(gl))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


def test_deterministic_repeat():
    out = []
    for _ in range(2):
        gl, _ = make_pair(Nx=40, Ny=30, kappa=4.0, sigma=200.0, H=0.2, mask="holes", seed=2)
        gl.solve.td(dt=0.1, Nt=5)
        gl.solve.cg(n_iter=5)
        out.append((gpu_state(gl), gl.observables.free_energy))
    assert np.array_equal(out[0][0][0], out[1][0][0]) and out[0][1] == out[1][1]


def test_c1_config_trajectory_fp64():
    """The plain small configuration (129x129, kappa=5, sigma=200, H=0.1) for 20 steps."""
    gl, orc = make_pair(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=5.0, sigma=200.0, H=0.1, seed=0)
    gl.solve.td(dt=0.1, Nt=20)
    orc.td(dt=0.1, Nt=20)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-11 and rel_err(ab, orc.ab) < 1e-11
    assert gl.solve._td.last_stats.total_sweeps_psi == sum(orc.sweeps_psi)
    E = gl.observables.free_energy
    assert abs(E - orc.free_energy()) < 1e-11 * abs(orc.free_energy())


def test_fp32_error_against_fp64_oracle():
    """FP32 stencils with FP64 reductions: errors after 20 TD steps + 20 CG iterations."""
    gl, orc = make_pair(Nx=33, Ny=33, kappa=5.0, sigma=200.0, H=0.1, seed=1, dtype=np.float32)
    gl.solve.td(dt=0.1, Nt=20)
    orc.td(dt=0.1, Nt=20)
    psi, ab = gpu_state(gl)
    assert np.max(np.abs(psi - orc.psi)) < 5e-4
    assert np.max(np.abs(ab - orc.ab)) < 5e-4
    assert abs(gl.observables.free_energy - orc.free_energy()) < 1e-4 * abs(orc.free_energy())


def test_reduce_sum_matches_numpy():
    gl, _ = make_pair(Nx=64, Ny=64)
    rng = np.random.default_rng(5)
    for n in (1, 255, 4097, 100003):
        x = rng.random(n)
        assert abs(gl.par.red.test_sum(x, n) - np.sum(x)) < 1e-10
    x = rng.random(5 * 7777)
    assert np.allclose(gl.par.red.test_sum_v(x, 7777, 5), x.reshape(-1, 5).sum(axis=0), atol=1e-10)


def test_nan_is_reported_not_hidden():
    gl, _ = make_pair(Nx=10, Ny=10)
    psi = gl.vars.order_parameter
    psi[3, 4] = np.nan
    gl.vars.order_parameter = psi
    with pytest.warns(RuntimeWarning):
        gl.solve.td(dt=0.1, Nt=2)
    assert gl.solve._td.last_stats.nan_seen == 1


def test_create_destroy_many():
    from svirl_gb300 import GLSolver
    rng = np.random.default_rng(0)
    for _ in range(10):
        gl = GLSolver(Nx=int(rng.integers(4, 300)), Ny=int(rng.integers(4, 300)), dx=0.3, dy=0.3,
                      gl_parameter=1.0 if rng.random() > 0.5 else np.inf)
        gl.solve.td(dt=0.05, Nt=1)
        gl.close()


def test_sweep_timer_runs_and_keeps_state():
    gl, _ = make_pair(Nx=200, Ny=150, kappa=3.0, sigma=100.0, seed=3)
    before = gpu_state(gl)
    ms_psi = gl._h.time_sweeps(0, 3)
    ms_A = gl._h.time_sweeps(1, 3)
    after = gpu_state(gl)
    assert ms_psi > 0 and ms_A > 0
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    # the A timing leaves its link terms in the link-factor buffer; the next TD call
    # rebuilds the table, so it continues exactly as an untimed twin does
    twin, _ = make_pair(Nx=200, Ny=150, kappa=3.0, sigma=100.0, seed=3)
    for x in (gl, twin):
        x.solve.td(dt=0.1, Nt=3)
    a, b = gpu_state(gl), gpu_state(twin)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
