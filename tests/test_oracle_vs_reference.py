"""Pin the oracle's host-level restatement against the reference's own host code.

The reference (microsoft/svirl) runs unmodified on the NumPy pycuda shim
(``oracle/fake_pycuda``); ``oracle.gl_oracle.GLOracle`` runs the same cases from
the same initial state.  Both use the kernels of ``oracle/kernels_np.py``, so
these tests pin the host logic: the TD time/Jacobi loops and their stop rule,
the A-sweep buffer aliasing, the CG beta/alpha/stop logic and its persistent
state, the observables' plumbing and the vortex detector.  Skipped where the
reference sources are not mounted.
"""
import numpy as np
import pytest

from oracle import gl_oracle as O
from tests.refshim import load_reference


def oracle_from_ref(gl, rand_t=1):
    cfg = gl.cfg
    psi = O.flatten_ij(gl.vars.order_parameter)
    a, b = gl.vars.vector_potential
    ab = np.concatenate([O.flatten_ij(a), O.flatten_ij(b)])
    mt = O.flatten_ij(gl.mesh.material_tiling) if gl.mesh.have_material_tiling() else None
    ei = gl.params.external_irregular_vector_potential
    abei = None if ei is None else np.concatenate([O.flatten_ij(ei[0]), O.flatten_ij(ei[1])])
    return O.GLOracle(cfg.Nx, cfg.Ny, cfg.dx, cfg.dy, psi, ab, mt=mt, abei=abei,
                      kappa=gl.params.gl_parameter, sigma=gl.params.normal_conductivity,
                      epsilon=float(np.asarray(gl.params.linear_coefficient_scalar_h()).reshape(-1)[0]),
                      epsilon_spatial=(None if gl.params._epsilon.size == 1
                                       else O.flatten_ij(gl.params.linear_coefficient)),
                      H=gl.params.homogeneous_external_field,
                      stop_psi=cfg.stop_criterion_order_parameter, stop_A=cfg.stop_criterion_vector_potential,
                      rand_t=rand_t, langevin_psi=gl.params.order_parameter_Langevin_coefficient,
                      langevin_A=gl.params.vector_potential_Langevin_coefficient,
                      convergence_rtol=cfg.convergence_rtol)


def ref_state(gl):
    psi = O.flatten_ij(gl.vars.order_parameter)
    a, b = gl.vars.vector_potential
    return psi, np.concatenate([O.flatten_ij(a), O.flatten_ij(b)])


def close(x, y, tol=1e-13):
    x, y = np.asarray(x), np.asarray(y)
    scale = max(np.max(np.abs(y)), 1e-300)
    return np.max(np.abs(x - y)) <= tol * scale


def random_mask(rng, nxc, nyc, frac=0.3):
    mt = np.ones((nxc, nyc), dtype=bool)
    k = int(frac * nxc * nyc)
    mt[rng.integers(0, nxc, k), rng.integers(0, nyc, k)] = False
    return mt


@pytest.mark.parametrize("kappa,sigma,H,masked,seed", [
    (5.0, 200.0, 0.1, False, 1),
    (2.0, 10.0, 0.3, True, 2),
    (np.inf, 1.0, 0.2, True, 3),
])
def test_td_then_cg_matches_reference(kappa, sigma, H, masked, seed):
    svirl = load_reference()
    rng = np.random.default_rng(seed)
    mt = random_mask(rng, 9, 8) if masked else None
    gl = svirl.GLSolver(Nx=10, Ny=9, dx=0.5, dy=0.45, order_parameter="random", random_seed=seed,
                        gl_parameter=kappa, normal_conductivity=sigma, homogeneous_external_field=H,
                        material_tiling=mt)
    orc = oracle_from_ref(gl, rand_t=seed)
    E0 = gl.observables.free_energy
    assert close(orc.free_energy(), E0, 1e-13)

    gl.solve.td(dt=0.1, Nt=12)
    orc.td(dt=0.1, Nt=12)
    psi, ab = ref_state(gl)
    assert close(orc.psi, psi) and close(orc.ab, ab)

    # kappa=inf: the quartic line search (polyroots) keeps the trajectories equal to
    # round-off.  Finite kappa: scipy BFGS (tol=1e-8) turns 1e-16 differences in
    # summation order into ~1e-10 differences of alpha, so the bound is looser.
    tol = 1e-13 if np.isinf(kappa) else 1e-8
    gl.solve.cg(n_iter=25)
    orc.cg(n_iter=25)
    psi, ab = ref_state(gl)
    assert len(orc.cg_energies) == len(gl.solve._cg.cg_energies)
    assert close(orc.cg_energies, gl.solve._cg.cg_energies, tol)
    assert close(orc.psi, psi, 10 * tol) and close(orc.ab, ab, 10 * tol)

    # a second cg() call starts from the persistent direction/beta (finite kappa)
    gl.solve.cg(n_iter=5)
    orc.cg(n_iter=5)
    psi, ab = ref_state(gl)
    assert close(orc.psi, psi, 10 * tol) and close(orc.ab, ab, 10 * tol)

    # observables, evaluated on the reference's state
    orc.psi, orc.ab = psi.copy(), ab.copy()
    B = O.flatten_ij(gl.observables.magnetic_field)
    assert close(orc.magnetic_field(), B, 1e-12)
    jx, jy = gl.observables.current_density
    assert close(orc.current_density(), np.concatenate([O.flatten_ij(jx), O.flatten_ij(jy)]), 1e-12)
    sx, sy = gl.observables.supercurrent_density
    assert close(orc.supercurrent_density(), np.concatenate([O.flatten_ij(sx), O.flatten_ij(sy)]), 1e-12)
    assert close(orc.free_energy(), gl.observables.free_energy, 1e-12)


@pytest.mark.parametrize("kappa,sigma,masked,form", [
    (3.0, 20.0, True, "array"),
    (np.inf, 1.0, True, "callable"),
    (2.0, 10.0, False, "callable"),
])
def test_spatial_linear_coefficient_matches_reference(kappa, sigma, masked, form):
    """epsilon(x, y) set as an (Nx, Ny) array (params.py:56-69): the kernels
    then take epsilon_spatial and a scalar epsilon of 0 (params.py:72-83).  The
    reference's callable form names an undefined `mesh` (params.py:59) and
    raises NameError, so a callable is evaluated on the node grid here and
    passed as the array."""
    svirl = load_reference()
    rng = np.random.default_rng(11)
    mt = random_mask(rng, 10, 8) if masked else None
    gl = svirl.GLSolver(Nx=11, Ny=9, dx=0.5, dy=0.45, order_parameter="random", random_seed=4,
                        gl_parameter=kappa, normal_conductivity=sigma, homogeneous_external_field=0.2,
                        material_tiling=mt)
    if form == "array":
        gl.params.linear_coefficient = 1.0 + 0.5 * rng.random((11, 9)) - 0.2
    else:
        f = lambda x, y: 1.0 - 0.3 * np.cos(0.7 * x) * np.sin(0.5 * y)  # noqa: E731
        with pytest.raises(NameError):
            gl.params.linear_coefficient = f
        gl.params.linear_coefficient = f(*gl.mesh.xy_grid)
    assert gl.params._epsilon.size > 1
    orc = oracle_from_ref(gl, rand_t=4)
    assert orc.epsilon == 0.0 and orc.epsilon_spatial is not None
    assert close(orc.free_energy(), gl.observables.free_energy, 1e-13)
    gl.solve.td(dt=0.1, Nt=8)
    orc.td(dt=0.1, Nt=8)
    psi, ab = ref_state(gl)
    assert close(orc.psi, psi) and close(orc.ab, ab)
    tol = 1e-13 if np.isinf(kappa) else 1e-8
    gl.solve.cg(n_iter=15)
    orc.cg(n_iter=15)
    psi, ab = ref_state(gl)
    assert close(orc.cg_energies, gl.solve._cg.cg_energies, tol)
    assert close(orc.psi, psi, 10 * tol) and close(orc.ab, ab, 10 * tol)


def test_langevin_and_eqn_variants_match_reference():
    svirl = load_reference()
    gl = svirl.GLSolver(Nx=9, Ny=11, dx=0.5, dy=0.5, order_parameter="random", random_seed=7,
                        gl_parameter=3.0, normal_conductivity=20.0, homogeneous_external_field=0.15,
                        order_parameter_Langevin_coefficient=0.05, vector_potential_Langevin_coefficient=0.02)
    orc = oracle_from_ref(gl, rand_t=7)
    for eqn, nt in (("order_parameter", 4), ("vector_potential", 3), (None, 5)):
        gl.solve.td(dt=0.07, Nt=nt, eqn=eqn)
        orc.td(dt=0.07, Nt=nt, eqn=eqn)
        psi, ab = ref_state(gl)
        assert close(orc.psi, psi) and close(orc.ab, ab)


def test_initial_state_helpers_match_reference():
    svirl = load_reference()
    gl = svirl.GLSolver(dx=0.5, dy=0.5, Lx=6, Ly=5, order_parameter="random", random_seed=11,
                        gl_parameter=5.0, homogeneous_external_field=0.1)
    Nx, dx, Lx, Ny, dy, Ly = O.geometry(dx=0.5, Lx=6, dy=0.5, Ly=5)
    assert (Nx, Ny) == (gl.cfg.Nx, gl.cfg.Ny)
    g = O.K.Grid(Nx, Ny, dx, dy)
    psi0 = O.random_order_parameter(g.N, 1.0, 11)
    psi, ab = ref_state(gl)
    assert np.array_equal(psi0, psi)
    assert np.array_equal(O.symmetric_gauge(g, 0.1, np.float64, Lx, Ly), ab)


def test_vortex_detector_matches_reference():
    svirl = load_reference()
    gl = svirl.GLSolver(Nx=25, Ny=23, dx=0.5, dy=0.5, order_parameter="random", random_seed=5,
                        gl_parameter=np.inf, homogeneous_external_field=0.4)
    gl.solve.td(dt=0.1, Nt=3)
    vx, vy, vv = gl.vortex_detector.vortices
    psi, ab = ref_state(gl)
    g = O.K.Grid(25, 23, 0.5, 0.5)
    ox, oy, ov = O.detect_vortices(g, psi, ab, 0.4)
    assert vx.size > 0
    assert np.array_equal(ox, vx) and np.array_equal(oy, vy) and np.array_equal(ov, vv)


@pytest.mark.parametrize("Nx,Ny,mask", [(4, 4, "none"), (4, 40, "random"), (40, 4, "random"), (9, 7, "empty")])
def test_edge_geometries_match_reference(Nx, Ny, mask):
    """The smallest grid the reference accepts (4 x 4, svirl/__init__.py:97-98),
    three-cell-wide strips in either direction, and a domain with every cell
    removed (psi is then 0 after the first step): TD and the energy follow the
    reference."""
    svirl = load_reference()
    rng = np.random.default_rng(Nx * 100 + Ny)
    mt = None
    if mask == "random":
        mt = random_mask(rng, Nx - 1, Ny - 1, 0.2)
    elif mask == "empty":
        mt = np.zeros((Nx - 1, Ny - 1), dtype=bool)
    gl = svirl.GLSolver(Nx=Nx, Ny=Ny, dx=0.5, dy=0.5, order_parameter="random", random_seed=2,
                        gl_parameter=3.0, normal_conductivity=50.0, homogeneous_external_field=0.2,
                        material_tiling=mt)
    orc = oracle_from_ref(gl, rand_t=2)
    assert close(orc.free_energy(), gl.observables.free_energy, 1e-13) or abs(gl.observables.free_energy) < 1e-300
    gl.solve.td(dt=0.1, Nt=6)
    orc.td(dt=0.1, Nt=6)
    psi, ab = ref_state(gl)
    assert close(orc.psi, psi) and close(orc.ab, ab)
    if mask == "empty":
        assert not np.any(psi)


@pytest.mark.parametrize("kappa,sigma", [(np.inf, 1.0), (4.0, 80.0)])
def test_external_field_with_mask_matches_reference(kappa, sigma):
    """An external field (the external irregular vector potential enters the link
    phases of the energy, the gradients and the CG, params.py:224-303) on a
    masked domain, for kappa = inf and finite kappa."""
    svirl = load_reference()
    rng = np.random.default_rng(21)
    mt = random_mask(rng, 12, 10, 0.15)
    gl = svirl.GLSolver(Nx=13, Ny=11, dx=0.5, dy=0.5, order_parameter="random", random_seed=6,
                        gl_parameter=kappa, normal_conductivity=sigma, homogeneous_external_field=0.15,
                        external_field=0.04, material_tiling=mt)
    orc = oracle_from_ref(gl, rand_t=6)
    assert orc.abei is not None
    assert close(orc.free_energy(), gl.observables.free_energy, 1e-13)
    gl.solve.td(dt=0.1, Nt=6)
    orc.td(dt=0.1, Nt=6)
    psi, ab = ref_state(gl)
    assert close(orc.psi, psi) and close(orc.ab, ab)
    tol = 1e-13 if np.isinf(kappa) else 1e-8
    gl.solve.cg(n_iter=20)
    orc.cg(n_iter=20)
    assert close(orc.cg_energies, gl.solve._cg.cg_energies, tol)
