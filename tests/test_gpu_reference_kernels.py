"""GPU parity against the reference's own CUDA kernels.

``oracle/ref_build.py`` compiles the reference's kernels (``svirl/cuda/*.h``,
unchanged, as ``svirl/parallel/startup.py:41-63`` assembles them) for sm_103a;
``oracle/ref_gpu.py`` launches them with the reference's launch geometry and
two-pass reductions.  On the same inputs this file compares three things: the
reference's kernels (R), the NumPy oracle (O) and libglgpu through its C ABI (G).

FP64 tolerances, relative to the largest magnitude of the field compared:
  per kernel, R against O: 1e-13 (this pins the oracle's arithmetic);
  per kernel, G against R: 1e-12; line-search coefficients 1e-12 of max |c|;
  Jacobi residual codes int(1e4 r / eps): equal, or off by one where r sits on a
  code boundary;
  TD trajectories (oracle host loop on R against G): 1e-12 with equal sweep counts;
  CG at kappa = inf (polyroots line search): energies 1e-10;
  CG at finite kappa (scipy BFGS, which turns 1e-16 changes of the coefficients
  into 1e-10..1e-8 changes of alpha): energies 1e-6.
FP32: the reference's FP32 kernels against libglgpu's FP32 path after 20 TD steps
of the 129x129 kappa = 5 workload: max |dpsi| <= 1e-4 (both against FP64: stated
in the printed line).
"""
import numpy as np
import pytest

from oracle import kernels_np as K
from tests._pairs import flat, gpu_state, make_pair, oracle_of, rel_err

pytestmark = pytest.mark.gpu


def _ref(dtype=np.float64):
    from oracle import ref_gpu
    if not ref_gpu.manifest():
        pytest.skip("reference kernels not built (python -m oracle.ref_build where the reference is mounted)")
    return ref_gpu.RefKernels(dtype)


GEOMS = [(12, 11, 0.5, 0.45), (33, 17, 0.5, 0.5), (40, 37, 0.4, 0.55)]


def _fields(orc):
    return (orc.kappa2, orc.epsilon, orc.epsilon_spatial, orc.H, orc.mt, orc.psi, orc.abei, orc.ab)


def _perturb_A(gl, orc, seed):
    """Make A non-trivial (a gauge of H plus a random part) on both sides."""
    rng = np.random.default_rng(seed)
    ab = orc.ab + 0.3 * rng.standard_normal(orc.g.Nab)
    g = orc.g
    a = ab[: g.Na].reshape(g.Nya, g.Nxa).T
    b = ab[g.Na:].reshape(g.Nyb, g.Nxb).T
    gl.vars.vector_potential = (a.copy(), b.copy())
    orc.ab = ab


@pytest.mark.parametrize("geom", GEOMS)
@pytest.mark.parametrize("mask", ["none", "random30", "holes", "q1"])
@pytest.mark.parametrize("kappa", [np.inf, 3.0])
def test_observables_gradients_coefficients_match_reference(geom, mask, kappa):
    R = _ref()
    Nx, Ny, dx, dy = geom
    gl, orc = make_pair(Nx=Nx, Ny=Ny, dx=dx, dy=dy, kappa=kappa, sigma=20.0, H=0.2, mask=mask,
                        seed=Nx + len(mask), external_field=0.05)
    _perturb_A(gl, orc, Nx)
    g = orc.g
    f = _fields(orc)

    F_r, F_o, F_g = R.free_energy(g, *f), K.free_energy(g, *f), gl.observables.free_energy
    assert abs(F_o - F_r) <= 1e-13 * abs(F_r) and abs(F_g - F_r) <= 1e-12 * abs(F_r), (F_r, F_o, F_g)

    B_r = R.magnetic_field(g, orc.abei, orc.ab)
    assert rel_err(K.magnetic_field(g, orc.abei, orc.ab), B_r) < 1e-13
    assert rel_err(flat(gl.observables.magnetic_field), B_r) < 1e-12

    js_r = R.supercurrent_density(g, orc.mt, orc.psi, orc.abei, orc.ab)
    assert rel_err(K.supercurrent_density(g, orc.mt, orc.psi, orc.abei, orc.ab), js_r) < 1e-13
    sx, sy = gl.observables.supercurrent_density
    assert rel_err(np.concatenate([flat(sx), flat(sy)]), js_r) < 1e-12
    if np.isfinite(kappa):
        j_r = R.current_density(g, orc.kappa2, orc.H, orc.abei, orc.ab)
        assert rel_err(K.current_density(g, orc.kappa2, orc.H, orc.abei, orc.ab), j_r) < 1e-13
        jx, jy = gl.observables.current_density
        assert rel_err(np.concatenate([flat(jx), flat(jy)]), j_r) < 1e-12

    gl.solve._init_cg()
    gp_r = R.free_energy_jacobian_psi(g, *f)
    assert rel_err(K.free_energy_jacobian_psi(g, *f), gp_r) < 1e-13
    assert rel_err(gl.solve._cg._free_energy_jacobian_psi.get(), gp_r) < 1e-12

    rng = np.random.default_rng(3 + Nx)
    dpsi = rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N)
    if np.isfinite(kappa):
        gA_r = R.free_energy_jacobian_A(g, orc.kappa2, orc.H, orc.mt, orc.psi, orc.abei, orc.ab)
        assert rel_err(K.free_energy_jacobian_A(g, orc.kappa2, orc.H, orc.mt, orc.psi, orc.abei, orc.ab), gA_r) < 1e-13
        assert rel_err(gl.solve._cg._free_energy_jacobian_A.get(), gA_r) < 1e-12
        dab = 0.1 * rng.standard_normal(g.Nab)
        c_r = R.free_energy_conjgrad_coef_total(g, *f[:6], dpsi, orc.abei, orc.ab, dab)
        c_o = K.free_energy_conjgrad_coef_total(g, *f[:6], dpsi, orc.abei, orc.ab, dab)
        c_g = gl._h.conjgrad_coef(dpsi, dab)
    else:
        c_r = R.free_energy_conjgrad_coef_psi_total(g, *f[:6], dpsi, orc.abei, orc.ab)
        c_o = K.free_energy_conjgrad_coef_psi_total(g, *f[:6], dpsi, orc.abei, orc.ab)
        c_g = gl._h.conjgrad_coef(dpsi)
    scale = np.max(np.abs(c_r))
    assert np.max(np.abs(c_o - c_r)) <= 1e-13 * scale
    assert np.max(np.abs(c_g - c_r)) <= 1e-12 * scale


@pytest.mark.parametrize("geom", GEOMS)
@pytest.mark.parametrize("mask", ["none", "random30", "holes"])
@pytest.mark.parametrize("variant", ["plain", "langevin", "eps_spatial"])
def test_single_sweeps_oracle_matches_reference(geom, mask, variant):
    """One psi sweep and one A sweep from arbitrary (rhs != current) inputs."""
    R = _ref()
    Nx, Ny, dx, dy = geom
    rng = np.random.default_rng(Nx * 7 + len(mask) + len(variant))
    g = K.Grid(Nx, Ny, dx, dy)
    from tests._pairs import random_mask
    mt2 = random_mask(rng, Nx - 1, Ny - 1, mask)
    mt = None if mt2 is None else flat(mt2)
    psi = rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N)
    rhs = psi + 0.1 * (rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N))
    ab = 0.5 * rng.standard_normal(g.Nab)
    lang = 0.05 if variant == "langevin" else 0.0
    eps_sp = 1.0 + 0.2 * rng.standard_normal(g.N) if variant == "eps_spatial" else None
    for jstep in (0, 1):
        rr, ro = rhs.copy(), rhs.copy()
        n_r, c_r = R.iterate_order_parameter_jacobi_step(g, 0.1, 1.0, eps_sp, mt, ab, rr, psi, lang, jstep, 7, 1e-6)
        n_o, c_o = K.iterate_order_parameter_jacobi_step(g, 0.1, 1.0, eps_sp, mt, ab, ro, psi, lang, jstep, 7, 1e-6)
        assert rel_err(n_o, n_r) < 1e-13 and rel_err(ro, rr) < 1e-15
        assert abs(c_o - c_r) <= 1, (c_o, c_r)
    abr = ab + 0.01 * rng.standard_normal(g.Nab)
    X = ab + 0.02 * rng.standard_normal(g.Nab)
    for jstep in (0, 1):
        rr, ro = abr.copy(), abr.copy()
        n_r, c_r = R.iterate_vector_potential_jacobi_step(g, 0.1, 9.0, 0.05, 0.2, mt, psi, X, rr, ab, lang, jstep, 7, 1e-6)
        n_o, c_o = K.iterate_vector_potential_jacobi_step(g, 0.1, 9.0, 0.05, 0.2, mt, psi, X, ro, ab, lang, jstep, 7, 1e-6)
        assert rel_err(n_o, n_r) < 1e-13 and rel_err(ro, rr) < 1e-15
        assert abs(c_o - c_r) <= 1, (c_o, c_r)


@pytest.mark.parametrize("mask", ["none", "random30", "holes"])
@pytest.mark.parametrize("kappa,sigma", [(5.0, 200.0), (2.0, 10.0), (np.inf, 1.0)])
def test_td_trajectory_matches_reference(mask, kappa, sigma):
    R = _ref()
    gl, _ = make_pair(Nx=33, Ny=17, dx=0.5, dy=0.5, kappa=kappa, sigma=sigma, H=0.15, mask=mask, seed=9)
    ref = oracle_of(gl, rand_t=9, kernels=R)
    gl.solve.td(dt=0.1, Nt=12)
    ref.td(dt=0.1, Nt=12)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, ref.psi) < 1e-12 and rel_err(ab, ref.ab) < 1e-12
    st = gl.solve._td.last_stats
    assert st.total_sweeps_psi == sum(ref.sweeps_psi) and st.total_sweeps_A == sum(ref.sweeps_A)


def test_td_langevin_and_fixed_vortices_match_reference():
    R = _ref()
    gl, _ = make_pair(Nx=12, Ny=11, dx=0.5, dy=0.45, kappa=3.0, sigma=20.0, H=0.15, seed=7, langevin=(0.05, 0.02))
    ref = oracle_of(gl, rand_t=7, kernels=R)
    for eqn, nt in (("order_parameter", 4), ("vector_potential", 3), (None, 5)):
        gl.solve.td(dt=0.07, Nt=nt, eqn=eqn)
        ref.td(dt=0.07, Nt=nt, eqn=eqn)
        psi, ab = gpu_state(gl)
        assert rel_err(psi, ref.psi) < 1e-12 and rel_err(ab, ref.ab) < 1e-12, eqn


@pytest.mark.parametrize("gauge,nt", [("landau", 1000), ("symmetric", 300)])
def test_plain_small_workload_matches_reference(gauge, nt):
    """The 129x129 plain workload: dx = 0.5, kappa = 5, sigma = 200, H = 0.1,
    random psi, full domain; TD dt = 0.1 for nt steps, then CG."""
    R = _ref()
    gl, _ = make_pair(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=5.0, sigma=200.0, H=0.1, mask="none", seed=1,
                      landau=(gauge == "landau"))
    ref = oracle_of(gl, rand_t=1, kernels=R)
    errs = []
    done = g_psi = g_A = 0
    for chunk in (10, 90, nt - 100):
        gl.solve.td(dt=0.1, Nt=chunk)
        ref.td(dt=0.1, Nt=chunk)
        done += chunk
        g_psi += gl.solve._td.last_stats.total_sweeps_psi
        g_A += gl.solve._td.last_stats.total_sweeps_A
        psi, ab = gpu_state(gl)
        errs.append((done, rel_err(psi, ref.psi), rel_err(ab, ref.ab)))
    print("TD divergence (step, psi, A):", errs)
    st_psi, st_A = sum(ref.sweeps_psi), sum(ref.sweeps_A)
    assert errs[-1][1] < 1e-12 and errs[-1][2] < 1e-12, errs
    assert (g_psi, g_A) == (st_psi, st_A)
    F_r = ref.free_energy()
    assert abs(gl.observables.free_energy - F_r) <= 1e-12 * abs(F_r)
    psi, ab = gpu_state(gl)
    ox, oy, ov = O_detect(ref.g, ref.psi, ref.ab, 0.1)
    vx, vy, vv = gl.vortex_detector.vortices
    gx, gy, gv = O_detect(ref.g, psi, ab, 0.1)
    assert np.array_equal(np.asarray(vx), gx) and np.array_equal(np.asarray(vv), gv)
    assert len(ox) == len(gx)
    gl.solve.cg(n_iter=30)
    ref.cg(n_iter=30)
    e_g, e_r = np.array(gl.solve._cg.cg_energies), np.array(ref.cg_energies)
    n = min(len(e_g), len(e_r))
    assert n > 0 and np.max(np.abs(e_g[:n] - e_r[:n]) / np.abs(e_r[:n])) < 1e-6
    print("sweeps psi/A", st_psi, st_A, "CG energies", e_g[-1], e_r[-1])


def O_detect(g, psi, ab, H):
    from oracle import gl_oracle as O
    return O.detect_vortices(g, psi, ab, H)


def test_cg_kappa_inf_matches_reference():
    R = _ref()
    gl, _ = make_pair(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=np.inf, H=0.1, mask="none", seed=2, landau=True)
    ref = oracle_of(gl, rand_t=2, kernels=R)
    gl.solve.td(dt=0.1, Nt=20)
    ref.td(dt=0.1, Nt=20)
    gl.solve.cg(n_iter=200)
    ref.cg(n_iter=200)
    e_g, e_r = np.array(gl.solve._cg.cg_energies), np.array(ref.cg_energies)
    assert len(e_g) == len(e_r)
    assert np.max(np.abs(e_g - e_r) / np.abs(e_r)) < 1e-10
    psi, _ = gpu_state(gl)
    assert rel_err(psi, ref.psi) < 1e-8


def test_fp32_td_against_reference_fp32():
    R32 = _ref(np.float32)
    gl, _ = make_pair(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=5.0, sigma=200.0, H=0.1, mask="none", seed=1,
                      landau=True, dtype=np.float32)
    ref32 = oracle_of(gl, rand_t=1, kernels=R32)
    gl64, orc64 = make_pair(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=5.0, sigma=200.0, H=0.1, mask="none", seed=1,
                            landau=True)
    gl.solve.td(dt=0.1, Nt=20)
    ref32.td(dt=0.1, Nt=20)
    gl64.solve.td(dt=0.1, Nt=20)
    psi32, _ = gpu_state(gl)
    psi64, _ = gpu_state(gl64)
    d_gr = np.max(np.abs(psi32 - ref32.psi))
    print("FP32 after 20 steps: |G32 - R32| %.2e, |G32 - G64| %.2e, |R32 - G64| %.2e; sweeps G32 %d R32 %d" % (
        d_gr, np.max(np.abs(psi32 - psi64)), np.max(np.abs(ref32.psi - psi64)),
        gl.solve._td.last_stats.total_sweeps_psi, sum(ref32.sweeps_psi)))
    assert d_gr <= 1e-4


@pytest.mark.parametrize("tag", ["c1_k5_129", "c1_kinf_129"])
def test_libglgpu_matches_reference_fixtures(tag):
    """libglgpu against the committed outputs of the reference's kernels for the
    129x129 workloads (tests/golden/refk_*.npz); needs no reference build."""
    import os
    from tests.golden import make_refk_golden as M
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refk_%s.npz" % tag)
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    ref = np.load(path)
    spec = M.WORKLOADS[tag]
    gl, orc = make_pair(Nx=spec["Nx"], Ny=spec["Ny"], dx=spec["dx"], dy=spec["dy"], kappa=spec["kappa"],
                        sigma=spec["sigma"], H=spec["H"], mask="none", seed=spec["seed"], landau=True)
    assert abs(gl.observables.free_energy - ref["F0"]) <= 1e-12 * abs(ref["F0"])
    assert rel_err(flat(gl.observables.magnetic_field), ref["B0"]) < 1e-12
    sx, sy = gl.observables.supercurrent_density
    assert rel_err(np.concatenate([flat(sx), flat(sy)]), ref["js0"]) < 1e-12
    gl.solve._init_cg()
    assert rel_err(gl.solve._cg._free_energy_jacobian_psi.get(), ref["gpsi0"]) < 1e-12
    dpsi, dab = M.direction(orc.g, spec["seed"])
    if np.isfinite(spec["kappa"]):
        jx, jy = gl.observables.current_density
        assert rel_err(np.concatenate([flat(jx), flat(jy)]), ref["j0"]) < 1e-12
        assert rel_err(gl.solve._cg._free_energy_jacobian_A.get(), ref["gA0"]) < 1e-12
        c = gl._h.conjgrad_coef(dpsi, dab)
    else:
        c = gl._h.conjgrad_coef(dpsi)
    assert np.max(np.abs(c - ref["coef"])) <= 1e-12 * np.max(np.abs(ref["coef"]))
    gl.solve.td(dt=0.1, Nt=spec["td_steps"])
    psi, ab = gpu_state(gl)
    assert rel_err(psi, ref["psi_td"]) < 1e-12 and rel_err(ab, ref["ab_td"]) < 1e-12
    st = gl.solve._td.last_stats
    assert st.total_sweeps_psi == int(ref["sweeps_psi"].sum()) and st.total_sweeps_A == int(ref["sweeps_A"].sum())
    gl.solve.cg(n_iter=spec["cg_iters"])
    e, er = np.array(gl.solve._cg.cg_energies), ref["cg_energies"]
    n = min(len(e), len(er))
    assert n > 0 and np.max(np.abs(e[:n] - er[:n]) / np.abs(er[:n])) < (1e-10 if np.isinf(spec["kappa"]) else 1e-6)
