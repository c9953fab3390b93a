"""Fixed vortices on the CUDA path against the reference's golden fixtures
(tests/golden/fv_*.npz, FP64): the irregular vector potential and phase-lock
list the solver builds from the vortex positions, TDGL in the combined,
psi-only and A-only modes (A_irr added to the first N link values around the
psi step, A added to A_irr around the A loop, the phase lock), the drift of the
device copy of A_irr, the free energy and the vortex list; then a batch
containing a fixed-vortex instance (bitwise equal to the instance alone) and a
checkpoint round trip with fixed vortices (bitwise resume)."""
import glob
import os

import numpy as np
import pytest

from tests._pairs import flat, gpu_state, rel_err

pytestmark = pytest.mark.gpu

GOLDEN_FV = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fv_*.npz")))


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def solver_of(f, dtype=np.float64):
    from svirl_gb300 import GLSolver
    from oracle import gl_oracle as O
    Nx, Ny = int(f["Nx"]), int(f["Ny"])
    vx, vy, vv = f["vort_in"]
    kw = dict(Nx=Nx, Ny=Ny, dx=float(f["dx"]), dy=float(f["dy"]), order_parameter="random", random_seed=int(f["seed"]),
              gl_parameter=float(f["kappa"]), normal_conductivity=float(f["sigma"]),
              homogeneous_external_field=float(f["H"]), fixed_vortices=(vx, vy, vv),
              fixed_vortices_correction="cell centers", phase_lock_radius=float(f["lock_radius"]), dtype=dtype)
    if f["mt"].size:
        kw["material_tiling"] = O.unflatten_ij(f["mt"], Nx - 1, Ny - 1)
    gl = GLSolver(**kw)
    gl.vars.order_parameter = O.unflatten_ij(f["psi0"], Nx, Ny)
    Na = (Nx - 1) * Ny
    gl.vars.vector_potential = (O.unflatten_ij(f["ab0"][:Na], Nx - 1, Ny), O.unflatten_ij(f["ab0"][Na:], Nx, Ny - 1))
    return gl


@pytest.mark.parametrize("path", GOLDEN_FV, ids=lambda p: os.path.basename(p))
def test_fixed_vortices_reproduce_golden(path):
    f = load(path)
    gl = solver_of(f)
    fvs = gl.params.fixed_vortices
    ai, bi = fvs.irregular_vector_potential
    assert rel_err(np.concatenate([flat(ai), flat(bi)]), f["ai0"]) < 1e-15
    assert np.allclose(np.stack(fvs.fixed_vortices), f["fv"], rtol=0, atol=1e-15)
    ei = gl.params.external_irregular_vector_potential
    assert rel_err(np.concatenate([flat(ei[0]), flat(ei[1])]), f["abei"]) < 1e-15
    n0, n1, n2 = (int(x) for x in f["steps"])
    sweeps = 0
    for tag, eqn, nt in (("td", None, n0), ("psi", "order_parameter", n1), ("A", "vector_potential", n2)):
        if nt == 0:
            continue
        gl.solve.td(dt=0.1, Nt=nt, eqn=eqn)
        sweeps += int(gl.solve._td.last_stats.total_sweeps_psi)
        psi, ab = gpu_state(gl)
        assert rel_err(psi, f["psi_" + tag]) < 1e-12 and rel_err(ab, f["ab_" + tag]) < 1e-12, tag
        assert rel_err(gl._h.get_irregular_vector_potential(), f["vpi_" + tag]) < 1e-12, tag
    assert sweeps == int(np.sum(f["sweeps_psi"]))
    assert abs(gl.observables.free_energy - f["F"]) <= 1e-12 * abs(f["F"])
    # the vortex list of the final state (the reference's detector read its host copy of A)
    from oracle import gl_oracle as O
    Nx, Ny = int(f["Nx"]), int(f["Ny"])
    Na = (Nx - 1) * Ny
    gl.vars.vector_potential = (O.unflatten_ij(f["ab_host"][:Na], Nx - 1, Ny),
                                O.unflatten_ij(f["ab_host"][Na:], Nx, Ny - 1))
    gl.solve.vortices_detected = False
    vx, vy, vv = gl.vortex_detector.vortices
    assert np.array_equal(vv, f["vv"]) and np.allclose(vx, f["vx"], atol=1e-12) and np.allclose(vy, f["vy"], atol=1e-12)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fixed_vortex_instance_in_a_batch(dtype):
    from svirl_gb300.batch import GLBatch
    f = load(GOLDEN_FV[0])
    alone = solver_of(f, dtype)
    alone.solve.td(dt=0.1, Nt=3)
    from svirl_gb300 import GLSolver
    others = [GLSolver(Nx=21, Ny=17, dx=0.5, dy=0.5, random_seed=s, gl_parameter=k, normal_conductivity=100.0,
                       homogeneous_external_field=0.1, dtype=dtype) for s, k in ((1, 2.0), (2, np.inf))]
    inb = solver_of(f, dtype)
    GLBatch([others[0], inb, others[1]]).td(dt=0.1, Nt=3)
    pa, aa = gpu_state(alone)
    pb, ab = gpu_state(inb)
    assert np.array_equal(pa, pb) and np.array_equal(aa, ab)
    assert np.array_equal(alone._h.get_irregular_vector_potential(), inb._h.get_irregular_vector_potential())


def test_fixed_vortex_checkpoint_resumes_bitwise(tmp_path):
    from svirl_gb300 import checkpoint
    f = load(GOLDEN_FV[0])
    a = solver_of(f)
    a.solve.td(dt=0.1, Nt=4)
    b = solver_of(f)
    b.solve.td(dt=0.1, Nt=2)
    path = str(tmp_path / "fv.npz")
    checkpoint.save(b, path)
    c = checkpoint.load(path)
    c.solve.td(dt=0.1, Nt=2)
    pa, aa = gpu_state(a)
    pc, ac = gpu_state(c)
    assert np.array_equal(pa, pc) and np.array_equal(aa, ac)
    assert np.array_equal(a._h.get_irregular_vector_potential(), c._h.get_irregular_vector_potential())


def test_release_moves_the_phase_into_psi():
    f = load(GOLDEN_FV[0])
    gl = solver_of(f)
    fvs = gl.params.fixed_vortices
    phase = fvs.fixed_vortices_phase
    psi0 = gl.vars.order_parameter
    fvs.fixed_vortices_release()
    assert np.allclose(gl.vars.order_parameter, psi0 * np.exp(-1j * phase), rtol=0, atol=1e-13)
    assert fvs.fixed_vortices_x.size == 0 and fvs.phase_lock_radius is None
    assert not np.any(gl._h.get_irregular_vector_potential())


@pytest.mark.parametrize("path", GOLDEN_FV, ids=lambda p: os.path.basename(p))
def test_fixed_vortices_fp32_near_golden(path):
    """The FP32 path with fixed vortices against the reference's FP64 states
    (FP32 rounding only: 1e-4 after the combined and psi-only steps)."""
    f = load(path)
    gl = solver_of(f, np.float32)
    n0, n1, _ = (int(x) for x in f["steps"])
    gl.solve.td(dt=0.1, Nt=n0)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, f["psi_td"]) < 1e-4 and rel_err(ab, f["ab_td"]) < 1e-4
    gl.solve.td(dt=0.1, Nt=n1, eqn="order_parameter")
    psi, ab = gpu_state(gl)
    assert rel_err(psi, f["psi_psi"]) < 1e-4 and rel_err(ab, f["ab_psi"]) < 1e-4
