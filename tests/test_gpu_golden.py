"""The CUDA path (GLSolver through the C ABI) against the committed golden
fixtures of the reference (tests/golden/), FP64, at the parity tolerances:
observables and gradients 1e-12, coefficients 1e-11, TDGL state 1e-12 with the
same Jacobi sweep counts, CG energies 1e-10 (kappa = inf) / 1e-6 (finite
kappa: the reference's BFGS step, see test_gpu_parity), vortex list exact for
the reference's final state."""
import glob
import os

import numpy as np
import pytest

from tests._pairs import flat, gpu_state, rel_err

pytestmark = pytest.mark.gpu


def near(x, y, tol, floor):
    """max|x - y| <= tol * max(max|y|, floor): fields that vanish in a case (the
    current of the symmetric-gauge start) are rounding noise in both codes."""
    x, y = np.asarray(x), np.asarray(y)
    return np.max(np.abs(x - y)) <= tol * max(np.max(np.abs(y)), floor)

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "case_*.npz")))


def solver_of(f):
    from svirl_gb300 import GLSolver
    from oracle import gl_oracle as O
    Nx, Ny = int(f["Nx"]), int(f["Ny"])
    kw = dict(Nx=Nx, Ny=Ny, dx=float(f["dx"]), dy=float(f["dy"]), order_parameter="random", random_seed=int(f["seed"]),
              gl_parameter=float(f["kappa"]), normal_conductivity=float(f["sigma"]),
              homogeneous_external_field=float(f["H"]))
    if f["mt"].size:
        kw["material_tiling"] = O.unflatten_ij(f["mt"], Nx - 1, Ny - 1)
    if float(f["ext"]):
        kw["external_field"] = float(f["ext"])
    gl = GLSolver(**kw)
    gl.vars.order_parameter = O.unflatten_ij(f["psi0"], Nx, Ny)
    Na = (Nx - 1) * Ny
    gl.vars.vector_potential = (O.unflatten_ij(f["ab0"][:Na], Nx - 1, Ny), O.unflatten_ij(f["ab0"][Na:], Nx, Ny - 1))
    if f["abei"].size:
        ev = gl.params.external_vector_potential
        assert rel_err(np.concatenate([flat(ev[0]), flat(ev[1])]), f["abei"]) < 1e-14
    return gl


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_gpu_reproduces_golden(path):
    z = np.load(path)
    f = {k: z[k] for k in z.files}
    gl = solver_of(f)
    assert abs(gl.observables.free_energy - f["F0"]) <= 1e-12 * abs(f["F0"])
    assert near(flat(gl.observables.magnetic_field), f["B0"], 1e-12, float(f["H"]))
    jx, jy = gl.observables.current_density
    assert near(np.concatenate([flat(jx), flat(jy)]), f["j0"], 1e-12, 1.0)
    sx, sy = gl.observables.supercurrent_density
    assert near(np.concatenate([flat(sx), flat(sy)]), f["js0"], 1e-12, 1.0)
    gl.solve._init_cg()
    assert rel_err(gl.solve._cg._free_energy_jacobian_psi.get(), f["gpsi0"]) < 1e-12
    if np.isfinite(f["kappa"]):
        assert rel_err(gl.solve._cg._free_energy_jacobian_A.get(), f["gA0"]) < 1e-12
        c = gl._h.conjgrad_coef(f["dpsi"], f["dab"])
    else:
        c = gl._h.conjgrad_coef(f["dpsi"])
    assert np.max(np.abs(c - f["coef"])) <= 1e-11 * np.max(np.abs(f["coef"]))
    gl.solve.td(dt=0.1, Nt=int(f["td_steps"]))
    psi, ab = gpu_state(gl)
    assert rel_err(psi, f["psi_td"]) < 1e-12 and rel_err(ab, f["ab_td"]) < 1e-12
    assert gl.solve._td.last_stats.total_sweeps_psi == int(np.sum(f["sweeps_psi"]))
    gl.solve.cg(n_iter=int(f["cg_iters"]))
    tol = 1e-10 if np.isinf(f["kappa"]) else 1e-6
    E = np.array(gl.solve._cg.cg_energies)
    assert E.shape == f["cg_energies"].shape and rel_err(E, f["cg_energies"]) < tol
    # the vortex detector on the reference's final state
    Nx, Ny = int(f["Nx"]), int(f["Ny"])
    Na = (Nx - 1) * Ny
    from oracle import gl_oracle as O
    gl.vars.order_parameter = O.unflatten_ij(f["psi_cg"], Nx, Ny)
    gl.vars.vector_potential = (O.unflatten_ij(f["ab_cg"][:Na], Nx - 1, Ny), O.unflatten_ij(f["ab_cg"][Na:], Nx, Ny - 1))
    vx, vy, vv = gl.vortex_detector.vortices
    assert np.array_equal(vx, f["vx"]) and np.array_equal(vy, f["vy"]) and np.array_equal(vv, f["vv"])
