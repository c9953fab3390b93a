"""The GLSolver surface around the hot path against the golden fixture made by
the reference's own host code (tests/golden/api_k4.npz): a callable material
tiling (svirl/mesh/grid.py:102-120), random_level and
random_seed at construction (svirl/vars/vars.py:93-109), randomize_order_parameter,
homogeneous_external_field_delta and _reset (svirl/vars/params.py:135-170),
td with an end time (svirl/solvers/td.py:75-107), and the observables
normalcurrent_density and superfluid_density (svirl/observables/observables.py:29-33,113-121)."""
import os

import numpy as np
import pytest

from tests._pairs import flat, rel_err
from tests.golden.make_golden import api_material

pytestmark = pytest.mark.gpu

API = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "api_k4.npz")


def test_api_surface_matches_reference_golden():
    from svirl_gb300 import GLSolver
    z = np.load(API)
    f = {k: z[k] for k in z.files}
    gl = GLSolver(Nx=int(f["Nx"]), Ny=int(f["Ny"]), dx=float(f["dx"]), dy=float(f["dy"]), order_parameter="random",
                  random_seed=int(f["seed"]), random_level=float(f["level"]), gl_parameter=float(f["kappa"]),
                  normal_conductivity=float(f["sigma"]), linear_coefficient=float(f["eps"]),
                  homogeneous_external_field=float(f["H"]), external_field=float(f["ext"]), dtype=np.float64,
                  material_tiling=api_material)
    assert np.array_equal(flat(gl.mesh.material_tiling), f["mt"])

    def ab():
        a, b = gl.vars.vector_potential
        return np.concatenate([flat(a), flat(b)])

    assert rel_err(flat(gl.vars.order_parameter), f["psi0"]) < 1e-15
    assert rel_err(ab(), f["ab0"]) < 1e-15
    ei = gl.params.external_irregular_vector_potential
    assert rel_err(np.concatenate([flat(ei[0]), flat(ei[1])]), f["abei"]) < 1e-15
    gl.vars.randomize_order_parameter(level=float(f["level2"]), seed=int(f["seed2"]))
    assert rel_err(flat(gl.vars.order_parameter), f["psi1"]) < 1e-15
    gl.params.homogeneous_external_field_delta = float(f["dH"])
    assert float(gl.params.homogeneous_external_field) == float(f["H2"])
    assert rel_err(ab(), f["ab2"]) < 1e-15
    gl.params.homogeneous_external_field_reset = float(f["H_reset"])
    assert float(gl.params.homogeneous_external_field) == float(f["H3"])
    assert rel_err(ab(), f["ab3"]) < 1e-15
    dt, Nt = float(f["dt"]), int(f["Nt"])
    with pytest.raises(AssertionError):
        gl.solve.td(dt=dt, Nt=Nt, T=dt * Nt + 1.0)
    gl.solve.td(dt=dt, Nt=Nt, T=dt * Nt)
    assert rel_err(flat(gl.vars.order_parameter), f["psi4"]) < 1e-12
    assert rel_err(ab(), f["ab4"]) < 1e-12
    assert abs(gl.observables.free_energy / float(f["F4"]) - 1.0) < 1e-12
    assert rel_err(flat(gl.observables.magnetic_field), f["B4"]) < 1e-12
    jx, jy = gl.observables.current_density
    assert rel_err(np.concatenate([flat(jx), flat(jy)]), f["j4"]) < 1e-12
    sx, sy = gl.observables.supercurrent_density
    assert rel_err(np.concatenate([flat(sx), flat(sy)]), f["js4"]) < 1e-12
    nx_, ny_ = gl.observables.normalcurrent_density
    assert rel_err(np.concatenate([flat(nx_), flat(ny_)]), f["jn4"]) < 1e-12
    assert rel_err(flat(gl.observables.superfluid_density), f["rho4"]) < 1e-12
    gl.close()
