"""The oracle against the committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py from the reference's own host code on the NumPy
pycuda shim): observables, gradients and line-search coefficients at the
initial state, the TDGL state and Jacobi sweep counts, the CG energies and the
vortex list.  Needs neither the reference sources nor a GPU."""
import glob
import os

import numpy as np
import pytest

from oracle import gl_oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "case_*.npz")))
GOLDEN_FV = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fv_*.npz")))


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def oracle_of(f):
    mt = f["mt"] if f["mt"].size else None
    abei = f["abei"] if f["abei"].size else None
    return O.GLOracle(int(f["Nx"]), int(f["Ny"]), float(f["dx"]), float(f["dy"]), f["psi0"].copy(), f["ab0"].copy(),
                      mt=mt, abei=abei, kappa=float(f["kappa"]), sigma=float(f["sigma"]), H=float(f["H"]),
                      rand_t=int(f["seed"]))


def rel(x, y):
    return np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(np.asarray(y))), 1e-300)


def test_fixtures_present():
    assert len(GOLDEN) >= 3


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p))
def test_oracle_reproduces_golden(path):
    f = load(path)
    orc = oracle_of(f)
    assert abs(orc.free_energy() - f["F0"]) <= 1e-13 * abs(f["F0"])
    assert rel(orc.magnetic_field(), f["B0"]) < 1e-12
    assert rel(orc.current_density(), f["j0"]) < 1e-12
    assert rel(orc.supercurrent_density(), f["js0"]) < 1e-12
    assert rel(orc.jacobian_psi(), f["gpsi0"]) < 1e-12
    if np.isfinite(f["kappa"]):
        assert rel(orc.jacobian_A(), f["gA0"]) < 1e-12
        assert rel(orc.coef(f["dpsi"], f["dab"]), f["coef"]) < 1e-12
    else:
        assert rel(orc.coef_psi(f["dpsi"]), f["coef"]) < 1e-12
    orc.td(dt=0.1, Nt=int(f["td_steps"]))
    assert rel(orc.psi, f["psi_td"]) < 1e-13 and rel(orc.ab, f["ab_td"]) < 1e-13
    assert list(orc.sweeps_psi) == list(f["sweeps_psi"])
    orc.cg(n_iter=int(f["cg_iters"]))
    tol = 1e-13 if np.isinf(f["kappa"]) else 1e-8
    assert rel(orc.cg_energies, f["cg_energies"]) < tol
    vx, vy, vv = O.detect_vortices(orc.g, f["psi_cg"], f["ab_cg"], float(f["H"]))
    assert np.array_equal(vx, f["vx"]) and np.array_equal(vy, f["vy"]) and np.array_equal(vv, f["vv"])


def test_fixed_vortex_fixtures_present():
    assert len(GOLDEN_FV) >= 2


@pytest.mark.parametrize("path", GOLDEN_FV, ids=lambda p: os.path.basename(p))
def test_oracle_reproduces_fixed_vortex_golden(path):
    """Fixed vortices: the irregular vector potential around the psi and A steps
    (with the reference's element ranges), the phase lock, the three TD modes,
    the A_irr drift, the energy and the vortex list."""
    f = load(path)
    mt = f["mt"] if f["mt"].size else None
    abei = f["abei"] if f["abei"].size else None
    orc = O.GLOracle(int(f["Nx"]), int(f["Ny"]), float(f["dx"]), float(f["dy"]), f["psi0"].copy(), f["ab0"].copy(),
                     mt=mt, abei=abei, kappa=float(f["kappa"]), sigma=float(f["sigma"]), H=float(f["H"]),
                     rand_t=int(f["seed"]), vpi=f["ai0"].copy(), lock_ns=f["lock"])
    n0, n1, n2 = (int(x) for x in f["steps"])
    for tag, eqn, nt in (("td", None, n0), ("psi", "order_parameter", n1), ("A", "vector_potential", n2)):
        if nt == 0:
            continue
        orc.td(dt=0.1, Nt=nt, eqn=eqn)
        assert rel(orc.psi, f["psi_" + tag]) < 1e-13 and rel(orc.ab, f["ab_" + tag]) < 1e-13, tag
        assert rel(orc.vpi, f["vpi_" + tag]) < 1e-13, tag
    assert list(orc.sweeps_psi) == list(f["sweeps_psi"]) and list(orc.sweeps_A) == list(f["sweeps_A"])
    assert abs(orc.free_energy() - f["F"]) <= 1e-12 * abs(f["F"])
    g = orc.g
    ai = O.unflatten_ij(f["ai0"][:g.Na], g.Nx - 1, g.Ny), O.unflatten_ij(f["ai0"][g.Na:], g.Nx, g.Ny - 1)
    vx, vy, vv = O.detect_vortices(g, orc.psi, f["ab_host"], float(f["H"]), ai_bi=ai)
    assert np.array_equal(vx, f["vx"]) and np.array_equal(vy, f["vy"]) and np.array_equal(vv, f["vv"])


API = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "api_k4.npz")


def test_oracle_reproduces_api_golden():
    """The API-surface fixture (field delta/reset, randomize_order_parameter, td
    with an end time, normal current, superfluid density): the oracle's
    initial-state helpers and its TD step from the state after the field reset."""
    f = load(API)
    Nx, Ny = int(f["Nx"]), int(f["Ny"])
    assert rel(O.random_order_parameter(Nx * Ny, float(f["level"]), int(f["seed"])), f["psi0"]) < 1e-15
    assert rel(O.random_order_parameter(Nx * Ny, float(f["level2"]), int(f["seed2"])), f["psi1"]) < 1e-15
    orc = O.GLOracle(Nx, Ny, float(f["dx"]), float(f["dy"]), f["psi1"].copy(), f["ab3"].copy(), mt=f["mt"],
                     abei=f["abei"],
                     kappa=float(f["kappa"]), sigma=float(f["sigma"]), epsilon=float(f["eps"]), H=float(f["H3"]),
                     rand_t=int(f["seed"]))
    orc.td(dt=float(f["dt"]), Nt=int(f["Nt"]))
    assert rel(orc.psi, f["psi4"]) < 1e-13 and rel(orc.ab, f["ab4"]) < 1e-13
    assert abs(orc.free_energy() / float(f["F4"]) - 1.0) < 1e-13
    assert rel(orc.current_density() - orc.supercurrent_density(), f["jn4"]) < 1e-12
    assert rel(np.abs(orc.psi) ** 2, f["rho4"]) < 1e-13
