"""The NumPy oracle against outputs of the reference's own CUDA kernels (CPU).

``tests/golden/refk_*.npz`` hold what the reference's kernels (``svirl/cuda/*.h``,
compiled unchanged by ``oracle/ref_build.py``) computed on a GPU for the inputs
of the committed case fixtures and of the 129x129 workloads
(``tests/golden/make_refk_golden.py``).  The oracle recomputes every value from
the same inputs here, so the oracle's kernel arithmetic is pinned to the
reference's, not only to its host code.

Tolerances (relative to the largest magnitude of the field): kernels 1e-13;
TDGL states 1e-12 with equal Jacobi sweep counts; CG energies 1e-10 at
kappa = inf, 1e-6 at finite kappa (scipy BFGS picks the step lengths and moves
with 1e-16 changes of the coefficients).
"""
import glob
import os

import numpy as np
import pytest

from tests.golden import make_refk_golden as M

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(HERE, "refk_*.npz")))


def rel(x, y, floor=1e-300):
    """max|x - y| / max(max|y|, floor): a field that vanishes in a case (the
    current of a symmetric-gauge start) is rounding noise in both codes, so it is
    compared against the scale of the field it would have (H for B, 1 for j)."""
    x, y = np.asarray(x), np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), floor))


def _oracle_and_direction(name):
    tag = name[len("refk_"):]
    if tag in M.WORKLOADS:
        spec = M.WORKLOADS[tag]
        orc = M.workload_oracle(spec, None)
        dpsi, dab = M.direction(orc.g, spec["seed"])
        return orc, dpsi, dab, spec["td_steps"], spec["cg_iters"]
    d = np.load(os.path.join(HERE, tag + ".npz"))
    orc = M.case_oracle(d, None)
    if tag.startswith("fv_"):
        return orc, None, None, int(d["steps"][0]), 0
    return orc, d["dpsi"], (d["dab"] if "dab" in d.files else None), int(d["td_steps"]), int(d["cg_iters"])


def test_fixtures_present():
    assert len(FIXTURES) >= 7, FIXTURES


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[5:-4] for p in FIXTURES])
def test_oracle_matches_reference_kernels(path):
    ref = np.load(path)
    orc, dpsi, dab, nt, ncg = _oracle_and_direction(os.path.basename(path)[:-4])
    got = M.record(orc, M.K, dpsi, dab, td_steps=nt, cg_iters=0, fv=orc.vpi is not None)
    assert abs(got["F0"] - ref["F0"]) <= 1e-13 * abs(ref["F0"])
    floors = {"B0": orc.H, "js0": 1.0, "j0": 1.0, "gpsi0": 1e-300, "gA0": 1e-300}
    for k, floor in floors.items():
        if k in ref.files:
            assert rel(got[k], ref[k], floor) < 1e-13, k
    if "coef" in ref.files:
        assert np.max(np.abs(got["coef"] - ref["coef"])) <= 1e-13 * np.max(np.abs(ref["coef"]))
    if nt:
        assert np.array_equal(got["sweeps_psi"], ref["sweeps_psi"])
        assert np.array_equal(got["sweeps_A"], ref["sweeps_A"])
        assert rel(got["psi_td"], ref["psi_td"]) < 1e-12 and rel(got["ab_td"], ref["ab_td"]) < 1e-12
        assert abs(got["F_td"] - ref["F_td"]) <= 1e-12 * abs(ref["F_td"])
        if "vpi_td" in ref.files:
            assert rel(got["vpi_td"], ref["vpi_td"]) < 1e-12
    if ncg and "cg_energies" in ref.files:
        orc.cg(n_iter=ncg)
        e, er = np.array(orc.cg_energies), ref["cg_energies"]
        n = min(len(e), len(er))
        tol = 1e-10 if np.isinf(orc.kappa) else 1e-6
        assert n > 0 and np.max(np.abs(e[:n] - er[:n]) / np.abs(er[:n])) < tol
        if np.isinf(orc.kappa):
            assert len(e) == len(er)
