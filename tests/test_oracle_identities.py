"""The reference's kernel identities, checked on the oracle's kernel restatement.

Ports of the reference's own acceptance tests (they ship no golden vectors):
``tests/at_cg_jacobians.py`` (gradients vs finite differences of the free
energy), ``tests/at_cg_coef_psi.py`` (the 5 quartic coefficients reproduce
F(psi + alpha dpsi)) and ``tests/at_cg_coef.py`` (the 17 coefficients: exact
in alpha_psi, improving Taylor orders in alpha_A).  Same sizes (8-11 nodes),
same parameter ranges, same tolerances, seeded.
"""
import numpy as np
import pytest

from oracle import gl_oracle as O
from oracle import kernels_np as K


def material_tiling(rng, g, kind):
    """``tests/common.py:13-58`` mask kinds."""
    mt = np.full((g.Nxc, g.Nyc), True)
    if kind == "empty":
        mt[:] = False
    elif kind.startswith("random"):
        p = int(kind[6:]) / 100.0
        for _ in range(int(p * g.Nxc * g.Nyc)):
            mt[rng.integers(g.Nxc), rng.integers(g.Nyc)] = False
    elif kind == "q1":
        mt[: g.Nxc // 2, : g.Nxc // 2] = False
    elif kind == "q4":
        mt[g.Nxc // 2:, g.Nxc // 2:] = False
    elif kind == "none":
        return None
    return O.flatten_ij(mt)


def make_case(seed, kappa=None):
    rng = np.random.default_rng(seed)
    Nx, Ny = 8 + int(rng.integers(4)), 8 + int(rng.integers(4))
    dx, dy = 0.5 - 0.1 * rng.random(), 0.5 - 0.1 * rng.random()
    g = K.Grid(Nx, Ny, dx, dy)
    Lx, Ly = dx * (Nx - 1), dy * (Ny - 1)
    kappa = 1.0 + 3.0 * rng.random() if kappa is None else kappa
    psi = (1.0 - 0.5 * rng.random(g.N)) * np.exp(0.5j * np.pi * (2.0 * rng.random(g.N) - 1.0))
    H = 0.01 + 0.1 * rng.random()
    ab = O.symmetric_gauge(g, H, np.float64, Lx, Ly)
    abei = O.symmetric_gauge(g, 0.01 + 0.1 * rng.random(), np.float64, Lx, Ly)
    kind = ["full", "empty", "q1", "q4", "none", "random10", "random30", "random90"][seed % 8]
    mt = material_tiling(rng, g, kind)
    nm = O.node_mask(g, mt).reshape(-1)
    psi = np.where(nm, psi, 0.0)
    orc = O.GLOracle(Nx, Ny, dx, dy, psi, ab, mt=mt, abei=abei, kappa=kappa, H=H)
    return orc, rng


@pytest.mark.parametrize("seed", range(8))
def test_jacobians_match_finite_differences(seed):
    orc, _ = make_case(seed)
    h = 3e-9
    E0 = orc.free_energy()
    jp = orc.jacobian_psi()
    fd = np.empty_like(jp)
    psi0 = orc.psi.copy()
    for n in range(orc.g.N):
        orc.psi = psi0.copy(); orc.psi[n] += h
        re = (orc.free_energy() - E0) / h
        orc.psi = psi0.copy(); orc.psi[n] += 1j * h
        im = (orc.free_energy() - E0) / h
        fd[n] = re + 1j * im
    orc.psi = psi0
    assert np.allclose(jp, fd, atol=1e-5, rtol=1e-3)
    jA = orc.jacobian_A()
    ab0 = orc.ab.copy()
    fdA = np.empty_like(jA)
    for n in range(orc.g.Nab):
        orc.ab = ab0.copy(); orc.ab[n] += h
        fdA[n] = (orc.free_energy() - E0) / h
    orc.ab = ab0
    assert np.allclose(jA, fdA, atol=1e-5, rtol=1e-3)


@pytest.mark.parametrize("seed", range(4))
def test_exact_A_jacobian_matches_finite_differences(seed):
    """``free_energy_jacobian_A_exact`` (used by the device CG's exact-boundary
    mode) is the derivative of the free energy on every link, and equals the
    reference's dF/dA on the interior links, also where curl A != H."""
    orc, rng = make_case(seed)
    orc.ab = orc.ab + 0.05 * rng.standard_normal(orc.g.Nab)
    g = orc.g
    args = (g, orc.kappa2, orc.H, orc.mt, orc.psi, orc.abei, orc.ab)
    jx = K.free_energy_jacobian_A_exact(*args)
    jr = K.free_energy_jacobian_A(*args)
    E0 = orc.free_energy()
    h = 1e-7
    ab0 = orc.ab.copy()
    fd = np.empty_like(jx)
    for n in range(g.Nab):
        orc.ab = ab0.copy(); orc.ab[n] += h
        Ep = orc.free_energy()
        orc.ab = ab0.copy(); orc.ab[n] -= h
        fd[n] = (Ep - orc.free_energy()) / (2 * h)
    orc.ab = ab0
    assert np.allclose(jx, fd, atol=1e-7, rtol=1e-6)
    a_int = np.zeros((g.Ny, g.Nx - 1), bool); a_int[1:-1, :] = True
    b_int = np.zeros((g.Ny - 1, g.Nx), bool); b_int[:, 1:-1] = True
    interior = np.concatenate([a_int.reshape(-1), b_int.reshape(-1)])
    assert np.allclose(jx[interior], jr[interior], atol=1e-12, rtol=1e-10)
    assert not np.allclose(jx[~interior], jr[~interior], atol=1e-7)


@pytest.mark.parametrize("seed", range(6))
def test_coef_psi_polynomial_reproduces_energy(seed):
    orc, rng = make_case(100 + seed, kappa=np.inf)
    orc.abei = None
    cases = [[1.0, 0.0, 0.0], [0.0, 1.0, 1.0], [0.5, 0.5, 1.0]]
    for _ in range(4):
        al, b = rng.random(2)
        cases.append([1.0 - b * al, b, al])
    psi0 = orc.psi.copy()
    for a, b, al in cases:
        orc.psi = psi0.copy()
        E0 = orc.free_energy()
        orc.psi = psi0 * a
        c = orc.coef_psi(psi0 * b)
        P = c[4] * al ** 4 + c[3] * al ** 3 + c[2] * al ** 2 + c[1] * al + c[0]
        assert np.isclose(P, E0)


@pytest.mark.parametrize("r", [0.0001, 0.01, 0.3, 1.0])
def test_coef17_exact_in_psi_and_converging_in_A(r):
    orc, rng = make_case(200, kappa=1.0 + 3.0 * 0.4)
    psi0, ab0 = orc.psi.copy(), orc.ab.copy()
    rows = [[1.0, 0.0, 0.0, 1.0 - r, r, 1.0],
            [0.5, 0.5, 1.0, 1.0 - r, r, 1.0],
            [0.6976, 0.72, 0.42, 1.0 - r, r, 1.0],
            [0.7923, 0.31, 0.67, 1.0 - 0.6 * r, 0.6 * r, 1.0]]
    for j, (a_p, b_p, al_p, a_A, b_A, al_A) in enumerate(rows):
        orc.psi, orc.ab = psi0.copy(), ab0.copy()
        E0 = orc.free_energy()
        orc.psi, orc.ab = psi0 * a_p, ab0 * a_A
        c = O.GLOracle.coef_matrix(orc.coef(psi0 * b_p, ab0 * b_A))
        E1 = orc.free_energy()

        def P(order):
            s = c[3, 0] * al_p ** 3 + c[4, 0] * al_p ** 4
            for i in range(3):
                s += sum(c[i, k] * al_A ** k for k in range(order + 1)) * al_p ** i
            return s
        assert np.isclose(P(4), E0)
        if j == 0:
            assert np.isclose(P(0), E1)
        approx = np.abs(np.array([P(0), P(2), P(4)]) - E0)
        approx[approx < 1e-9] = 0.0
        assert np.all(np.diff(approx) < 1e-14)


def test_rand_hash_known_values():
    """Thomas Wang's hash on a few inputs, computed by hand from its definition."""
    def ref(s):
        s &= 0xFFFFFFFF
        s = (s ^ 61) ^ (s >> 16)
        s = (s * 9) & 0xFFFFFFFF
        s = s ^ (s >> 4)
        s = (s * 0x27D4EB2D) & 0xFFFFFFFF
        s = s ^ (s >> 15)
        return s
    xs = np.array([0, 1, 61, 12345, 0xFFFFFFFF, 2 ** 31], dtype=np.uint64)
    assert [int(v) for v in K.rand_hash(xs.astype(np.uint32))] == [ref(int(x)) for x in xs]


def test_residual_code_matches_stop_rule():
    eps = 1e-6
    r = np.array([0.0, 0.99999e-6, 1e-6, 5.0, np.nan])
    code = K.residual_code(r, eps)
    assert list(code) == [0, 9999, 10000, 100000000, 0]
