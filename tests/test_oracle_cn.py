"""The oracle's Crank-Nicolson sweeps (svirl/cuda/td.h:136-292, the reference's
commented-out kernel) on the CPU.

* "crank_nicolson" (explicit part from psi_rhs on all links) is the trapezoidal
  rule: for a uniform state on a field-free full domain the interior fixed point of
  its Jacobi loop is p (1 - dt/2 a) / (1 + dt/2 a), a = |p|^2 - 1.  The kernel
  takes the nonlinear coefficient |psi|^2 from the step's start (psi_rhs) in both
  halves, so over a relaxation run the step is first order in time like backward
  Euler (error against the same scheme at a fine step about halves when dt
  halves), with about half of backward Euler's error at equal dt.
* "crank_nicolson_as_written" takes three links' explicit part from psi (as the
  kernel is written): its fixed point is p (1 - c dt (a + idx2 + 2 idy2)) /
  (1 + c dt (a - idx2 - 2 idy2)), c = 1/2, which grows |p| (not a Crank-Nicolson
  step); pinned against the reference's own compiled kernel in
  tests/test_gpu_reference_kernels.py.
* The residual code is that of the squared change; the scheme switch leaves
  backward Euler untouched.
"""
import numpy as np

from oracle import gl_oracle as O
from oracle import kernels_np as K


def _fixed_point(as_written, p=0.6 + 0.3j, dt=0.1):
    g = K.Grid(9, 8, 0.5, 0.5)
    psi = np.full(g.N, p)
    cur = psi.copy()
    code = None
    for k in range(300):
        cur, code = K.iterate_order_parameter_jacobi_step_cn(g, dt, 1.0, None, None, np.zeros(g.Nab), psi.copy(), cur,
                                                             0.0, k, 1, 1e-12, as_written=as_written)
    return g, cur.reshape(g.Ny, g.Nx)[2:-2, 2:-2], code


def test_cn_fixed_point_is_the_trapezoidal_rule():
    p, c, a = 0.6 + 0.3j, 0.05, abs(0.6 + 0.3j) ** 2 - 1.0
    g, inner, code = _fixed_point(False)
    assert np.max(np.abs(inner - p * (1 - c * a) / (1 + c * a))) < 1e-12 and code < 10000


def test_cn_as_written_fixed_point():
    # the left link's explicit part comes from psi_rhs and the right one's from psi,
    # so the boundary columns perturb the interior: compare the middle column at 1 %
    p, c, a = 0.6 + 0.3j, 0.05, abs(0.6 + 0.3j) ** 2 - 1.0
    g, inner, code = _fixed_point(True)
    want = p * (1 - c * (a + g.idx2 + 2 * g.idy2)) / (1 + c * (a - g.idx2 - 2 * g.idy2))
    mid = inner[:, inner.shape[1] // 2]
    assert np.max(np.abs(mid - want)) < 1e-2 * abs(want) and abs(want) > 1.1 * abs(p)


def _run(scheme, dt, T=2.0):
    g = K.Grid(17, 15, 0.5, 0.5)
    psi = O.random_order_parameter(g.N, 0.3, 5)
    o = O.GLOracle(g.Nx, g.Ny, g.dx, g.dy, psi, np.zeros(g.Nab), kappa=np.inf, H=0.0, stop_psi=1e-12)
    o.scheme = scheme
    o.td(dt=dt, Nt=int(round(T / dt)))
    return o.psi


def test_time_step_convergence():
    err = {}
    for s in ("crank_nicolson", "backward_euler"):
        fine = _run(s, 0.0125)
        err[s] = [np.max(np.abs(_run(s, dt) - fine)) for dt in (0.1, 0.05)]
        assert 1.7 < err[s][0] / err[s][1] < 2.8, (s, err[s])
    assert err["crank_nicolson"][0] < 0.7 * err["backward_euler"][0], err


def test_residual_code_is_squared_change():
    g = K.Grid(6, 5, 0.5, 0.5)
    rng = np.random.default_rng(0)
    psi = rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N)
    nxt, code = K.iterate_order_parameter_jacobi_step_cn(g, 0.1, 1.0, None, None, np.zeros(g.Nab), psi.copy(), psi, 0.0, 1,
                                                         1, 1e-6)
    d = nxt - psi
    assert code == int(K.residual_code((d.real ** 2 + d.imag ** 2), 1e-6).max())


def test_scheme_switch_leaves_backward_euler():
    g = K.Grid(12, 11, 0.5, 0.45)
    psi = O.random_order_parameter(g.N, 1.0, 1)
    runs = {}
    for s in ("backward_euler", "crank_nicolson", "crank_nicolson_as_written", None):
        o = O.GLOracle(12, 11, 0.5, 0.45, psi, np.zeros(g.Nab), kappa=np.inf, H=0.1)
        if s:
            o.scheme = s
        o.td(dt=0.1, Nt=3)
        runs[s] = (o.psi, o.sweeps_psi)
    assert np.array_equal(runs[None][0], runs["backward_euler"][0]) and runs[None][1] == runs["backward_euler"][1]
    assert not np.allclose(runs["crank_nicolson"][0], runs["backward_euler"][0])
    assert not np.allclose(runs["crank_nicolson"][0], runs["crank_nicolson_as_written"][0])
