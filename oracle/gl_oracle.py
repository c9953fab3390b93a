"""CPU oracle: host-level restatement of svirl's 2D GL solver (TDGL, CG, observables,
vortex detector) on top of the NumPy kernels in ``oracle/kernels_np.py``.

TEST INFRASTRUCTURE ONLY (see ``oracle/kernels_np.py``).  It follows the
reference's host code step for step, including its quirks:

* TD time loop and per-step Jacobi loops, <=1024 sweeps, stop when
  ``1e-4*dtype(max code) < 1`` (``svirl/solvers/td.py:157-218,252-325,342-366``);
* stop-criterion clamp 1e-6 (FP32) / 1e-12 (FP64) (``svirl/solvers/td.py:52-66``);
* in the A loop the supercurrent is evaluated with the buffer that held A at
  loop entry, which the pointer swap overwrites every second sweep
  (``svirl/solvers/td.py:266,303``): sweep k sees A^(2*floor(k/2));
* the A kernel receives ``self.dt`` (``svirl/solvers/td.py:278``);
* CG: Polak-Ribiere+ (beta >= 0), quartic line search via ``polyroots`` (kappa=inf),
  2-D polynomial BFGS (finite kappa), energy-ratio stop, and persistent
  direction/beta across calls (``svirl/solvers/cg.py``).

Parity pinning: ``tests/test_oracle_vs_reference.py`` runs the reference's own host
code (through ``oracle/fake_pycuda``) against this module, and
``tests/golden/make_golden.py`` stores reference-run fixtures.
"""

import numpy as np
import scipy.optimize

from oracle import kernels_np as K


# ---------------------------------------------------------------------------
# initial state as GLSolver builds it
# ---------------------------------------------------------------------------

def geometry(Nx=None, dx=None, Lx=None, Ny=None, dy=None, Ly=None):
    """Two of (N, d, L) per axis (``svirl/__init__.py:73-93``)."""
    def one(N, d, L):
        if N is not None and L is not None and d is None:
            d = float(L) / (N - 1)
        elif N is not None and L is None and d is not None:
            L = float(d) * (N - 1)
        elif N is None and L is not None and d is not None:
            N = int(np.round(L / d) + 1)
        return N, d, L
    Nx, dx, Lx = one(Nx, dx, Lx)
    Ny, dy, Ly = one(Ny, dy, Ly)
    return Nx, dx, Lx, Ny, dy, Ly


def node_mask(g, mt):
    """OR of the 4 adjacent cells (``svirl/mesh/grid.py:160-171``); (Ny, Nx) bool."""
    if mt is None:
        return np.ones((g.Ny, g.Nx), dtype=bool)
    mm, mp, pm, pp = K._cells_at_nodes(g, mt)
    return mm | mp | pm | pp


def random_order_parameter(N, level=1.0, seed=None):
    """``Vars.randomize_order_parameter`` (``svirl/vars/vars.py:93-109``): legacy MT19937."""
    if seed is not None:
        np.random.seed(seed)
    return (1.0 - level * np.random.rand(N)) * np.exp(level * 1.0j * np.pi * (2.0 * np.random.rand(N) - 1.0))


def symmetric_gauge(g, H, dtype, Lx, Ly):
    """A of a homogeneous field H in the g=0.5 gauge (``svirl/vars/params.py:135-170``)."""
    dt_ = dtype
    xa = np.linspace(0.5 * dt_(g.dx), dt_(Lx) - 0.5 * dt_(g.dx), num=g.Nxa, endpoint=True, dtype=dt_)
    ya = np.linspace(0.0, dt_(Ly), num=g.Nya, endpoint=True, dtype=dt_)
    xb = np.linspace(0.0, dt_(Lx), num=g.Nxb, endpoint=True, dtype=dt_)
    yb = np.linspace(0.5 * dt_(g.dy), dt_(Ly) - 0.5 * dt_(g.dy), num=g.Nyb, endpoint=True, dtype=dt_)
    _, yg = np.meshgrid(xa, ya, indexing="ij")
    xg, _ = np.meshgrid(xb, yb, indexing="ij")
    a = np.zeros((g.Nxa, g.Nya), dtype=dt_)
    b = np.zeros((g.Nxb, g.Nyb), dtype=dt_)
    dH = dt_(H)
    a -= 0.5 * (yg - 0.5 * dt_(Ly)) * dH
    b += (1.0 - 0.5) * (xg - 0.5 * dt_(Lx)) * dH
    return np.concatenate([a.T.reshape(-1), b.T.reshape(-1)])


def flatten_ij(x):
    """(Nx, Ny) user array -> flat n = i + Nx*j (``svirl/storage/arrays.py:327-331``)."""
    return np.reshape(np.asarray(x).T, -1)


def unflatten_ij(x, nx, ny):
    return np.reshape(x, (ny, nx)).T


# ---------------------------------------------------------------------------
# the oracle solver
# ---------------------------------------------------------------------------

class GLOracle:
    """One GL instance in flat reference layout, FP64 arithmetic.

    ``psi`` complex (N,), ``ab`` real (Nab,), ``mt`` bool cells (Nc,) or None,
    ``abei`` real (Nab,) or None (external + irregular vector potential),
    ``vpi`` real (Nab,) or None (irregular vector potential of fixed vortices, as
    the TD step uses it), ``lock_ns`` int node indices or None (phase lock).
    """

    def __init__(self, Nx, Ny, dx, dy, psi, ab, mt=None, abei=None, kappa=np.inf, sigma=1.0,
                 epsilon=1.0, epsilon_spatial=None, H=0.0, stop_psi=1e-6, stop_A=1e-6,
                 rand_t=1, langevin_psi=0.0, langevin_A=0.0, convergence_rtol=1e-6,
                 dtype=np.float64, vpi=None, lock_ns=None, kernels=None):
        # kernels: a module or object with kernels_np's functions; oracle.ref_gpu.RefKernels
        # runs these host loops on the reference's own compiled kernels instead
        self.K = K if kernels is None else kernels
        # psi time stepping: "backward_euler" (the reference's), "crank_nicolson" or
        # "crank_nicolson_as_written" (the reference's commented-out kernel,
        # td.h:136-292, see kernels_np), with the same host loop
        self.scheme = "backward_euler"
        self.g = K.Grid(Nx, Ny, dx, dy)
        self.dtype = dtype
        self.psi = np.array(psi, dtype=np.complex128).reshape(-1).copy()
        self.ab = np.array(ab, dtype=np.float64).reshape(-1).copy()
        self.mt = None if mt is None else np.asarray(mt, dtype=bool).reshape(-1).copy()
        self.abei = None if abei is None else np.asarray(abei, dtype=np.float64).reshape(-1).copy()
        self.vpi = None if vpi is None else np.asarray(vpi, dtype=np.float64).reshape(-1).copy()
        self.lock_ns = None if lock_ns is None or len(lock_ns) == 0 else np.asarray(lock_ns, dtype=np.int64).copy()
        self.kappa = float(kappa)
        self.sigma = float(sigma)
        self.rho = 1.0 / self.sigma
        self.epsilon = float(epsilon)
        self.epsilon_spatial = epsilon_spatial
        self.H = float(H)
        self.stop_psi = float(stop_psi)
        self.stop_A = float(stop_A)
        self.rand_t = int(rand_t)
        self.langevin_psi = float(langevin_psi)
        self.langevin_A = float(langevin_A)
        self.convergence_rtol = float(convergence_rtol)
        self._cg_state = None
        self._dt = None                   # TD.dt: also what the A kernel receives (td.py:278)
        self.sweeps_psi = []
        self.sweeps_A = []
        self.cg_energies = []

    # params -----------------------------------------------------------------
    @property
    def solveA(self):
        return not np.isposinf(self.kappa)

    @property
    def kappa2(self):
        return self.kappa ** 2 if self.solveA else -1.0

    def _clamped_stops(self):
        lo = 1e-6 if self.dtype is np.float32 else 1e-12
        return max(self.stop_psi, lo), max(self.stop_A, lo)

    @staticmethod
    def _converged(code, dtype):
        return 1.0e-4 * dtype(code) < 1.0

    # TDGL ---------------------------------------------------------------------
    def _psi_step(self, dt, stop):
        g = self.g
        rhs = self.psi.copy()
        cur = self.psi
        nsw = 0
        if self.scheme == "backward_euler":
            sweep = self.K.iterate_order_parameter_jacobi_step
        else:
            aw = self.scheme == "crank_nicolson_as_written"
            sweep = lambda *a: self.K.iterate_order_parameter_jacobi_step_cn(*a, as_written=aw)  # noqa: E731
        for j in range(1024):
            nxt, code = sweep(
                g, dt, self.epsilon, self.epsilon_spatial, self.mt, self.ab, rhs, cur,
                self.langevin_psi, j, self.rand_t, stop)
            cur = nxt
            nsw += 1
            if self._converged(code, self.dtype):
                break
        self.psi = cur
        self.rand_t = (self.rand_t + 1) & 0xFFFFFFFF
        self.sweeps_psi.append(nsw)
        if self.lock_ns is not None:  # td.py:206-216
            self.K.order_parameter_phase_lock(self.psi, self.lock_ns)

    # fixed vortices around the psi step (td.py:120-154): xpy_r / xmy_r over the
    # first N elements of the link array
    def _fv_pre(self):
        if self.vpi is not None:
            N = self.g.N
            self.ab[:N] += self.vpi[:N]

    def _fv_post(self):
        if self.vpi is not None:
            N = self.g.N
            self.ab[:N] -= self.vpi[:N]

    def _A_step(self, dt, stop):
        g = self.g
        if self.vpi is not None:
            # td.py:256-270: A_irr += A on the first N elements, and A_irr is the
            # supercurrent argument (no aliasing with the A iterates)
            self.vpi[:g.N] += self.ab[:g.N]
            X = self.vpi
            cur, nxt_buf = self.ab, np.empty_like(self.ab)
        else:
            X = self.ab                       # buffer bound to the supercurrent argument
            cur, nxt_buf = X, np.empty_like(X)
        rhs = self.ab.copy()
        nsw = 0
        for j in range(1024):
            vals, code = self.K.iterate_vector_potential_jacobi_step(
                g, dt, self.kappa2, self.rho, self.H, self.mt, self.psi, X, rhs, cur,
                self.langevin_A, j, self.rand_t, stop)
            nxt_buf[:] = vals
            cur, nxt_buf = nxt_buf, cur
            nsw += 1
            if self._converged(code, self.dtype):
                break
        self.ab = cur
        self.rand_t = (self.rand_t + 1) & 0xFFFFFFFF
        self.sweeps_A.append(nsw)
        if self.vpi is not None:  # td.py:314-322
            self.vpi[:g.N] -= self.ab[:g.N]

    def td(self, dt=0.1, Nt=1000, eqn=None):
        """``TD._solve`` (``svirl/solvers/td.py:370-377``)."""
        dt = float(self.dtype(dt))
        sp, sa = self._clamped_stops()
        if eqn == "order_parameter":
            # td.py:216-223: A += A_irr once before the time loop, A -= A_irr after every step
            self._dt = dt
            self._fv_pre()
            for _ in range(Nt):
                self._psi_step(dt, sp)
                self._fv_post()
        elif eqn == "vector_potential":
            if self.solveA:
                if self._dt is None:
                    raise TypeError("the vector-potential step uses the order-parameter dt, which is unset")
                for _ in range(Nt):
                    self._A_step(self._dt, sa)
        else:
            self._dt = dt
            for _ in range(Nt):
                self._fv_pre()
                self._psi_step(dt, sp)
                self._fv_post()
                if self.solveA:
                    self._A_step(dt, sa)

    # observables --------------------------------------------------------------
    def free_energy(self):
        return self.K.free_energy(self.g, self.kappa2, self.epsilon, self.epsilon_spatial, self.H,
                             self.mt, self.psi, self.abei, self.ab)

    def magnetic_field(self):
        return self.K.magnetic_field(self.g, self.abei, self.ab)

    def supercurrent_density(self):
        return self.K.supercurrent_density(self.g, self.mt, self.psi, self.abei, self.ab)

    def current_density(self):
        if not self.solveA:
            return self.supercurrent_density()
        return self.K.current_density(self.g, self.kappa2, self.H, self.abei, self.ab)

    def jacobian_psi(self):
        return self.K.free_energy_jacobian_psi(self.g, self.kappa2, self.epsilon, self.epsilon_spatial, self.H,
                                          self.mt, self.psi, self.abei, self.ab)

    def jacobian_A(self):
        return self.K.free_energy_jacobian_A(self.g, self.kappa2, self.H, self.mt, self.psi, self.abei, self.ab)

    def coef_psi(self, dpsi):
        return self.K.free_energy_conjgrad_coef_psi_total(self.g, self.kappa2, self.epsilon, self.epsilon_spatial,
                                                     self.H, self.mt, self.psi, dpsi, self.abei, self.ab)

    def coef(self, dpsi, dab):
        return self.K.free_energy_conjgrad_coef_total(self.g, self.kappa2, self.epsilon, self.epsilon_spatial,
                                                 self.H, self.mt, self.psi, dpsi, self.abei, self.ab, dab)

    # CG -----------------------------------------------------------------------
    @staticmethod
    def alpha_psi(c):
        """``CG._cg_alpha_psi_min`` (``svirl/solvers/cg.py:227-235``)."""
        am = np.polynomial.polynomial.polyroots([c[1], 2.0 * c[2], 3.0 * c[3], 4.0 * c[4]])
        am = am[np.isclose(am.imag, 0)].real
        am = am[am >= 0]
        return np.min(am)

    @staticmethod
    def coef_matrix(c17):
        c = np.zeros((5, 5))
        c[0, :] = c17[0:5]
        c[1, :] = c17[5:10]
        c[2, :] = c17[10:15]
        c[3, 0] = c17[15]
        c[4, 0] = c17[16]
        return c

    @staticmethod
    def alpha_joint(c, alpha0=(0.0, 0.0), tol=1e-8):
        """``CG._cg_alpha_min`` (``svirl/solvers/cg.py:378-419``)."""
        cj0 = np.polynomial.polynomial.polyder(c, axis=0)
        cj1 = np.polynomial.polynomial.polyder(c, axis=1)

        def f(al):
            return np.polynomial.polynomial.polyval2d(al[0], al[1], c)

        def jac(al):
            return np.array([np.polynomial.polynomial.polyval2d(al[0], al[1], cj0),
                             np.polynomial.polynomial.polyval2d(al[0], al[1], cj1)])

        r = scipy.optimize.minimize(f, x0=np.array(alpha0), jac=jac, method="BFGS", tol=tol)
        return r.x

    def cg(self, n_iter=1000):
        """``CG._solve`` (``svirl/solvers/cg.py:554-558``)."""
        g = self.g
        if self._cg_state is None:
            self._cg_state = dict(dir_psi=np.zeros(g.N, complex), jac_psi_prev=np.zeros(g.N, complex),
                                  beta_psi=0.0, dir_A=np.zeros(g.Nab), jac_A_prev=np.zeros(g.Nab), beta_A=0.0)
        st = self._cg_state
        self.cg_energies = []
        if not self.solveA:
            st["dir_psi"][:] = 0.0
        for i in range(n_iter):
            jp = self.jacobian_psi()
            if self.solveA:
                jA = self.jacobian_A()
            if i > 0:
                den = np.sum(st["jac_psi_prev"].real ** 2 + st["jac_psi_prev"].imag ** 2)
                num = np.sum(jp.real * (jp.real - st["jac_psi_prev"].real) + jp.imag * (jp.imag - st["jac_psi_prev"].imag))
                with np.errstate(divide="ignore", invalid="ignore"):
                    st["beta_psi"] = float(np.fmax(num / den, 0.0))
                if self.solveA:
                    den = np.sum(st["jac_A_prev"] ** 2)
                    num = np.sum(jA * (jA - st["jac_A_prev"]))
                    with np.errstate(divide="ignore", invalid="ignore"):
                        st["beta_A"] = float(np.fmax(num / den, 0.0))
            st["dir_psi"] = st["beta_psi"] * st["dir_psi"] - jp
            if self.solveA:
                st["dir_A"] = st["beta_A"] * st["dir_A"] - jA
                c = self.coef_matrix(self.coef(st["dir_psi"], st["dir_A"]))
                a_psi, a_A = self.alpha_joint(c)
                self.psi = float(self.dtype(a_psi)) * st["dir_psi"] + self.psi
                self.ab = float(self.dtype(a_A)) * st["dir_A"] + self.ab
                st["jac_A_prev"] = jA.copy()
            else:
                c = self.coef_psi(st["dir_psi"])
                a = self.alpha_psi(c)
                self.psi = float(self.dtype(a)) * st["dir_psi"] + self.psi
            st["jac_psi_prev"] = jp.copy()
            E = self.free_energy()
            self.cg_energies.append(E)
            if i > 0 and np.abs(self.cg_energies[i] / self.cg_energies[i - 1] - 1.0) < self.convergence_rtol:
                break
        return self.cg_energies

    # vortex detector ------------------------------------------------------------
    def vortices(self, ai_bi=None):
        """``VortexDetector.vortices`` (``svirl/observables/vortex_detector.py:31-156``)."""
        return detect_vortices(self.g, self.psi, self.ab, self.H, ai_bi=ai_bi, dtype=self.dtype)


def winding_numbers(g, psi, ab, H, dtype=np.float64):
    """Per-cell vorticity v (``vortex_detector.py:55-67``), vectorised with the
    same elementwise NumPy operations.  Shape (Nxc, Nyc) indexed [i, j]."""
    P = unflatten_ij(np.asarray(psi), g.Nx, g.Ny)
    t = np.angle(P)
    a = np.reshape(ab[: g.Na], (g.Nya, g.Nxa)).T
    b = np.reshape(ab[g.Na:], (g.Nyb, g.Nxb)).T
    dx, dy = dtype(g.dx), dtype(g.dy)
    Hd = dtype(H)
    t00, tp0, tpp, t0p = t[:-1, :-1], t[1:, :-1], t[1:, 1:], t[:-1, 1:]
    v = -(0.5 / np.pi) * (
        np.mod(tp0 - t00 - dx * a[:, :-1] + np.pi, 2.0 * np.pi)
        + np.mod(tpp - tp0 - dy * b[1:, :] + np.pi, 2.0 * np.pi)
        + np.mod(t0p - tpp + dx * a[:, 1:] + np.pi, 2.0 * np.pi)
        + np.mod(t00 - t0p + dy * b[:-1, :] + np.pi, 2.0 * np.pi)
        - 4.0 * np.pi
        + dx * dy * Hd
    )
    return v


def triangulate(g, psi2, a_ai, b_bi, cells, dtype=np.float64):
    """Sub-cell vortex position for each (n, v) in ``cells``
    (``svirl/observables/vortex_detector.py:75-147``)."""
    dx, dy = dtype(g.dx), dtype(g.dy)

    def find_zero(x1, y1, f1, x2, y2, f2):
        return (f2 * x1 - x2 * f1) / (f2 - f1), (f2 * y1 - y2 * f1) / (f2 - f1)

    def find_zero_line(x1, y1, f1, x2, y2, f2, x3, y3, f3, x4, y4, f4):
        out = []
        if f2 * f1 < -1e-10: out.append(find_zero(x2, y2, f2, x1, y1, f1))
        if f3 * f2 < -1e-10: out.append(find_zero(x3, y3, f3, x2, y2, f2))
        if f4 * f3 < -1e-10: out.append(find_zero(x4, y4, f4, x3, y3, f3))
        if f1 * f4 < -1e-10: out.append(find_zero(x1, y1, f1, x4, y4, f4))
        return out

    def find_intersection(l1x1, l1y1, l1x2, l1y2, l2x1, l2y1, l2x2, l2y2):
        D = (l1x1 - l1x2) * (l2y1 - l2y2) - (l1y1 - l1y2) * (l2x1 - l2x2)
        ph = np.arctan2(D, (l1y1 - l1y2) * (l2y1 - l2y2) - (l1x1 - l1x2) * (l2x1 - l2x2))
        ph = np.mod(np.abs(ph), 0.5 * np.pi)
        if np.abs(ph) > 1e-10:
            ix = ((l1x1 * l1y2 - l1y1 * l1x2) * (l2x1 - l2x2) - (l1x1 - l1x2) * (l2x1 * l2y2 - l2y1 * l2x2)) / D
            iy = ((l1x1 * l1y2 - l1y1 * l1x2) * (l2y1 - l2y2) - (l1y1 - l1y2) * (l2x1 * l2y2 - l2y1 * l2x2)) / D
            return ix, iy, ph
        return np.nan, np.nan, ph

    found = []
    for n, v in cells:
        i, j = n % g.Nxc, n // g.Nxc
        ip, jp = i + 1, j + 1
        x, y = dx * i, dy * j
        inta_00 = dx * a_ai[i, j]
        inta_0p = dx * a_ai[i, jp]
        intb_00 = dy * b_bi[i, j]
        intb_p0 = dy * b_bi[ip, j]
        tpsi_00 = psi2[i, j]
        tpsi_p0 = psi2[ip, j] * np.exp(-1j * (0.75 * inta_00 + 0.25 * (intb_00 + inta_0p - intb_p0)))
        tpsi_pp = psi2[ip, jp] * np.exp(-1j * (0.5 * (inta_00 + intb_p0) + 0.5 * (intb_00 + inta_0p)))
        tpsi_0p = psi2[i, jp] * np.exp(-1j * (0.75 * intb_00 + 0.25 * (inta_00 + intb_p0 - inta_0p)))
        re_xy = find_zero_line(x, y, np.real(tpsi_00), x + dx, y, np.real(tpsi_p0),
                               x + dx, y + dy, np.real(tpsi_pp), x, y + dy, np.real(tpsi_0p))
        im_xy = find_zero_line(x, y, np.imag(tpsi_00), x + dx, y, np.imag(tpsi_p0),
                               x + dx, y + dy, np.imag(tpsi_pp), x, y + dy, np.imag(tpsi_0p))
        if len(re_xy) == 2 and len(im_xy) == 2:
            ix, iy, ph = find_intersection(re_xy[0][0], re_xy[0][1], re_xy[1][0], re_xy[1][1],
                                           im_xy[0][0], im_xy[0][1], im_xy[1][0], im_xy[1][1])
            if x - dx < ix < x + 2.0 * dx and y - dy < iy < y + 2.0 * dy:
                found.append([ix, iy, np.round(v)])
    if found:
        arr = np.array(found, dtype=dtype)
    else:
        arr = np.zeros((0, 3), dtype=dtype)
    return arr[:, 0], arr[:, 1], arr[:, 2]


def detect_vortices(g, psi, ab, H, ai_bi=None, dtype=np.float64):
    psi = np.asarray(psi).astype(np.complex64 if dtype is np.float32 else np.complex128)
    ab = np.asarray(ab).astype(dtype)
    v = winding_numbers(g, psi, ab, H, dtype)
    sel = (np.abs(v) > 0.5) & (np.abs(v - np.round(v)) < 0.1)
    ii, jj = np.nonzero(sel)
    n = ii + g.Nxc * jj
    order = np.argsort(n, kind="stable")
    cells = [(int(n[k]), v[ii[k], jj[k]]) for k in order]
    a = np.reshape(ab[: g.Na], (g.Nya, g.Nxa)).T
    b = np.reshape(ab[g.Na:], (g.Nyb, g.Nxb)).T
    if ai_bi is not None:
        a = a + ai_bi[0]
        b = b + ai_bi[1]
    psi2 = unflatten_ij(psi, g.Nx, g.Ny)
    return triangulate(g, psi2, a, b, cells, dtype)
