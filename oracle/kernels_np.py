"""CPU oracle: NumPy restatement of svirl's CUDA kernels for the 2D GL hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``svirl_gb300``) imports this
module; only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` use it, and only as the checker or as
the timed CPU baseline.

Every function restates one ``__global__`` kernel of the reference (file:line
given in each docstring, paths relative to the svirl project root).  Layouts are
the reference's flat layouts:

* order parameter ``psi``: complex, ``n = i + Nx*j`` (N = Nx*Ny nodes);
* vector potential ``ab``: real, ``[a | b]`` with ``a[i + Nxa*j]`` (Nxa = Nx-1,
  Nya = Ny) and ``b[Na + i + Nxb*j]`` (Nxb = Nx, Nyb = Ny-1);
* material tiling ``mt``: bool per cell ``i + Nxc*j`` (Nxc = Nx-1), ``None`` =
  the whole domain is superconducting.

Internally the arrays are viewed as C-order 2D arrays indexed ``[j, i]``.
Each kernel computes its whole output before it is stored, which reproduces the
reference's per-thread read-before-write semantics when argument buffers alias
(the A-sweep aliasing of ``svirl/solvers/td.py:380-419``).
"""

import numpy as np

BLOCK = 128  # the reference launches every kernel with 128-thread blocks (svirl/parallel/startup.py:65)


class Grid:
    """Geometry of one instance (``svirl/__init__.py:100-122``)."""

    def __init__(self, Nx, Ny, dx, dy):
        self.Nx, self.Ny = int(Nx), int(Ny)
        self.dx, self.dy = float(dx), float(dy)
        self.N = self.Nx * self.Ny
        self.Nxa, self.Nya = self.Nx - 1, self.Ny
        self.Nxb, self.Nyb = self.Nx, self.Ny - 1
        self.Na, self.Nb = self.Nxa * self.Nya, self.Nxb * self.Nyb
        self.Nab = self.Na + self.Nb
        self.Nxc, self.Nyc = self.Nx - 1, self.Ny - 1
        self.Nc = self.Nxc * self.Nyc
        self.idx, self.idy = 1.0 / self.dx, 1.0 / self.dy
        self.idx2, self.idy2 = 1.0 / (self.dx * self.dx), 1.0 / (self.dy * self.dy)
        self.idxy = 1.0 / (self.dx * self.dy)

    # 2D views ---------------------------------------------------------------
    def psi2(self, psi):
        return psi.reshape(self.Ny, self.Nx)

    def a2(self, ab):
        return ab[: self.Na].reshape(self.Nya, self.Nxa)

    def b2(self, ab):
        return ab[self.Na:].reshape(self.Nyb, self.Nxb)

    def mt2(self, mt):
        return None if mt is None else np.asarray(mt, dtype=bool).reshape(self.Nyc, self.Nxc)


def _cells_at_nodes(g, mt):
    """Per node (i, j): are the 4 adjacent cells inside the grid and in material.

    Restates the ``mt_mm/mt_mp/mt_pm/mt_pp`` block repeated in every kernel
    (e.g. ``svirl/cuda/td.h:129-138``).
    """
    Nx, Ny = g.Nx, g.Ny
    I = np.arange(Nx)[None, :]
    J = np.arange(Ny)[:, None]
    mm = (I > 0) & (J > 0)
    mp = (I > 0) & (J < Ny - 1)
    pm = (I < Nx - 1) & (J > 0)
    pp = (I < Nx - 1) & (J < Ny - 1)
    mm, mp, pm, pp = [np.broadcast_to(x, (Ny, Nx)).copy() for x in (mm, mp, pm, pp)]
    if mt is not None:
        m = np.zeros((Ny + 1, Nx + 1), dtype=bool)
        m[1:Ny, 1:Nx] = g.mt2(mt)
        mm &= m[0:Ny, 0:Nx]
        mp &= m[1:Ny + 1, 0:Nx]
        pm &= m[0:Ny, 1:Nx + 1]
        pp &= m[1:Ny + 1, 1:Nx + 1]
    return mm, mp, pm, pp


def _du_weights(mm, mp, pm, pp):
    """Du discretisation link weights (``svirl/cuda/observables.h:294-299``)."""
    f = lambda x: x.astype(np.float64)
    r_m0 = 0.5 * (f(mm) + f(mp))
    r_p0 = 0.5 * (f(pm) + f(pp))
    r_0m = 0.5 * (f(mm) + f(pm))
    r_0p = 0.5 * (f(mp) + f(pp))
    gw = 0.25 * (r_m0 + r_p0 + r_0m + r_0p)
    return r_m0, r_p0, r_0m, r_0p, gw


def U(ph):
    """Link factor exp(-i*ph) (``svirl/cuda/common.h:28-33``)."""
    return np.cos(ph) - 1j * np.sin(ph)


def js(psi0, ph, psi1):
    """Im(conj(psi0) U(ph) psi1) (``svirl/cuda/common.h:66-73``)."""
    x0, y0, x1, y1 = psi0.real, psi0.imag, psi1.real, psi1.imag
    return (x0 * y1 - y0 * x1) * np.cos(ph) - (x0 * x1 + y0 * y1) * np.sin(ph)


def g_grad(psi0, ph, psi1):
    """|psi1 U(ph) - psi0|^2 (``svirl/cuda/observables.h:238-247``)."""
    x1, y1 = psi1.real, psi1.imag
    c, s = np.cos(ph), np.sin(ph)
    re = x1 * c + y1 * s - psi0.real
    im = y1 * c - x1 * s - psi0.imag
    return re * re + im * im


def grad_c(psi0, ph, psi1):
    """psi1 U(ph) - psi0 (``svirl/cuda/cg.h:304-311``)."""
    x1, y1 = psi1.real, psi1.imag
    c, s = np.cos(ph), np.sin(ph)
    return (x1 * c + y1 * s) + 1j * (y1 * c - x1 * s) - psi0


def g_grad_jac_psi(psi0, ph, psi1):
    """2 (psi0 - psi1 U(ph)) (``svirl/cuda/cg.h:4-12``)."""
    x1, y1 = psi1.real, psi1.imag
    c, s = np.cos(ph), np.sin(ph)
    return 2.0 * (psi0 - ((x1 * c + y1 * s) + 1j * (y1 * c - x1 * s)))


# ---------------------------------------------------------------------------
# random numbers for the Langevin terms (svirl/cuda/common.h:36-63)
# ---------------------------------------------------------------------------

def rand_hash(s):
    """Thomas Wang 32-bit integer hash (``svirl/cuda/common.h:36-46``)."""
    s = np.asarray(s, dtype=np.uint32)
    with np.errstate(over="ignore"):
        s = (s ^ np.uint32(61)) ^ (s >> np.uint32(16))
        s = s * np.uint32(9)
        s = s ^ (s >> np.uint32(4))
        s = s * np.uint32(0x27D4EB2D)
        s = s ^ (s >> np.uint32(15))
    return s


def rand_1(n, t):
    with np.errstate(over="ignore"):
        m = np.uint32(71) * np.asarray(n, dtype=np.uint32) + np.uint32(9887) * np.uint32(t)
    return 2.0 ** -32 * rand_hash(m).astype(np.float64)


def rand_2(n, t):
    with np.errstate(over="ignore"):
        m = np.uint32(73) * np.asarray(n, dtype=np.uint32) + np.uint32(9901) * np.uint32(t) + np.uint32(1)
    return 2.0 ** -32 * rand_hash(m).astype(np.float64)


def residual_code(r, stop_eps):
    """int32(min(1e4*r/stop_eps, 1e8)) per element, NaN contributing 0.

    ``svirl/cuda/td.h:205-213``; CUDA's float->int conversion maps NaN to 0.
    """
    x = 1.0e4 * r / stop_eps
    x = np.where(np.isnan(x), 0.0, np.minimum(x, 1.0e8))
    return x.astype(np.int64)


# ---------------------------------------------------------------------------
# TDGL Jacobi sweeps
# ---------------------------------------------------------------------------

def iterate_order_parameter_jacobi_step(g, dt, epsilon, epsilon_spatial, mt, ab_abi,
                                        psi_rhs, psi, langevin_c, jstep, rand_t, stop_eps):
    """One Jacobi sweep of the backward-Euler psi step (``svirl/cuda/td.h:4-133``).

    Winecki-Adams link weights (``td.h:78-82``).  Returns ``(psi_next, r2_max)``
    where ``r2_max`` is the integer residual code the kernel ``atomicMax``es.
    ``psi_rhs`` is updated in place when the Langevin term is applied (sweep 0).
    """
    Nx, Ny = g.Nx, g.Ny
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    active = mm | mp | pm | pp
    r_m0 = (mm | mp)
    r_p0 = (pm | pp)
    r_0m = (mm | pm)
    r_0p = (mp | pp)

    P = g.psi2(psi)
    rhs = g.psi2(psi_rhs).copy()
    if jstep == 0 and langevin_c > 1.0e-32:
        n = np.arange(g.N, dtype=np.uint32).reshape(Ny, Nx)
        noise = langevin_c * ((rand_1(n, rand_t) - 0.5) + 1j * (rand_2(n, rand_t) - 0.5))
        rhs = np.where(active, rhs + noise, rhs)
        psi_rhs[:] = rhs.reshape(-1)

    if ab_abi is None:
        a = np.zeros((g.Nya, g.Nxa))
        b = np.zeros((g.Nyb, g.Nxb))
    else:
        a, b = g.a2(ab_abi), g.b2(ab_abi)
    t_m0 = np.zeros((Ny, Nx), complex)
    t_p0 = np.zeros((Ny, Nx), complex)
    t_0m = np.zeros((Ny, Nx), complex)
    t_0p = np.zeros((Ny, Nx), complex)
    t_m0[:, 1:] = U(-g.dx * a) * P[:, :-1]
    t_p0[:, :-1] = U(g.dx * a) * P[:, 1:]
    t_0m[1:, :] = U(-g.dy * b) * P[:-1, :]
    t_0p[:-1, :] = U(g.dy * b) * P[1:, :]
    t_m0 = np.where(r_m0, t_m0, 0.0)
    t_p0 = np.where(r_p0, t_p0, 0.0)
    t_0m = np.where(r_0m, t_0m, 0.0)
    t_0p = np.where(r_0p, t_0p, 0.0)

    eps = epsilon if epsilon_spatial is None else g.psi2(epsilon_spatial)
    f = lambda x: x.astype(np.float64)
    diag = 1.0 + dt * (rhs.real * rhs.real + rhs.imag * rhs.imag - eps
                       + 1.0 * (g.idx2 * (f(r_m0) + f(r_p0)) + g.idy2 * (f(r_0m) + f(r_0p))))
    with np.errstate(invalid="ignore", divide="ignore"):
        nxt = (rhs + dt * 1.0 * (g.idx2 * (t_m0 + t_p0) + g.idy2 * (t_0m + t_0p))) / diag
    nxt = np.where(active, nxt, 0.0)

    r = np.fmax(np.abs(nxt.real - P.real), np.abs(nxt.imag - P.imag))
    r2_max = int(residual_code(r, stop_eps).max())
    return nxt.reshape(-1), r2_max


def iterate_order_parameter_jacobi_step_cn(g, dt, epsilon, epsilon_spatial, mt, ab_abi,
                                           psi_rhs, psi, langevin_c, jstep, rand_t, stop_eps, as_written=False):
    """One Jacobi sweep of the Crank-Nicolson psi step of the reference's
    commented-out kernel (``svirl/cuda/td.h:136-292``, never launched by
    ``svirl/solvers/td.py``): c_lhs = c_rhs = 1/2, Du link weights
    (``td.h:209-212``) with ig = 4 / (sum of the four), the diagonal from
    |psi_rhs|^2, and the residual code from the SQUARED change
    ``1e4 (dre^2 + dim^2) / stop`` (``td.h:285-291``).  The explicit part of the
    links: from psi_rhs on all four (the trapezoidal rule the kernel's variable
    names describe), or with ``as_written`` from psi_rhs on the left x link only
    and from psi on the other three, as ``td.h:238-251`` writes it (which counts
    those neighbours twice: not a Crank-Nicolson step).  Returns
    ``(psi_next, r2_max)``; ``psi_rhs`` gets the Langevin term in sweep 0 as in the
    backward-Euler kernel."""
    Nx, Ny = g.Nx, g.Ny
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    active = mm | mp | pm | pp
    r_m0, r_p0, r_0m, r_0p, _ = _du_weights(mm, mp, pm, pp)
    P = g.psi2(psi)
    rhs = g.psi2(psi_rhs).copy()
    if jstep == 0 and langevin_c > 1.0e-32:
        n = np.arange(g.N, dtype=np.uint32).reshape(Ny, Nx)
        noise = langevin_c * ((rand_1(n, rand_t) - 0.5) + 1j * (rand_2(n, rand_t) - 0.5))
        rhs = np.where(active, rhs + noise, rhs)
        psi_rhs[:] = rhs.reshape(-1)
    a, b = (np.zeros((g.Nya, g.Nxa)), np.zeros((g.Nyb, g.Nxb))) if ab_abi is None else (g.a2(ab_abi), g.b2(ab_abi))
    z = lambda: np.zeros((Ny, Nx), complex)  # noqa: E731
    u_m0, u_p0, u_0m, u_0p = z(), z(), z(), z()
    u_m0[:, 1:] = U(-g.dx * a)
    u_p0[:, :-1] = U(g.dx * a)
    u_0m[1:, :] = U(-g.dy * b)
    u_0p[:-1, :] = U(g.dy * b)
    nb_m0, nb_p0, nb_0m, nb_0p = z(), z(), z(), z()   # psi at the four neighbours
    nr_m0, nr_p0, nr_0m, nr_0p = z(), z(), z(), z()   # the explicit part's neighbours
    Q = P if as_written else rhs
    nb_m0[:, 1:], nr_m0[:, 1:] = P[:, :-1], rhs[:, :-1]
    nb_p0[:, :-1], nr_p0[:, :-1] = P[:, 1:], Q[:, 1:]
    nb_0m[1:, :], nr_0m[1:, :] = P[:-1, :], Q[:-1, :]
    nb_0p[:-1, :], nr_0p[:-1, :] = P[1:, :], Q[1:, :]
    on_m0, on_p0, on_0m, on_0p = (mm | mp), (pm | pp), (mm | pm), (mp | pp)
    rU_m0 = np.where(on_m0, r_m0 * u_m0, 0.0)
    rU_p0 = np.where(on_p0, r_p0 * u_p0, 0.0)
    rU_0m = np.where(on_0m, r_0m * u_0m, 0.0)
    rU_0p = np.where(on_0p, r_0p * u_0p, 0.0)
    psi_m0, psi_p0, psi_0m, psi_0p = rU_m0 * nb_m0, rU_p0 * nb_p0, rU_0m * nb_0m, rU_0p * nb_0p
    rhs_m0, rhs_p0, rhs_0m, rhs_0p = rU_m0 * nr_m0, rU_p0 * nr_p0, rU_0m * nr_0m, rU_0p * nr_0p
    wsum = r_m0 + r_p0 + r_0m + r_0p
    with np.errstate(invalid="ignore", divide="ignore"):
        ig = np.where(active, 4.0 / np.where(wsum > 0, wsum, 1.0), 0.0)
        eps = epsilon if epsilon_spatial is None else g.psi2(epsilon_spatial)
        c_lhs = c_rhs = 0.5
        a2 = rhs.real * rhs.real + rhs.imag * rhs.imag
        lap_w = g.idx2 * (r_m0 + r_p0) + g.idy2 * (r_0m + r_0p)
        num = (rhs * (1.0 - c_rhs * dt * (a2 - eps))
               + c_rhs * dt * ig * (g.idx2 * (rhs_m0 + rhs_p0) + g.idy2 * (rhs_0m + rhs_0p) - lap_w * rhs)
               + c_lhs * dt * ig * (g.idx2 * (psi_m0 + psi_p0) + g.idy2 * (psi_0m + psi_0p)))
        den = 1.0 + c_lhs * dt * (a2 - eps + ig * lap_w)
        nxt = num / den
    nxt = np.where(active, nxt, 0.0)
    dre, dim = nxt.real - P.real, nxt.imag - P.imag
    r2 = dre * dre + dim * dim
    r2_max = int(residual_code(r2, stop_eps).max())
    return nxt.reshape(-1), r2_max


def order_parameter_phase_lock(psi, lock_ns):
    """psi[n] = |psi[n]| at phase-lock nodes (``svirl/cuda/td.h:295-307``)."""
    psi[lock_ns] = np.abs(psi[lock_ns])


def iterate_vector_potential_jacobi_step(g, dt, kappa2, rho, H, mt, psi, abi_ab_rhs, ab_rhs, ab,
                                         langevin_c, jstep, rand_t, stop_eps):
    """One Jacobi sweep of the A step (``svirl/cuda/td.h:310-463``).

    Returns ``(ab_next, r2_max)``; ``ab_rhs`` is updated in place when the
    Langevin term is applied (sweep 0).  ``abi_ab_rhs`` is read before any
    output is stored, as each reference thread reads its own link before it
    writes it.
    """
    Nx, Ny = g.Nx, g.Ny
    dt_rho = dt * rho
    dt_rho_kappa2 = dt_rho * kappa2
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    P = g.psi2(psi)
    ABI_a, ABI_b = g.a2(abi_ab_rhs).copy(), g.b2(abi_ab_rhs).copy()
    a, b = g.a2(ab), g.b2(ab)
    a_rhs, b_rhs = g.a2(ab_rhs).copy(), g.b2(ab_rhs).copy()

    if jstep == 0 and langevin_c > 1.0e-32:
        na = np.arange(g.Na, dtype=np.uint32).reshape(g.Nya, g.Nxa)
        nb = (g.Na + np.arange(g.Nb, dtype=np.uint32)).reshape(g.Nyb, g.Nxb)
        a_rhs = a_rhs + langevin_c * (rand_1(na, rand_t) - 0.5)
        b_rhs = b_rhs + langevin_c * (rand_2(nb, rand_t) - 0.5)
        ab_rhs[: g.Na] = a_rhs.reshape(-1)
        ab_rhs[g.Na:] = b_rhs.reshape(-1)

    # --- x links: a[j, i], i < Nx-1
    Ja = np.arange(g.Nya)[:, None]
    rh = np.where(Ja == 0, 2.0 * kappa2 * H * g.idy, np.where(Ja == g.Nya - 1, -2.0 * kappa2 * H * g.idy, 0.0))
    dd = np.where((Ja == 0) | (Ja == g.Nya - 1), 2.0, 1.0)
    lm = (pm | pp)[:, :Nx - 1]
    jl = np.where(lm, g.idx * js(P[:, :-1], g.dx * ABI_a, P[:, 1:]), 0.0)
    lo = np.zeros((g.Nya, g.Nxa))
    hi = np.zeros((g.Nya, g.Nxa))
    lo[1:, :] = g.idy2 * a[:-1, :] - g.idxy * b[:, :-1] + g.idxy * b[:, 1:]
    hi[:-1, :] = g.idy2 * a[1:, :] + g.idxy * b[:, :-1] - g.idxy * b[:, 1:]
    a_next = (a_rhs + dt_rho * (jl + rh) + dt_rho_kappa2 * dd * (lo + hi)) / (1.0 + 2.0 * dt_rho_kappa2 * g.idy2)
    ra = np.abs(a_next - a)

    # --- y links: b[j, i], j < Ny-1
    Ib = np.arange(g.Nxb)[None, :]
    rh = np.where(Ib == 0, -2.0 * kappa2 * H * g.idx, np.where(Ib == g.Nxb - 1, 2.0 * kappa2 * H * g.idx, 0.0))
    dd = np.where((Ib == 0) | (Ib == g.Nxb - 1), 2.0, 1.0)
    lm = (mp | pp)[:Ny - 1, :]
    jl = np.where(lm, g.idy * js(P[:-1, :], g.dy * ABI_b, P[1:, :]), 0.0)
    lo = np.zeros((g.Nyb, g.Nxb))
    hi = np.zeros((g.Nyb, g.Nxb))
    lo[:, 1:] = g.idx2 * b[:, :-1] - g.idxy * a[:-1, :] + g.idxy * a[1:, :]
    hi[:, :-1] = g.idx2 * b[:, 1:] + g.idxy * a[:-1, :] - g.idxy * a[1:, :]
    b_next = (b_rhs + dt_rho * (jl + rh) + dt_rho_kappa2 * dd * (lo + hi)) / (1.0 + 2.0 * dt_rho_kappa2 * g.idx2)
    rb = np.abs(b_next - b)

    r = max(residual_code(ra, stop_eps).max(initial=0), residual_code(rb, stop_eps).max(initial=0))
    return np.concatenate([a_next.reshape(-1), b_next.reshape(-1)]), int(r)


# ---------------------------------------------------------------------------
# observables (svirl/cuda/observables.h)
# ---------------------------------------------------------------------------

def _curl(g, ab):
    a, b = g.a2(ab), g.b2(ab)
    return g.idx * (b[:, 1:] - b[:, :-1]) - g.idy * (a[1:, :] - a[:-1, :])


def magnetic_field(g, abei, ab):
    """B = curl(A + A_ei) on cells (``svirl/cuda/observables.h:4-37``).  Shape (Nyc, Nxc)."""
    B = np.zeros((g.Nyc, g.Nxc))
    if abei is not None:
        B = B + _curl(g, abei)
    if ab is not None:
        B = B + _curl(g, ab)
    return B.reshape(-1)


def _curlcurl_parts(g, ab, self_scale_edge, nb_scale_edge):
    """The (bulk + boundary) curl-curl stencil shared by ``current_density`` and
    ``free_energy_jacobian_A`` with the reference's per-term boundary factors."""
    a, b = g.a2(ab), g.b2(ab)
    Ja = np.arange(g.Nya)[:, None]
    dd_a = np.where((Ja == 0) | (Ja == g.Nya - 1), 2.0, 1.0)
    ca = self_scale_edge(dd_a) * g.idy2 * a
    lo = np.zeros_like(a)
    hi = np.zeros_like(a)
    lo[1:, :] = -g.idy2 * a[:-1, :] + g.idxy * b[:, :-1] - g.idxy * b[:, 1:]
    hi[:-1, :] = -g.idy2 * a[1:, :] - g.idxy * b[:, :-1] + g.idxy * b[:, 1:]
    ca = ca + nb_scale_edge(dd_a) * lo + nb_scale_edge(dd_a) * hi

    Ib = np.arange(g.Nxb)[None, :]
    dd_b = np.where((Ib == 0) | (Ib == g.Nxb - 1), 2.0, 1.0)
    cb = self_scale_edge(dd_b) * g.idx2 * b
    lo = np.zeros_like(b)
    hi = np.zeros_like(b)
    lo[:, 1:] = -g.idx2 * b[:, :-1] + g.idxy * a[:-1, :] - g.idxy * a[1:, :]
    hi[:, :-1] = -g.idx2 * b[:, 1:] - g.idxy * a[:-1, :] + g.idxy * a[1:, :]
    cb = cb + nb_scale_edge(dd_b) * lo + nb_scale_edge(dd_b) * hi
    return ca, cb


def _boundary_H(g, H):
    Ja = np.arange(g.Nya)[:, None]
    ha = np.where(Ja == 0, -2.0 * H * g.idy, np.where(Ja == g.Nya - 1, 2.0 * H * g.idy, 0.0))
    Ib = np.arange(g.Nxb)[None, :]
    hb = np.where(Ib == 0, 2.0 * H * g.idx, np.where(Ib == g.Nxb - 1, -2.0 * H * g.idx, 0.0))
    return np.broadcast_to(ha, (g.Nya, g.Nxa)), np.broadcast_to(hb, (g.Nyb, g.Nxb))


def current_density(g, kappa2, H, abei, ab):
    """j = kappa^2 curl curl A with no-current boundaries (``svirl/cuda/observables.h:40-156``)."""
    ca, cb = _boundary_H(g, H)
    ca, cb = ca.copy(), cb.copy()
    if abei is not None:
        ea, eb = _curlcurl_parts(g, abei, lambda dd: 2.0 / dd, lambda dd: dd / dd)
        ca, cb = ca + ea, cb + eb
    if ab is not None:
        ea, eb = _curlcurl_parts(g, ab, lambda dd: 2.0, lambda dd: dd)
        ca, cb = ca + ea, cb + eb
    return np.concatenate([(kappa2 * ca).reshape(-1), (kappa2 * cb).reshape(-1)])


def _phase_sum(g, abei, ab):
    """abei + ab link phases, each term present only when its pointer is non-NULL."""
    out = np.zeros(g.Nab)
    if abei is not None:
        out = out + abei
    if ab is not None:
        out = out + ab
    return out


def supercurrent_density(g, mt, psi, abei, ab):
    """js = r d^-1 Im(conj(psi) U psi') on links, Du weights (``svirl/cuda/observables.h:159-235``)."""
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    P = g.psi2(psi)
    ph = _phase_sum(g, abei, ab)
    pa, pb = g.a2(ph), g.b2(ph)
    f = lambda x: x.astype(np.float64)
    lm = (pm | pp)[:, :-1]
    r_p0 = 0.5 * (f(pm) + f(pp))[:, :-1]
    ja = np.where(lm, r_p0 * g.idx * js(P[:, :-1], g.dx * pa, P[:, 1:]), 0.0)
    lm = (mp | pp)[:-1, :]
    r_0p = 0.5 * (f(mp) + f(pp))[:-1, :]
    jb = np.where(lm, r_0p * g.idy * js(P[:-1, :], g.dy * pb, P[1:, :]), 0.0)
    return np.concatenate([ja.reshape(-1), jb.reshape(-1)])


def free_energy_density(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
    """Per-node free-energy pseudo-density before the dx*dy factor
    (``svirl/cuda/observables.h:250-362``).  Shape (Ny, Nx)."""
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    active = mm | mp | pm | pp
    r_m0, r_p0, r_0m, r_0p, gw = _du_weights(mm, mp, pm, pp)
    P = g.psi2(psi)
    eps = epsilon if epsilon_spatial is None else g.psi2(epsilon_spatial)
    p2 = P.real * P.real + P.imag * P.imag
    e = gw * (0.5 * p2 - eps) * p2
    ph = _phase_sum(g, abei, ab)
    pa, pb = g.a2(ph), g.b2(ph)
    ex = np.zeros_like(e)
    ex[:, :-1] = r_p0[:, :-1] * g.idx2 * g_grad(P[:, :-1], g.dx * pa, P[:, 1:])
    ex = np.where(pm | pp, ex, 0.0)
    ey = np.zeros_like(e)
    ey[:-1, :] = r_0p[:-1, :] * g.idy2 * g_grad(P[:-1, :], g.dy * pb, P[1:, :])
    ey = np.where(mp | pp, ey, 0.0)
    e = np.where(active, e + ex + ey, 0.0)
    if kappa2 > 0.0:
        dB = np.full((g.Nyc, g.Nxc), -H)
        if abei is not None:
            dB = dB + _curl(g, abei)
        if ab is not None:
            dB = dB + _curl(g, ab)
        e[:-1, :-1] += kappa2 * dB * dB
    return e


def free_energy_pseudodensity(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
    """Per-128-block partial sums times dx*dy, as the kernel writes them."""
    e = free_energy_density(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab).reshape(-1)
    nb = (g.N + BLOCK - 1) // BLOCK
    pad = np.zeros(nb * BLOCK)
    pad[: g.N] = e
    return g.dx * g.dy * pad.reshape(nb, BLOCK).sum(axis=1)


def free_energy(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
    """Total GL free energy (``svirl/observables/observables.py:124-149``)."""
    return float(free_energy_pseudodensity(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab).sum())


# ---------------------------------------------------------------------------
# CG gradients and line-search coefficients (svirl/cuda/cg.h)
# ---------------------------------------------------------------------------

def free_energy_jacobian_psi(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
    """dF/d(Re psi) + i dF/d(Im psi), Du weights (``svirl/cuda/cg.h:15-121``)."""
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    active = mm | mp | pm | pp
    r_m0, r_p0, r_0m, r_0p, gw = _du_weights(mm, mp, pm, pp)
    P = g.psi2(psi)
    eps = epsilon if epsilon_spatial is None else g.psi2(epsilon_spatial)
    p = P.real * P.real + P.imag * P.imag - eps
    jac = 2.0 * gw * p * P
    ph = _phase_sum(g, abei, ab)
    pa, pb = g.a2(ph), g.b2(ph)
    t = np.zeros_like(jac)
    t[:, 1:] = r_m0[:, 1:] * g.idx2 * g_grad_jac_psi(P[:, 1:], -g.dx * pa, P[:, :-1])
    jac = jac + np.where(mm | mp, t, 0.0)
    t = np.zeros_like(jac)
    t[:, :-1] = r_p0[:, :-1] * g.idx2 * g_grad_jac_psi(P[:, :-1], g.dx * pa, P[:, 1:])
    jac = jac + np.where(pm | pp, t, 0.0)
    t = np.zeros_like(jac)
    t[1:, :] = r_0m[1:, :] * g.idy2 * g_grad_jac_psi(P[1:, :], -g.dy * pb, P[:-1, :])
    jac = jac + np.where(mm | pm, t, 0.0)
    t = np.zeros_like(jac)
    t[:-1, :] = r_0p[:-1, :] * g.idy2 * g_grad_jac_psi(P[:-1, :], g.dy * pb, P[1:, :])
    jac = jac + np.where(mp | pp, t, 0.0)
    jac = np.where(active, jac, 0.0)
    return (g.dx * g.dy * jac).reshape(-1)


def free_energy_jacobian_A(g, kappa2, H, mt, psi, abei, ab):
    """dF/dA on links (``svirl/cuda/cg.h:124-301``)."""
    ca, cb = _boundary_H(g, H)
    ca, cb = ca.copy(), cb.copy()
    if abei is not None:
        ea, eb = _curlcurl_parts(g, abei, lambda dd: 2.0 / dd, lambda dd: 1.0)
        ca, cb = ca + ea, cb + eb
    if ab is not None:
        ea, eb = _curlcurl_parts(g, ab, lambda dd: 2.0, lambda dd: dd)
        ca, cb = ca + ea, cb + eb
    ca, cb = kappa2 * ca, kappa2 * cb
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    P = g.psi2(psi)
    ph = _phase_sum(g, abei, ab)
    f = lambda x: x.astype(np.float64)
    lm = (pm | pp)[:, :-1]
    r_p0 = 0.5 * (f(pm) + f(pp))[:, :-1]
    ca = ca + np.where(lm, -r_p0 * g.idx * js(P[:, :-1], g.dx * g.a2(ph), P[:, 1:]), 0.0)
    lm = (mp | pp)[:-1, :]
    r_0p = 0.5 * (f(mp) + f(pp))[:-1, :]
    cb = cb + np.where(lm, -r_0p * g.idy * js(P[:-1, :], g.dy * g.b2(ph), P[1:, :]), 0.0)
    s = 2.0 * g.dx * g.dy
    return np.concatenate([(s * ca).reshape(-1), (s * cb).reshape(-1)])


def free_energy_jacobian_A_exact(g, kappa2, H, mt, psi, abei, ab):
    """The exact derivative of ``free_energy`` with respect to A.  Not in the
    reference: its dF/dA (``svirl/cuda/cg.h:124-301``, above) doubles the H and A
    terms of the magnetic part on the boundary links, which belong to one cell
    only.  Here the magnetic part is assembled cell by cell from
    d/dA kappa^2 dx dy (curl A - H)^2; the supercurrent part is the reference's."""
    r = -H * np.ones((g.Nyc, g.Nxc))
    if abei is not None:
        r = r + _curl(g, abei)
    if ab is not None:
        r = r + _curl(g, ab)
    ca = np.zeros((g.Nya, g.Nxa))
    cb = np.zeros((g.Nyb, g.Nxb))
    ca[:-1, :] += g.idy * r   # link a(i, j) is the lower edge of cell (i, j)
    ca[1:, :] -= g.idy * r    # ... and the upper edge of cell (i, j-1)
    cb[:, :-1] -= g.idx * r   # link b(i, j) is the left edge of cell (i, j)
    cb[:, 1:] += g.idx * r    # ... and the right edge of cell (i-1, j)
    ref = free_energy_jacobian_A(g, kappa2, H, mt, psi, abei, ab)
    mag_ref = free_energy_jacobian_A(g, kappa2, H, mt, np.zeros_like(psi), abei, ab)
    s = 2.0 * g.dx * g.dy
    return ref - mag_ref + s * kappa2 * np.concatenate([ca.reshape(-1), cb.reshape(-1)])


def _link_phase_scaled(g, abei, ab, d, which):
    """ph = d*abei + d*ab as accumulated by the coefficient kernels (``cg.h:410-412``)."""
    ph = 0.0
    pick = g.a2 if which == "a" else g.b2
    if abei is not None:
        ph = ph + d * pick(abei)
    if ab is not None:
        ph = ph + d * pick(ab)
    return ph


def free_energy_conjgrad_coef_psi_total(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, dpsi, abei, ab):
    """c0..c4 of F(psi + alpha dpsi) (``svirl/cuda/cg.h:314-474``), summed over the grid."""
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    active = mm | mp | pm | pp
    r_m0, r_p0, r_0m, r_0p, gw = _du_weights(mm, mp, pm, pp)
    P, D = g.psi2(psi), g.psi2(dpsi)
    eps = epsilon if epsilon_spatial is None else g.psi2(epsilon_spatial)
    p2 = P.real ** 2 + P.imag ** 2
    d2 = D.real ** 2 + D.imag ** 2
    tw = 2.0 * (P.real * D.real + P.imag * D.imag)
    c = np.zeros((5,) + P.shape)
    c[4] = gw * 0.5 * d2 * d2
    c[3] = gw * tw * d2
    c[2] = gw * (-eps * d2 + 0.5 * tw * tw + p2 * d2)
    c[1] = gw * tw * (p2 - eps)
    c[0] = gw * (0.5 * p2 - eps) * p2
    for which, sl0, sl1, r, msk, id2, d in (
        ("a", (slice(None), slice(None, -1)), (slice(None), slice(1, None)), r_p0, pm | pp, g.idx2, g.dx),
        ("b", (slice(None, -1), slice(None)), (slice(1, None), slice(None)), r_0p, mp | pp, g.idy2, g.dy),
    ):
        ph = _link_phase_scaled(g, abei, ab, d, which)
        p0, p1, d0, d1 = P[sl0], P[sl1], D[sl0], D[sl1]
        w = np.where(msk[sl0], r[sl0] * id2, 0.0)
        c[2][sl0] += w * g_grad(d0, ph, d1)
        z = np.conj(grad_c(p0, ph, p1)) * grad_c(d0, ph, d1)
        c[1][sl0] += w * 2.0 * z.real
        c[0][sl0] += w * g_grad(p0, ph, p1)
    c = np.where(active[None], c, 0.0)
    if kappa2 > 0.0:
        dB = _curl(g, ab) - H
        c[0][:-1, :-1] += kappa2 * dB * dB
    return g.dx * g.dy * c.reshape(5, -1).sum(axis=1)


def free_energy_conjgrad_coef_total(g, kappa2, epsilon, epsilon_spatial, H, mt, psi, dpsi, abei, ab, dab):
    """The 17 coefficients of F(psi + a_psi dpsi, A + a_A dA) (``svirl/cuda/cg.h:477-731``):
    exact quartic in a_psi, 4th-order Taylor in a_A.  Order c00..c04, c10..c14,
    c20..c24, c30, c40 (``cg.h:491-495``)."""
    mm, mp, pm, pp = _cells_at_nodes(g, mt)
    active = mm | mp | pm | pp
    r_m0, r_p0, r_0m, r_0p, gw = _du_weights(mm, mp, pm, pp)
    P, D = g.psi2(psi), g.psi2(dpsi)
    eps = epsilon if epsilon_spatial is None else g.psi2(epsilon_spatial)
    p2 = P.real ** 2 + P.imag ** 2
    d2 = D.real ** 2 + D.imag ** 2
    tw = 2.0 * (P.real * D.real + P.imag * D.imag)
    c = np.zeros((17,) + P.shape)
    c[0] = gw * (0.5 * p2 - eps) * p2
    c[5] = gw * tw * (p2 - eps)
    c[10] = gw * (-eps * d2 + 0.5 * tw * tw + p2 * d2)
    c[15] = gw * tw * d2
    c[16] = gw * 0.5 * d2 * d2
    for which, sl0, sl1, r, msk, id2, d in (
        ("a", (slice(None), slice(None, -1)), (slice(None), slice(1, None)), r_p0, pm | pp, g.idx2, g.dx),
        ("b", (slice(None, -1), slice(None)), (slice(1, None), slice(None)), r_0p, mp | pp, g.idy2, g.dy),
    ):
        ph = _link_phase_scaled(g, abei, ab, d, which)
        dph = d * (g.a2(dab) if which == "a" else g.b2(dab))
        dph2 = dph * dph
        p0, p1, d0, d1 = P[sl0], P[sl1], D[sl0], D[sl1]
        w = np.where(msk[sl0], r[sl0] * id2, 0.0)
        c[0][sl0] += w * g_grad(p0, ph, p1)
        z = np.conj(grad_c(p0, ph, p1)) * grad_c(d0, ph, d1)
        c[5][sl0] += w * 2.0 * z.real
        c[10][sl0] += w * g_grad(d0, ph, d1)
        Um = U(-ph)
        for base, z in ((1, p0 * Um * np.conj(p1)),
                        (6, p0 * Um * np.conj(d1) + d0 * Um * np.conj(p1)),
                        (11, d0 * Um * np.conj(d1))):
            c[base + 0][sl0] += w * 2.0 * z.imag * dph
            c[base + 1][sl0] += w * z.real * dph2
            c[base + 2][sl0] += -w / 3.0 * z.imag * dph2 * dph
            c[base + 3][sl0] += -w / 12.0 * z.real * dph2 * dph2
    c = np.where(active[None], c, 0.0)
    if kappa2 > 0.0:
        tot = _phase_sum(g, abei, ab)
        BH = _curl(g, tot) - H
        dB = _curl(g, dab)
        c[0][:-1, :-1] += kappa2 * BH * BH
        c[1][:-1, :-1] += kappa2 * 2.0 * BH * dB
        c[2][:-1, :-1] += kappa2 * dB * dB
    return g.dx * g.dy * c.reshape(17, -1).sum(axis=1)
