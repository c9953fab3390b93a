"""GLSolver: drop-in replacement of microsoft/svirl's 2D GL solver API on GB300.

The object graph and the public surface follow the reference
(``svirl/__init__.py:30-206``): ``gl.cfg``, ``gl.mesh``, ``gl.vars``,
``gl.params``, ``gl.observables``, ``gl.solve``, ``gl.vortex_detector`` and the
flatten helpers.  Unlike the reference there is no module-global config: each
GLSolver owns its parameters and one ``glgpu_handle`` (device-resident psi, A,
mask), so several solvers can live in one process.  All arithmetic on the
fields runs in libglgpu's sm_103a kernels; the host does what the reference's
host does (initial state, gauge set-up, line-search root finding, the vortex
detector's final predicate and triangulation on the GPU's candidate cells).
"""
import types

import numpy as np
import scipy.optimize

from . import _lib


def _dtypes(dtype):
    assert dtype in (np.float32, np.float64)
    return dtype, (np.complex64 if dtype is np.float32 else np.complex128)


def _flat(x):
    """(Nx, Ny)-shaped user array -> flat n = i + Nx*j (``svirl/storage/arrays.py:327-331``)."""
    return np.reshape(np.asarray(x).T, -1)


def _unflat(x, nx, ny):
    return np.reshape(x, (ny, nx)).T


class Mesh:
    """Grid coordinates and material tiling (``svirl/mesh/grid.py``)."""

    def __init__(self, gl, material_tiling):
        self._gl = gl
        self._mt = None
        self.material_tiling = material_tiling

    @property
    def _cfg(self):
        return self._gl.cfg

    def have_material_tiling(self):
        return self._mt is not None

    @property
    def xy(self):
        c = self._cfg
        return (np.linspace(0.0, c.Lx, num=c.Nx, endpoint=True, dtype=c.dtype),
                np.linspace(0.0, c.Ly, num=c.Ny, endpoint=True, dtype=c.dtype))

    @property
    def xy_grid(self):
        return np.meshgrid(*self.xy, indexing="ij")

    @property
    def xy_a(self):
        c = self._cfg
        return (np.linspace(0.5 * c.dx, c.Lx - 0.5 * c.dx, num=c.Nxa, endpoint=True, dtype=c.dtype),
                np.linspace(0.0, c.Ly, num=c.Nya, endpoint=True, dtype=c.dtype))

    @property
    def xy_a_grid(self):
        return np.meshgrid(*self.xy_a, indexing="ij")

    @property
    def xy_b(self):
        c = self._cfg
        return (np.linspace(0.0, c.Lx, num=c.Nxb, endpoint=True, dtype=c.dtype),
                np.linspace(0.5 * c.dy, c.Ly - 0.5 * c.dy, num=c.Nyb, endpoint=True, dtype=c.dtype))

    @property
    def xy_b_grid(self):
        return np.meshgrid(*self.xy_b, indexing="ij")

    @property
    def xy_c(self):
        c = self._cfg
        return (np.linspace(0.5 * c.dx, c.Lx - 0.5 * c.dx, num=c.Nxc, endpoint=True, dtype=c.dtype),
                np.linspace(0.5 * c.dy, c.Ly - 0.5 * c.dy, num=c.Nyc, endpoint=True, dtype=c.dtype))

    @property
    def xy_c_grid(self):
        return np.meshgrid(*self.xy_c, indexing="ij")

    @property
    def material_tiling(self):
        c = self._cfg
        if self._mt is not None:
            return self._mt.copy()
        return np.full((c.Nxc, c.Nyc), True, dtype=bool)

    @material_tiling.setter
    def material_tiling(self, material_tiling):
        c = self._cfg
        mt = material_tiling(*self.xy_c_grid) if callable(material_tiling) else material_tiling
        if mt is not None:
            mt = np.asarray(mt)
            assert mt.shape == (c.Nxc, c.Nyc)
            self._mt = mt.astype(bool)
            self._gl._h.set_mask(_flat(self._mt).astype(np.uint8))
        else:
            self._mt = None
            self._gl._h.set_mask(None)

    def _get_material_tiling_at_nodes(self):
        """OR of the (up to) 4 cells around each node (``svirl/mesh/grid.py:160-171``)."""
        c = self._cfg
        mt = self._mt
        out = np.zeros((c.Nx, c.Ny), dtype=bool)
        out[:-1, :-1] |= mt
        out[1:, :-1] |= mt
        out[:-1, 1:] |= mt
        out[1:, 1:] |= mt
        return out

    def interpolate_ab_array_to_c_array(self, a, b):
        return 0.5 * (a[:, :-1] + a[:, 1:]), 0.5 * (b[:-1, :] + b[1:, :])

    def interpolate_ab_array_to_c_array_abs(self, a, b):
        cx, cy = self.interpolate_ab_array_to_c_array(a, b)
        return np.sqrt(np.square(cx) + np.square(cy))


class Vars:
    """Order parameter and vector potential (``svirl/vars/vars.py``); device-resident."""

    def __init__(self, gl):
        self._gl = gl

    @property
    def _cfg(self):
        return self._gl.cfg

    @property
    def order_parameter(self):
        c = self._cfg
        return _unflat(self._gl._h.get_psi(), c.Nx, c.Ny).copy()

    @order_parameter.setter
    def order_parameter(self, order_parameter):
        c = self._cfg
        if isinstance(order_parameter, (np.complexfloating, complex, np.floating, float, np.integer, int)):
            order_parameter = c.dtype_complex(order_parameter) * np.ones((c.Nx, c.Ny), c.dtype_complex)
        order_parameter = np.asarray(order_parameter)
        assert order_parameter.shape == (c.Nx, c.Ny)
        psi = order_parameter.astype(c.dtype_complex)
        if self._gl.mesh.have_material_tiling():
            psi = psi.copy()
            psi[~self._gl.mesh._get_material_tiling_at_nodes()] = 0.0
        self._gl._h.set_psi(_flat(psi))

    def set_order_parameter_to_zero_outside_material(self):
        if not self._gl.mesh.have_material_tiling():
            return
        psi = self.order_parameter
        psi[~self._gl.mesh._get_material_tiling_at_nodes()] = 0.0
        self._gl._h.set_psi(_flat(psi))

    def randomize_order_parameter(self, level=1.0, seed=None):
        """|psi| *= 1 - level*rand, phase = level*pi*(2 rand - 1): legacy NumPy MT19937
        draws in the reference's order (``svirl/vars/vars.py:93-109``)."""
        assert 0.0 <= level <= 1.0
        c = self._cfg
        if seed is not None:
            np.random.seed(seed)
        data = (1.0 - level * np.random.rand(c.N)) * np.exp(level * 1.0j * np.pi * (2.0 * np.random.rand(c.N) - 1.0))
        self._gl._h.set_psi(data.astype(c.dtype_complex))

    @property
    def vector_potential(self):
        c = self._cfg
        ab = self._gl._h.get_ab()
        return (_unflat(ab[: c.Na], c.Nxa, c.Nya).copy(), _unflat(ab[c.Na:], c.Nxb, c.Nyb).copy())

    @vector_potential.setter
    def vector_potential(self, vector_potential):
        c = self._cfg
        a, b = vector_potential
        assert np.shape(a) == (c.Nxa, c.Nya) and np.shape(b) == (c.Nxb, c.Nyb)
        self._gl._h.set_ab(np.concatenate([_flat(a), _flat(b)]).astype(c.dtype))


class FixedVortices:
    """Fixed (pinned) vortices (``svirl/vars/fixed_vortices.py``): the irregular
    vector potential A_irr of phase windings around the given points, which the
    TDGL step adds to A (``svirl/solvers/td.py:120-154``) and the A step adds to
    the supercurrent argument (``td.py:252-325``), with the reference's element
    ranges; the phase lock (|psi| at the lock nodes after each psi step); the
    host-side phase winding of psi and the release of fixed vortices.  A_irr as
    set is kept here (``irregular_vector_potential``); the device copy the TD step
    works on changes during A loops, as the reference's does."""

    def __init__(self, gl):
        self._gl = gl
        c = gl.cfg
        self._ai = None  # A_irr as set: (a, b) or None
        corr = c.fixed_vortices_correction if c.fixed_vortices_correction is not None else "none"
        assert corr in ("none", "cell centers", "vertices")
        self.fixed_vortices_correction = corr
        self._phase_lock_radius = c.phase_lock_radius
        self.fixed_vortices_x = np.zeros(0, dtype=c.dtype)
        self.fixed_vortices_y = np.zeros(0, dtype=c.dtype)
        self.fixed_vortices_vorticity = np.zeros(0, dtype=c.dtype)
        self.fixed_vortices = c.fixed_vortices

    @staticmethod
    def _psi_abs(x, y):
        r2 = x ** 2 + y ** 2
        return (1.0 - np.exp(-r2)) / (1.0 + np.exp(-r2))

    def _vortices_format(self, vortices):
        c = self._gl.cfg
        if vortices is None:
            vortices = [[], []]
        if isinstance(vortices, dict):
            vx, vy = vortices["x"], vortices["y"]
            vv = vortices.get("vorticity", [])
        else:
            vx, vy = vortices[0], vortices[1]
            vv = vortices[2] if len(vortices) == 3 else []
        vx, vy, vv = [np.array([] if v is None else v).flatten() for v in (vx, vy, vv)]
        vN = max(vx.size, vy.size, vv.size)
        if vx.size > 0 and vv.size == 0:
            vv = np.array([1])
        assert vx.size in (1, vN) and vy.size in (1, vN) and vv.size in (1, vN)
        fvx, fvy, fvv = [], [], []
        x = y = v = np.nan
        for i in range(vN):
            if i < vx.size: x = vx[i]
            if i < vy.size: y = vy[i]
            if i < vv.size: v = vv[i]
            if np.isnan(x) or np.isnan(y) or np.isnan(v):
                continue
            fvx.append(x); fvy.append(y); fvv.append(v)
        return (np.array(fvx).astype(c.dtype), np.array(fvy).astype(c.dtype), np.array(fvv).astype(c.dtype))

    def _correct(self):
        """Integer vorticity; positions moved to cell centres or vertices
        (``fixed_vortices.py:113-126``)."""
        c = self._gl.cfg
        self.fixed_vortices_vorticity = np.round(self.fixed_vortices_vorticity)
        if self.fixed_vortices_correction == "cell centers":
            self.fixed_vortices_x = c.dx * (np.round(self.fixed_vortices_x / c.dx + 0.5) - 0.5)
            self.fixed_vortices_y = c.dy * (np.round(self.fixed_vortices_y / c.dy + 0.5) - 0.5)
        elif self.fixed_vortices_correction == "vertices":
            self.fixed_vortices_x = c.dx * np.round(self.fixed_vortices_x / c.dx)
            self.fixed_vortices_y = c.dy * np.round(self.fixed_vortices_y / c.dy)

    def order_parameter_add_vortices(self, vortices, phase=True, deep=False):
        """Adds phase windings (and optionally |psi| dips) around the given points."""
        vx, vy, vv = self._vortices_format(vortices)
        xg, yg = self._gl.mesh.xy_grid
        psi = self._gl.vars.order_parameter
        for k in range(vx.size):
            if phase:
                psi *= np.exp(1.0j * vv[k] * np.arctan2(yg - vy[k], xg - vx[k]))
            if deep:
                psi *= np.power(self._psi_abs(xg - vx[k], yg - vy[k]), np.abs(vv[k]))
        self._gl._h.set_psi(_flat(psi.astype(self._gl.cfg.dtype_complex)))

    @property
    def irregular_vector_potential(self):
        c = self._gl.cfg
        if self._ai is None:
            return np.zeros((c.Nxa, c.Nya), dtype=c.dtype), np.zeros((c.Nxb, c.Nyb), dtype=c.dtype)
        return self._ai[0].copy(), self._ai[1].copy()

    def _ab_phase(self, a, b):
        """Phase whose link differences are (a, b), zero at node (0, 0)."""
        c = self._gl.cfg
        a = c.dx * np.r_[np.zeros((1, c.Nya), dtype=c.dtype), a].cumsum(axis=0)
        b = c.dy * np.c_[np.zeros((c.Nxb, 1), dtype=c.dtype), b].cumsum(axis=1)
        return np.repeat(b[0:1, :], c.Nx, axis=0) + a

    @property
    def fixed_vortices_phase(self):
        return self._ab_phase(*self.irregular_vector_potential)

    def fixed_vortices_release(self):
        """Turns the fixed vortices into free ones: their phase goes into psi, then
        A_irr and the phase lock are removed (``fixed_vortices.py:60-73``)."""
        psi = self._gl.vars.order_parameter
        psi *= np.exp(-1.0j * self.fixed_vortices_phase)
        self._gl._h.set_psi(_flat(psi.astype(self._gl.cfg.dtype_complex)))
        self.fixed_vortices = None
        self.phase_lock_radius = None

    @property
    def fixed_vortices(self):
        return self.fixed_vortices_x.copy(), self.fixed_vortices_y.copy(), self.fixed_vortices_vorticity.copy()

    @fixed_vortices.setter
    def fixed_vortices(self, fixed_vortices):
        c = self._gl.cfg
        self.fixed_vortices_x, self.fixed_vortices_y, self.fixed_vortices_vorticity = self._vortices_format(fixed_vortices)
        self._correct()
        if self.fixed_vortices_x.size > 0:
            ai = np.zeros((c.Nxa, c.Nya), dtype=c.dtype)
            bi = np.zeros((c.Nxb, c.Nyb), dtype=c.dtype)
            xg, yg = self._gl.mesh.xy_grid
            for k in range(self.fixed_vortices_x.size):
                # winding angle around the vortex, zero at node (0, 0); its link differences
                ang = np.arctan2(yg - self.fixed_vortices_y[k], xg - self.fixed_vortices_x[k])
                ang -= ang[0, 0]
                ai += self.fixed_vortices_vorticity[k] * c.idx * np.diff(ang, axis=0)
                bi += self.fixed_vortices_vorticity[k] * c.idy * np.diff(ang, axis=1)
            self._ai = (ai, bi)
            self._gl._h.set_irregular_vector_potential(np.concatenate([_flat(ai), _flat(bi)]))
        else:
            self._ai = None
            self._gl._h.set_irregular_vector_potential(None)
        self._update_phase_lock()

    @property
    def phase_lock_radius(self):
        return self._phase_lock_radius

    @phase_lock_radius.setter
    def phase_lock_radius(self, radius):
        assert radius is None or (isinstance(radius, (np.floating, float, np.integer, int)) and radius > 0.0)
        self._phase_lock_radius = radius
        self._update_phase_lock()

    def _update_phase_lock(self):
        """Nodes within the lock radius of a fixed vortex.  The reference takes
        ``np.where(lock_grid)[0]`` of the (Nx, Ny) grid, the x index of each locked
        node, as the flat node index (``fixed_vortices.py:218-236``); kept."""
        c = self._gl.cfg
        ns = None
        if self._phase_lock_radius is not None:
            xg, yg = self._gl.mesh.xy_grid
            lock = np.zeros((c.Nx, c.Ny), dtype=bool)
            for k in range(self.fixed_vortices_x.size):
                lock |= (np.square(xg - self.fixed_vortices_x[k]) + np.square(yg - self.fixed_vortices_y[k])
                         <= np.square(self._phase_lock_radius))
            ns = np.where(lock)[0].astype(np.int32)
        self._gl._h.set_phase_lock(ns if ns is not None and ns.size > 0 else None)

    @property
    def vortices(self):
        """Alias of ``gl.vortex_detector.vortices`` (the name used in the reference's README)."""
        return self._gl.vortex_detector.vortices


class Params:
    """Model parameters (``svirl/vars/params.py``)."""

    def __init__(self, gl, cfg):
        self._gl = gl
        self.fixed_vortices = FixedVortices(gl)
        self._epsilon = None
        self.linear_coefficient = cfg.linear_coefficient
        self.gl_parameter = cfg.gl_parameter
        self.normal_conductivity = cfg.normal_conductivity
        self._H = cfg.dtype(0.0)
        self.homogeneous_external_field_reset = cfg.homogeneous_external_field
        self.ae, self.be = None, None
        self._vpei = None
        self.external_field = cfg.external_field
        self.order_parameter_Langevin_coefficient = cfg.order_parameter_Langevin_coefficient
        self.vector_potential_Langevin_coefficient = cfg.vector_potential_Langevin_coefficient

    @property
    def _cfg(self):
        return self._gl.cfg

    def _push(self, **kw):
        self._gl._h.set_params(**kw)

    # epsilon ------------------------------------------------------------------
    @property
    def linear_coefficient(self):
        c = self._cfg
        if np.ndim(self._epsilon) == 0:
            return np.full((c.Nx, c.Ny), self._epsilon, dtype=c.dtype)
        return self._epsilon.copy()

    @linear_coefficient.setter
    def linear_coefficient(self, linear_coefficient):
        c = self._cfg
        lc = linear_coefficient(*self._gl.mesh.xy_grid) if callable(linear_coefficient) else linear_coefficient
        if np.isscalar(lc):
            self._epsilon = c.dtype(lc)
            self._gl._h.set_eps_field(None)
            self._push(epsilon=float(self._epsilon))
        else:
            lc = np.asarray(lc)
            assert lc.shape == (c.Nx, c.Ny)
            self._epsilon = lc.astype(c.dtype)
            self._gl._h.set_eps_field(_flat(self._epsilon))
            self._push(epsilon=0.0)

    # kappa ---------------------------------------------------------------------
    @property
    def gl_parameter(self):
        return self._kappa

    @gl_parameter.setter
    def gl_parameter(self, gl_parameter):
        if gl_parameter is None or np.isnan(gl_parameter) or np.isinf(gl_parameter):
            gl_parameter = np.inf
        assert isinstance(gl_parameter, (np.floating, float, np.integer, int)) and (np.isposinf(gl_parameter) or gl_parameter > 0.0)
        self._kappa = self._cfg.dtype(gl_parameter)
        self._push(kappa=float("inf") if np.isposinf(self._kappa) else float(self._kappa))

    @property
    def solveA(self):
        return bool(not np.isposinf(self._kappa))

    def gl_parameter_squared_h(self):
        return self._cfg.dtype(self._kappa ** 2) if self.solveA else self._cfg.dtype(-1.0)

    # sigma ---------------------------------------------------------------------
    @property
    def normal_conductivity(self):
        return self._sigma

    @normal_conductivity.setter
    def normal_conductivity(self, normal_conductivity):
        assert isinstance(normal_conductivity, (np.floating, float, np.integer, int)) and normal_conductivity > 0.0
        self._sigma = self._cfg.dtype(normal_conductivity)
        self._rho = self._cfg.dtype(1.0 / normal_conductivity)
        self._push(sigma=float(normal_conductivity))

    # H -------------------------------------------------------------------------
    @property
    def homogeneous_external_field(self):
        return self._H

    @homogeneous_external_field.setter
    def homogeneous_external_field(self, homogeneous_external_field):
        self._H = self._cfg.dtype(homogeneous_external_field)
        self._push(H=float(self._H))

    def _update_vector_potential(self, homogeneous_external_field, reset):
        """Symmetric gauge A = (-g y H, (1-g) x H), g = 1/2, about the domain centre
        (``svirl/vars/params.py:135-170``)."""
        c = self._cfg
        assert isinstance(homogeneous_external_field, (np.floating, float, np.integer, int))
        if reset:
            self._H = c.dtype(homogeneous_external_field)
            a = np.zeros((c.Nxa, c.Nya), dtype=c.dtype)
            b = np.zeros((c.Nxb, c.Nyb), dtype=c.dtype)
            delta_H = self._H
        else:
            delta_H = -self._H
            self._H = c.dtype(homogeneous_external_field)
            delta_H += self._H
            a, b = self._gl.vars.vector_potential
        g = 0.5
        _, yg = self._gl.mesh.xy_a_grid
        xg, _ = self._gl.mesh.xy_b_grid
        a -= g * (yg - 0.5 * c.Ly) * delta_H
        b += (1.0 - g) * (xg - 0.5 * c.Lx) * delta_H
        self._gl.vars.vector_potential = (a, b)
        self._push(H=float(self._H))

    homogeneous_external_field_delta = property(
        fset=lambda self, H: self._update_vector_potential(H, reset=False),
        doc="Sets H and adds the gauge field of H - H_old to A.")
    homogeneous_external_field_reset = property(
        fset=lambda self, H: self._update_vector_potential(H, reset=True),
        doc="Sets H and resets A to the gauge field of H.")

    # external vector potential ------------------------------------------------------
    def _update_gvpei(self):
        """The external + irregular vector potential the energy, currents and CG
        use: A_ext + A_irr of the fixed vortices at this moment (``params.py:193-222``;
        like the reference, setting fixed vortices later does not update it)."""
        ai = self.fixed_vortices._ai
        if self.ae is None and ai is None:
            self._vpei = None
            self._gl._h.set_abei(None)
            return
        if self.ae is None:
            self._vpei = ai
        elif ai is None:
            self._vpei = (self.ae, self.be)
        else:
            self._vpei = (self.ae + ai[0], self.be + ai[1])
        flat = np.concatenate([_flat(self._vpei[0]), _flat(self._vpei[1])]).astype(self._cfg.dtype)
        # an all-zero external potential adds exact zeros: leave it out of the kernels
        self._gl._h.set_abei(None if not np.any(flat) else flat)

    @property
    def external_vector_potential(self):
        return None if self.ae is None else (self.ae, self.be)

    @external_vector_potential.setter
    def external_vector_potential(self, external_vector_potential):
        c = self._cfg
        Ax = Ay = None
        if external_vector_potential is not None:
            Ax, Ay = external_vector_potential
        if Ax is not None:
            assert np.shape(Ax) == (c.Nxa, c.Nya) and np.shape(Ay) == (c.Nxb, c.Nyb)
            self.ae, self.be = np.asarray(Ax), np.asarray(Ay)
        else:
            self.ae, self.be = None, None
        self._update_gvpei()

    @property
    def external_irregular_vector_potential(self):
        return self._vpei

    @property
    def external_field(self):
        A = self.external_vector_potential
        if A is None:
            return None
        Ax, Ay = A
        return -np.diff(Ax, axis=1) * self._cfg.idy + np.diff(Ay, axis=0) * self._cfg.idx

    @external_field.setter
    def external_field(self, external_field):
        c = self._cfg
        if external_field is not None:
            g = 0.5
            _, yg = self._gl.mesh.xy_a_grid
            xg, _ = self._gl.mesh.xy_b_grid
            Ax = -g * (yg - 0.5 * c.Ly) * external_field
            Ay = (1.0 - g) * (xg - 0.5 * c.Lx) * external_field
            self.external_vector_potential = (Ax, Ay)
        else:
            self.external_vector_potential = None

    # Langevin --------------------------------------------------------------------
    @property
    def order_parameter_Langevin_coefficient(self):
        return self._psi_langevin_c

    @order_parameter_Langevin_coefficient.setter
    def order_parameter_Langevin_coefficient(self, v):
        assert isinstance(v, (np.floating, float, np.integer, int))
        self._psi_langevin_c = self._cfg.dtype(v)
        self._push(langevin_psi=float(self._psi_langevin_c))

    @property
    def vector_potential_Langevin_coefficient(self):
        return self._ab_langevin_c

    @vector_potential_Langevin_coefficient.setter
    def vector_potential_Langevin_coefficient(self, v):
        assert isinstance(v, (np.floating, float, np.integer, int))
        self._ab_langevin_c = self._cfg.dtype(v)
        self._push(langevin_A=float(self._ab_langevin_c))


class _HostArray:
    """Result holder with the ``.get()`` accessor the reference's tests call on
    gpuarrays (``tests/at_cg_jacobians.py:104,152``)."""

    def __init__(self, a):
        self._a = a

    def get(self):
        return self._a.copy()


class Observables:
    """``svirl/observables/observables.py``."""

    def __init__(self, gl):
        self._gl = gl

    @property
    def superfluid_density(self):
        psi = self._gl.vars.order_parameter
        return np.square(psi.real) + np.square(psi.imag)

    @property
    def magnetic_field(self):
        c = self._gl.cfg
        return _unflat(self._gl._h.magnetic_field(), c.Nxc, c.Nyc).copy()

    def _links(self, flat):
        c = self._gl.cfg
        return _unflat(flat[: c.Na], c.Nxa, c.Nya).copy(), _unflat(flat[c.Na:], c.Nxb, c.Nyb).copy()

    @property
    def supercurrent_density(self):
        return self._links(self._gl._h.supercurrent_density())

    @property
    def current_density(self):
        return self._links(self._gl._h.current_density())

    @property
    def normalcurrent_density(self):
        jx, jy = self.current_density
        jsx, jsy = self.supercurrent_density
        return jx - jsx, jy - jsy

    @property
    def free_energy(self):
        return self._gl._h.free_energy()


class VortexDetector:
    """Plaquette phase-winding vortex detector (``svirl/observables/vortex_detector.py``).

    The GPU scans every cell and returns the cells whose winding passes a relaxed
    test together with their corner values; the reference's exact predicate and
    sub-cell triangulation are then applied to those cells here, with the same
    NumPy operations in the solver's dtype, so the result equals the reference's
    for the same order parameter."""

    def __init__(self, gl):
        self._gl = gl
        self._detected_vortices = np.zeros((0, 3))

    @property
    def vortices(self):
        gl = self._gl
        c = gl.cfg
        if gl.solve.vortices_detected is not True:
            cells, corners = gl._h.vortex_candidates()
            ctype = c.dtype_complex
            p = corners[:, 0:8].astype(c.dtype).reshape(-1, 4, 2)
            psi = (p[..., 0] + 1j * p[..., 1]).astype(ctype)
            t = np.angle(psi)
            a00, a0p, b00, bp0 = (corners[:, k].astype(c.dtype) for k in (8, 9, 10, 11))
            t00, tp0, tpp, t0p = t[:, 0], t[:, 1], t[:, 2], t[:, 3]
            H = gl.params.homogeneous_external_field
            v = -(0.5 / np.pi) * (
                np.mod(tp0 - t00 - c.dx * a00 + np.pi, 2.0 * np.pi)
                + np.mod(tpp - tp0 - c.dy * bp0 + np.pi, 2.0 * np.pi)
                + np.mod(t0p - tpp + c.dx * a0p + np.pi, 2.0 * np.pi)
                + np.mod(t00 - t0p + c.dy * b00 + np.pi, 2.0 * np.pi)
                - 4.0 * np.pi
                + c.dx * c.dy * H)
            sel = (np.abs(v) > 0.5) & (np.abs(v - np.round(v)) < 0.1)
            ai = gl.params.fixed_vortices._ai
            if ai is not None:
                # the triangulation reads A + A_irr (host copy, as set), the winding A alone
                # (vortex_detector.py:43-50,55-72)
                ci, cj = cells % c.Nxc, cells // c.Nxc
                a00 = a00 + ai[0][ci, cj]
                a0p = a0p + ai[0][ci, cj + 1]
                b00 = b00 + ai[1][ci, cj]
                bp0 = bp0 + ai[1][ci + 1, cj]
            found = []
            for k in np.nonzero(sel)[0]:
                r = _triangulate(c, int(cells[k]), v[k], psi[k], a00[k], a0p[k], b00[k], bp0[k])
                if r is not None:
                    found.append(r)
            self._detected_vortices = (np.array(found, dtype=c.dtype) if found
                                       else np.zeros((0, 3), dtype=c.dtype))
            gl.solve.vortices_detected = True
        d = self._detected_vortices
        return d[:, 0], d[:, 1], d[:, 2]


def _triangulate(c, n, v, psi4, a00, a0p, b00, bp0):
    """Sub-cell vortex position from the zero lines of Re psi and Im psi after
    gauge transport to the cell corner (``svirl/observables/vortex_detector.py:75-147``)."""
    i, j = n % c.Nxc, n // c.Nxc
    x, y = c.dx * i, c.dy * j
    inta_00, inta_0p = c.dx * a00, c.dx * a0p
    intb_00, intb_p0 = c.dy * b00, c.dy * bp0
    t00 = psi4[0]
    tp0 = psi4[1] * np.exp(-1j * (0.75 * inta_00 + 0.25 * (intb_00 + inta_0p - intb_p0)))
    tpp = psi4[2] * np.exp(-1j * (0.5 * (inta_00 + intb_p0) + 0.5 * (intb_00 + inta_0p)))
    t0p = psi4[3] * np.exp(-1j * (0.75 * intb_00 + 0.25 * (inta_00 + intb_p0 - inta_0p)))
    X = (x, x + c.dx, x + c.dx, x)
    Y = (y, y, y + c.dy, y + c.dy)

    def zeros_on_border(f):
        # linear zero between corners (a, b), walking the border 00 -> p0 -> pp -> 0p
        out = []
        for (a, b) in ((1, 0), (2, 1), (3, 2), (0, 3)):
            if f[a] * f[b] < -1e-10:
                out.append(((f[b] * X[a] - X[b] * f[a]) / (f[b] - f[a]),
                            (f[b] * Y[a] - Y[b] * f[a]) / (f[b] - f[a])))
        return out

    vals = (t00, tp0, tpp, t0p)
    re_xy = zeros_on_border([np.real(q) for q in vals])
    im_xy = zeros_on_border([np.imag(q) for q in vals])
    if len(re_xy) != 2 or len(im_xy) != 2:
        return None
    (l1x1, l1y1), (l1x2, l1y2) = re_xy
    (l2x1, l2y1), (l2x2, l2y2) = im_xy
    D = (l1x1 - l1x2) * (l2y1 - l2y2) - (l1y1 - l1y2) * (l2x1 - l2x2)
    ph = np.arctan2(D, (l1y1 - l1y2) * (l2y1 - l2y2) - (l1x1 - l1x2) * (l2x1 - l2x2))
    ph = np.mod(np.abs(ph), 0.5 * np.pi)
    if not np.abs(ph) > 1e-10:
        return None
    ix = ((l1x1 * l1y2 - l1y1 * l1x2) * (l2x1 - l2x2) - (l1x1 - l1x2) * (l2x1 * l2y2 - l2y1 * l2x2)) / D
    iy = ((l1x1 * l1y2 - l1y1 * l1x2) * (l2y1 - l2y2) - (l1y1 - l1y2) * (l2x1 * l2y2 - l2y1 * l2x2)) / D
    if x - c.dx < ix < x + 2.0 * c.dx and y - c.dy < iy < y + 2.0 * c.dy:
        return [ix, iy, np.round(v)]
    return None


class TD:
    """TDGL driver (``svirl/solvers/td.py``): the time loop and the Jacobi loops
    run on the device in one CUDA-graph launch per call."""

    SCHEMES = ("backward_euler", "crank_nicolson", "crank_nicolson_as_written")

    def __init__(self, gl):
        self._gl = gl
        self.dt = self.Nt = self.T = None
        self.dtA = self.NtA = self.TA = None
        self.last_stats = None
        self._scheme = "backward_euler"

    @property
    def scheme(self):
        """Time stepping of the order parameter: "backward_euler" (the reference's,
        the default), "crank_nicolson" (the reference's commented-out sweep,
        svirl/cuda/td.h:136-292, with the explicit half of every link from the
        step's start) or "crank_nicolson_as_written" (that sweep as written), with
        the same Jacobi loop and stop rule."""
        return self._scheme

    @scheme.setter
    def scheme(self, value):
        if value not in self.SCHEMES:
            raise ValueError("scheme must be one of %s" % (self.SCHEMES,))
        self._gl._h.set_psi_scheme(self.SCHEMES.index(value))
        self._scheme = value

    @property
    def _random_t(self):
        return np.uint32(self._gl._h.get_params().rand_t)

    def _set_iterator_options(self, iterator_type, Nt=None, dt=None, T=None):
        c = self._gl.cfg
        if Nt is not None and T is not None and dt is None:
            dt = float(T) / Nt
        elif Nt is not None and T is None and dt is not None:
            T = float(dt) * Nt
        elif Nt is None and T is not None and dt is not None:
            Nt = int(np.round(T / dt))
        elif Nt is not None and T is not None and dt is not None:
            assert np.isclose(T, dt * Nt)
        assert isinstance(dt, (np.floating, float, np.integer, int)) and dt >= 0.0
        assert isinstance(Nt, (np.integer, int)) and Nt >= 0
        if iterator_type == "order_parameter":
            self.Nt, self.dt, self.T = np.int32(Nt), c.dtype(dt), c.dtype(T)
        else:
            self.NtA, self.dtA, self.TA = np.int32(Nt), c.dtype(dt), c.dtype(T)

    def _warn(self):
        c, p = self._gl.cfg, self._gl.params
        if self.dt is not None and self.dt / min(c.dx, c.dy) ** 2 > 1.0:
            print("Warning (order parameter):  dt/min(dx,dy)^2 = %g is too large" % (self.dt / min(c.dx, c.dy) ** 2))
        if p.solveA and self.dtA is not None:
            d = self.dtA * p.gl_parameter ** 2 / (p.normal_conductivity * min(c.dx, c.dy) ** 2)
            if d > 1.0:
                print("Warning (vector potential):  dt*kappa^2/(sigma*min(dx,dy)^2) = %g is too large" % d)
            d = self.dtA / (p.normal_conductivity * min(c.dx, c.dy))
            if d > 1.0:
                print("Warning (vector potential):  dt/(sigma*min(dx,dy)) = %g is too large" % d)

    def _solve(self, dt=None, Nt=None, T=None, eqn=None):
        h = self._gl._h
        if eqn == "order_parameter":
            self._set_iterator_options("order_parameter", Nt, dt, T)
            self._warn()
            self.last_stats = h.td(self.dt, self.Nt, 1)
        elif eqn == "vector_potential":
            if not self._gl.params.solveA:
                return
            self._set_iterator_options("vector_potential", Nt, dt, T)
            if self.dt is None:
                # the reference's A kernel receives TD.dt, unset before any psi step (td.py:278)
                raise TypeError("vector-potential steps use the order-parameter dt, which is not set yet")
            self._warn()
            self.last_stats = h.td(self.dt, self.NtA, 2)
        else:
            self._set_iterator_options("order_parameter", Nt, dt, T)
            self._set_iterator_options("vector_potential", Nt, dt, T)
            self._warn()
            self.last_stats = h.td(self.dt, self.Nt, 0)


class CG:
    """Modified nonlinear CG (``svirl/solvers/cg.py``).  Gradients, direction
    updates, line-search coefficients (5 or 17, FP64 sums), updates and the
    energy run on the GPU; the step length is chosen on the host from the
    coefficients with the reference's own root finder (kappa = inf: NumPy
    ``polyroots``) or 2-D BFGS (finite kappa: ``scipy.optimize.minimize``), so
    the iteration makes the reference's decisions."""

    def __init__(self, gl):
        self._gl = gl
        self._convergence_rtol = gl.cfg.convergence_rtol
        self.cg_energies = []
        self._c = None

    @property
    def _free_energy_jacobian_psi(self):
        gp, _ = self._gl._h.jacobian(False)
        return _HostArray(gp)

    @property
    def _free_energy_jacobian_A(self):
        if not self._gl.params.solveA:
            return None
        _, gA = self._gl._h.jacobian(True)
        return _HostArray(gA)

    @staticmethod
    def _as_flat(x):
        if hasattr(x, "get") and not isinstance(x, np.ndarray):
            x = x.get()
        return np.asarray(x).reshape(-1) if np.ndim(x) == 1 else _flat(x)

    def _free_energy_conjgrad_coef_psi(self, dpsi):
        self._c = self._gl._h.conjgrad_coef(self._as_flat(dpsi))
        return self._c.copy()

    def _free_energy_conjgrad_coef(self, dpsi, dab):
        if isinstance(dab, tuple):
            dab = np.concatenate([_flat(dab[0]), _flat(dab[1])])
        c17 = self._gl._h.conjgrad_coef(self._as_flat(dpsi), self._as_flat(dab))
        self._c = _coef_matrix(c17)
        return self._c.copy()

    @staticmethod
    def _alpha_psi(c):
        """Smallest real non-negative root of dP/dalpha (``svirl/solvers/cg.py:227-235``)."""
        am = np.polynomial.polynomial.polyroots([c[1], 2.0 * c[2], 3.0 * c[3], 4.0 * c[4]])
        am = am[np.isclose(am.imag, 0)].real
        am = am[am >= 0]
        return np.min(am)

    @staticmethod
    def _alpha_joint(c, alpha0=(0.0, 0.0), tol=1e-8):
        """BFGS on the (alpha_psi, alpha_A) polynomial (``svirl/solvers/cg.py:378-419``)."""
        cj0 = np.polynomial.polynomial.polyder(c, axis=0)
        cj1 = np.polynomial.polynomial.polyder(c, axis=1)
        f = lambda al: np.polynomial.polynomial.polyval2d(al[0], al[1], c)
        j = lambda al: np.array([np.polynomial.polynomial.polyval2d(al[0], al[1], cj0),
                                 np.polynomial.polynomial.polyval2d(al[0], al[1], cj1)])
        return scipy.optimize.minimize(f, x0=np.array(alpha0), jac=j, method="BFGS", tol=tol).x

    def _solve(self, n_iter=1000):
        gl, h = self._gl, self._gl._h
        dt = gl.cfg.dtype
        solveA = gl.params.solveA
        self.cg_energies = []
        if not solveA:
            h.cg_reset_direction()
        for i in range(n_iter):
            h.cg_gradient(i > 0)
            if solveA:
                c = _coef_matrix(h.cg_coefficients(17))
                a_psi, a_A = self._alpha_joint(c)
                E = h.cg_update(float(dt(a_psi)), float(dt(a_A)))
            else:
                c = h.cg_coefficients(5)
                a = self._alpha_psi(c)
                E = h.cg_update(float(dt(a)), 0.0)
            self._c = c
            self.cg_energies.append(E)
            if i > 0 and np.abs(self.cg_energies[i] / self.cg_energies[i - 1] - 1.0) < self._convergence_rtol:
                break


def _coef_matrix(c17):
    c = np.zeros((5, 5))
    c[0, :] = c17[0:5]
    c[1, :] = c17[5:10]
    c[2, :] = c17[10:15]
    c[3, 0] = c17[15]
    c[4, 0] = c17[16]
    return c


class Solvers:
    """``svirl/solvers/solvers.py``."""

    def __init__(self, gl):
        self._gl = gl
        self._td = None
        self._cg = None
        self.__detected = False

    def td(self, dt=0.1, Nt=1000, T=None, eqn=None):
        assert isinstance(Nt, (np.integer, int))
        assert isinstance(dt, (np.floating, float, np.integer, int))
        if eqn is not None:
            assert eqn in ["order_parameter", "vector_potential"]
        if T is not None:
            assert isinstance(T, (np.floating, float, np.integer, int))
        self._init_td()
        self._td._solve(dt=dt, Nt=Nt, T=T, eqn=eqn)
        self.vortices_detected = False

    def cg(self, n_iter=1000):
        self._init_cg()
        self._cg._solve(n_iter)
        self.vortices_detected = False

    @property
    def td_scheme(self):
        """The order parameter's time stepping in ``td``: "backward_euler" (the
        reference's, default), "crank_nicolson" or "crank_nicolson_as_written"
        (see TD.scheme; the reference cannot reach them: its kernel is commented
        out, svirl/cuda/td.h:136-292)."""
        self._init_td()
        return self._td.scheme

    @td_scheme.setter
    def td_scheme(self, value):
        self._init_td()
        self._td.scheme = value

    @property
    def vortices_detected(self):
        return self.__detected

    @vortices_detected.setter
    def vortices_detected(self, status):
        assert isinstance(status, bool)
        self.__detected = status

    def _init_td(self):
        if self._td is None:
            self._td = TD(self._gl)

    def _init_cg(self):
        if self._cg is None:
            self._cg = CG(self._gl)


class _Reduction:
    """``gl.par.red`` test hooks (``svirl/parallel/reduction.py:179-198``): the sums
    run in the library's single-launch FP64 reduction kernel.  ``block_size`` is
    accepted for compatibility; the launch shape is the library's."""

    def __init__(self, gl):
        self._gl = gl

    def test_sum(self, a_in, N, block_size=256):
        return float(self._gl._h.reduce_sum(np.asarray(a_in, dtype=np.float64)[:N], 1)[0])

    def test_sum_v(self, a_in, nv, ne, block_size=256):
        return self._gl._h.reduce_sum(np.asarray(a_in, dtype=np.float64)[: nv * ne], ne)


class GLSolver:
    """2D Ginzburg-Landau solver on one GB300 GPU, API of ``svirl.GLSolver``
    (``svirl/__init__.py:30-63``)."""

    def __init__(self,
                 Nx=None, dx=None, Lx=None,
                 Ny=None, dy=None, Ly=None,
                 Nt=None, dt=None, T=None,
                 NtA=None, dtA=None, TA=None,
                 material_tiling=None,
                 order_parameter="random",
                 random_seed=None,
                 random_level=1.0,
                 gl_parameter=np.inf,
                 normal_conductivity=1.0,
                 linear_coefficient=1.0,
                 homogeneous_external_field=0.0,
                 external_field=0.0,
                 fixed_vortices=None,
                 fixed_vortices_correction="cell centers",
                 phase_lock_radius=None,
                 device_id=0,
                 dtype=np.float64,
                 stop_criterion_order_parameter=1e-6,
                 stop_criterion_vector_potential=1e-6,
                 order_parameter_Langevin_coefficient=0.0,
                 vector_potential_Langevin_coefficient=0.0,
                 convergence_rtol=1e-6):
        self.dtypes = (np.float32, np.float64)
        cfg = types.SimpleNamespace()
        cfg.device_id = device_id
        cfg.dtype, cfg.dtype_complex = _dtypes(dtype)

        if Nx is not None and Lx is not None and dx is None:
            dx = float(Lx) / (Nx - 1)
        elif Nx is not None and Lx is None and dx is not None:
            Lx = float(dx) * (Nx - 1)
        elif Nx is None and Lx is not None and dx is not None:
            Nx = int(np.round(Lx / dx) + 1)
        elif Nx is not None and Lx is not None and dx is not None:
            assert np.isclose(Lx, dx * (Nx - 1))
        else:
            raise TypeError("Two out of three Nx, Lx, dx must be defined")
        if Ny is not None and Ly is not None and dy is None:
            dy = float(Ly) / (Ny - 1)
        elif Ny is not None and Ly is None and dy is not None:
            Ly = float(dy) * (Ny - 1)
        elif Ny is None and Ly is not None and dy is not None:
            Ny = int(np.round(Ly / dy) + 1)
        elif Ny is not None and Ly is not None and dy is not None:
            assert np.isclose(Ly, dy * (Ny - 1))
        else:
            raise TypeError("Two out of three Ny, Ly, and dy must be defined")
        assert isinstance(Lx, (np.floating, float, np.integer, int)) and Lx > 0.0
        assert isinstance(Ly, (np.floating, float, np.integer, int)) and Ly > 0.0
        assert isinstance(Nx, (np.integer, int)) and Nx >= 4
        assert isinstance(Ny, (np.integer, int)) and Ny >= 4

        d = cfg.dtype
        cfg.Nx, cfg.Ny = np.int32(Nx), np.int32(Ny)
        cfg.Lx, cfg.Ly = d(Lx), d(Ly)
        cfg.dx, cfg.dy = d(dx), d(dy)
        cfg.N = cfg.Nx * cfg.Ny
        cfg.Nxa, cfg.Nya = cfg.Nx - 1, cfg.Ny
        cfg.Nxb, cfg.Nyb = cfg.Nx, cfg.Ny - 1
        cfg.Na, cfg.Nb = cfg.Nxa * cfg.Nya, cfg.Nxb * cfg.Nyb
        cfg.Nab = cfg.Na + cfg.Nb
        cfg.Nxc, cfg.Nyc = cfg.Nx - 1, cfg.Ny - 1
        cfg.Nc = cfg.Nxc * cfg.Nyc
        cfg.idx, cfg.idy = 1.0 / cfg.dx, 1.0 / cfg.dy
        cfg.idx2, cfg.idy2, cfg.idxy = cfg.idx * cfg.idx, cfg.idy * cfg.idy, cfg.idx * cfg.idy
        cfg.j_dx, cfg.j_dy = 1.0j * cfg.dx, 1.0j * cfg.dy
        cfg.material_tiling = material_tiling
        cfg.order_parameter = order_parameter
        cfg.random_seed = random_seed
        cfg.random_level = random_level
        cfg.gl_parameter = gl_parameter
        cfg.linear_coefficient = linear_coefficient
        cfg.normal_conductivity = normal_conductivity
        cfg.homogeneous_external_field = homogeneous_external_field
        cfg.external_field = external_field
        cfg.fixed_vortices = fixed_vortices
        cfg.fixed_vortices_correction = fixed_vortices_correction
        cfg.phase_lock_radius = phase_lock_radius
        cfg.order_parameter_Langevin_coefficient = order_parameter_Langevin_coefficient
        cfg.vector_potential_Langevin_coefficient = vector_potential_Langevin_coefficient
        cfg.Nt, cfg.dt, cfg.T = Nt, dt, T
        cfg.NtA, cfg.dtA, cfg.TA = NtA, dtA, TA
        assert isinstance(stop_criterion_order_parameter, (np.floating, float, np.integer, int)) and stop_criterion_order_parameter > 0.0
        assert isinstance(stop_criterion_vector_potential, (np.floating, float, np.integer, int)) and stop_criterion_vector_potential > 0.0
        cfg.stop_criterion_order_parameter = d(stop_criterion_order_parameter)
        cfg.stop_criterion_vector_potential = d(stop_criterion_vector_potential)
        cfg.convergence_rtol = convergence_rtol
        self.cfg = cfg

        self._h = _lib.Handle(cfg.Nx, cfg.Ny, float(cfg.dx), float(cfg.dy), cfg.dtype, device=device_id)
        self._h.set_params(stop_psi=float(cfg.stop_criterion_order_parameter),
                           stop_A=float(cfg.stop_criterion_vector_potential),
                           rand_t=int(random_seed) & 0xFFFFFFFF if random_seed is not None else 1)
        self.par = types.SimpleNamespace(red=_Reduction(self))
        self.mesh = Mesh(self, material_tiling)
        self.vars = Vars(self)
        if order_parameter == "random":
            self.vars.order_parameter = 1.0
            self.vars.randomize_order_parameter(level=random_level, seed=random_seed)
        else:
            self.vars.order_parameter = order_parameter
        self.params = Params(self, cfg)
        self.observables = Observables(self)
        self.solve = Solvers(self)
        self.vortex_detector = VortexDetector(self)

    def close(self):
        """Release the device buffers now (they are also released on garbage collection)."""
        self._h.close()

    # flatten helpers (svirl/__init__.py:185-206)
    def flatten_a_array(self, a):
        return np.reshape(a.T, self.cfg.Na)

    def unflatten_a_array(self, a):
        return np.reshape(a, (self.cfg.Nya, self.cfg.Nxa)).T

    def flatten_b_array(self, b):
        return np.reshape(b.T, self.cfg.Nb)

    def unflatten_b_array(self, b):
        return np.reshape(b, (self.cfg.Nyb, self.cfg.Nxb)).T

    def flatten_array(self, psi):
        return np.reshape(psi.T, self.cfg.N)

    def unflatten_array(self, psi):
        return np.reshape(psi, (self.cfg.Ny, self.cfg.Nx)).T
