"""``pycuda.compiler.SourceModule`` whose functions are the NumPy kernels.

``get_function(name)`` returns a callable with the reference's launch
convention (positional kernel arguments, ``grid=``/``block=`` keywords).  The
grid geometry, which the reference bakes into its kernels at compile time
(``svirl/parallel/startup.py:54-63``), is read from ``svirl.config`` at call
time.  Arguments are GPUArray objects, NumPy scalars, or an integer 0 for NULL.
"""

import sys

import numpy as np

from oracle import kernels_np as K
from .gpuarray import GPUArray


def _arr(x):
    return x._a if isinstance(x, GPUArray) else None


def _f(x):
    # pycuda packs a 1-element host array argument as its scalar value
    return float(np.asarray(x).reshape(-1)[0])


def _grid():
    cfg = sys.modules["svirl.config"]
    return K.Grid(cfg.Nx, cfg.Ny, cfg.dx, cfg.dy), cfg


def _store(dst, values):
    dst[: values.size] = values.astype(dst.dtype, copy=False)


def _block_partials(values, nblocks, bs):
    pad = np.zeros(nblocks * bs, dtype=np.float64)
    pad[: values.size] = values[: nblocks * bs]
    return pad.reshape(nblocks, bs).sum(axis=1)


def iterate_order_parameter_jacobi_step(dt, eps, eps_sp, mt, ab_abi, psi_rhs, psi, psi_next,
                                        langevin_c, jstep, rand_t, stop_eps, r2_max, **launch):
    g, _ = _grid()
    rhs = _arr(psi_rhs)
    rhs64 = rhs.astype(np.complex128)
    nxt, r = K.iterate_order_parameter_jacobi_step(
        g, _f(dt), _f(eps), None if _arr(eps_sp) is None else _arr(eps_sp).astype(np.float64),
        _arr(mt), None if _arr(ab_abi) is None else _arr(ab_abi).astype(np.float64),
        rhs64, _arr(psi).astype(np.complex128), _f(langevin_c), int(jstep), int(rand_t), _f(stop_eps))
    rhs[:] = rhs64.astype(rhs.dtype)
    _store(_arr(psi_next), nxt)
    r2 = _arr(r2_max)
    r2[0] = max(int(r2[0]), min(r, 2 ** 31 - 1))


def order_parameter_phase_lock(psi, lock_N, lock_ns, **launch):
    ns = _arr(lock_ns)[: int(lock_N)].astype(np.int64)
    K.order_parameter_phase_lock(_arr(psi), ns)


def iterate_vector_potential_jacobi_step(dt, kappa2, rho, H, mt, psi, abi_ab_rhs, ab_rhs, ab, ab_next,
                                         langevin_c, jstep, rand_t, stop_eps, r2_max, **launch):
    g, _ = _grid()
    rhs = _arr(ab_rhs)
    rhs64 = rhs.astype(np.float64)
    nxt, r = K.iterate_vector_potential_jacobi_step(
        g, _f(dt), _f(kappa2), _f(rho), _f(H), _arr(mt), _arr(psi).astype(np.complex128),
        _arr(abi_ab_rhs).astype(np.float64), rhs64, _arr(ab).astype(np.float64),
        _f(langevin_c), int(jstep), int(rand_t), _f(stop_eps))
    rhs[:] = rhs64.astype(rhs.dtype)
    _store(_arr(ab_next), nxt)
    r2 = _arr(r2_max)
    r2[0] = max(int(r2[0]), min(r, 2 ** 31 - 1))


def _opt64(x):
    a = _arr(x)
    return None if a is None else a.astype(np.float64)


def magnetic_field(abei, ab, B, **launch):
    g, _ = _grid()
    _store(_arr(B), K.magnetic_field(g, _opt64(abei), _opt64(ab)))


def current_density(kappa2, H, abei, ab, jxjy, **launch):
    g, _ = _grid()
    _store(_arr(jxjy), K.current_density(g, _f(kappa2), _f(H), _opt64(abei), _opt64(ab)))


def supercurrent_density(mt, psi, abei, ab, jsxjsy, **launch):
    g, _ = _grid()
    _store(_arr(jsxjsy), K.supercurrent_density(g, _arr(mt), _arr(psi).astype(np.complex128),
                                                _opt64(abei), _opt64(ab)))


def free_energy_pseudodensity(kappa2, eps, eps_sp, H, mt, psi, abei, ab, G, **launch):
    g, _ = _grid()
    part = K.free_energy_pseudodensity(g, _f(kappa2), _f(eps), _opt64(eps_sp), _f(H), _arr(mt),
                                       _arr(psi).astype(np.complex128), _opt64(abei), _opt64(ab))
    _store(_arr(G), part)


def free_energy_jacobian_psi(kappa2, eps, eps_sp, H, mt, psi, abei, ab, G, **launch):
    g, _ = _grid()
    jac = K.free_energy_jacobian_psi(g, _f(kappa2), _f(eps), _opt64(eps_sp), _f(H), _arr(mt),
                                     _arr(psi).astype(np.complex128), _opt64(abei), _opt64(ab))
    out = _arr(G)
    out[:] = (out.astype(np.complex128) + jac).astype(out.dtype)


def free_energy_jacobian_A(kappa2, H, mt, psi, abei, ab, G, **launch):
    g, _ = _grid()
    jac = K.free_energy_jacobian_A(g, _f(kappa2), _f(H), _arr(mt), _arr(psi).astype(np.complex128),
                                   _opt64(abei), _opt64(ab))
    out = _arr(G)
    out[:] = (out.astype(np.float64) + jac).astype(out.dtype)


def _write_coef(C, tot, nv, grid):
    out = _arr(C)
    nblocks = int(grid[0])
    vals = np.zeros(nblocks * nv)
    vals[:nv] = tot  # grid total in block 0's slot, zeros in the others
    _store(out, vals)


def free_energy_conjgrad_coef_psi(kappa2, eps, eps_sp, H, mt, psi, dpsi, abei, ab, C, grid=(1, 1, 1), **launch):
    g, _ = _grid()
    tot = K.free_energy_conjgrad_coef_psi_total(g, _f(kappa2), _f(eps), _opt64(eps_sp), _f(H), _arr(mt),
                                                _arr(psi).astype(np.complex128), _arr(dpsi).astype(np.complex128),
                                                _opt64(abei), _opt64(ab))
    _write_coef(C, tot, 5, grid)


def free_energy_conjgrad_coef(kappa2, eps, eps_sp, H, mt, psi, dpsi, abei, ab, dab, C, grid=(1, 1, 1), **launch):
    g, _ = _grid()
    tot = K.free_energy_conjgrad_coef_total(g, _f(kappa2), _f(eps), _opt64(eps_sp), _f(H), _arr(mt),
                                            _arr(psi).astype(np.complex128), _arr(dpsi).astype(np.complex128),
                                            _opt64(abei), _opt64(ab), _arr(dab).astype(np.float64))
    _write_coef(C, tot, 17, grid)


def _partials(vals, z, grid, block):
    nb, bs = int(grid[0]), int(block[0])
    _store(_arr(z), _block_partials(vals, nb, bs))


def xmyx_c_sum(x, y, z, N, grid=(1, 1, 1), block=(128, 1, 1)):
    n = int(N)
    a, b = _arr(x)[:n].astype(np.complex128), _arr(y)[:n].astype(np.complex128)
    _partials(a.real * (a.real - b.real) + a.imag * (a.imag - b.imag), z, grid, block)


def xmyx_r_sum(x, y, z, N, grid=(1, 1, 1), block=(128, 1, 1)):
    n = int(N)
    a, b = _arr(x)[:n].astype(np.float64), _arr(y)[:n].astype(np.float64)
    _partials(a * (a - b), z, grid, block)


def x_mag2_c_sum(x, y, N, grid=(1, 1, 1), block=(128, 1, 1)):
    n = int(N)
    a = _arr(x)[:n].astype(np.complex128)
    _partials(a.real * a.real + a.imag * a.imag, y, grid, block)


def x_mag2_r_sum(x, y, N, grid=(1, 1, 1), block=(128, 1, 1)):
    n = int(N)
    a = _arr(x)[:n].astype(np.float64)
    _partials(a * a, y, grid, block)


def axpy_c(x, y, z, alpha, N, **launch):
    n = int(N)
    _arr(z)[:n] = (_f(alpha) * _arr(x)[:n] + _arr(y)[:n]).astype(_arr(z).dtype)


def axpy_r(x, y, z, alpha, N, **launch):
    axpy_c(x, y, z, alpha, N)


def axmy_c(x, y, z, alpha, N, **launch):
    n = int(N)
    al = float(_arr(alpha)[0])
    _arr(z)[:n] = (al * _arr(x)[:n] - _arr(y)[:n]).astype(_arr(z).dtype)


def axmy_r(x, y, z, alpha, N, **launch):
    axmy_c(x, y, z, alpha, N)


def xpy_r(x, y, N, **launch):
    n = int(N)
    _arr(x)[:n] += _arr(y)[:n]


def xmy_r(x, y, N, **launch):
    n = int(N)
    _arr(x)[:n] -= _arr(y)[:n]


def divide_scalars_positive(x, y, z, **launch):
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.float64(_arr(x)[0]) / np.float64(_arr(y)[0])
    _arr(z)[0] = np.fmax(q, 0.0)


def sum(inp, out, N, grid=(1, 1, 1), block=(128, 1, 1)):
    """Grid-stride block sums (``svirl/cuda/block_reduction.h:80-92``)."""
    n, nb, bs = int(N), int(grid[0]), int(block[0])
    vals = _arr(inp)[:n].astype(np.float64)
    stride = nb * bs
    k = (n + stride - 1) // stride
    pad = np.zeros(max(k, 1) * stride)
    pad[:n] = vals
    _store(_arr(out), pad.reshape(-1, nb, bs).sum(axis=(0, 2)))


def sum_v(inp, out, N, grid=(1, 1, 1), block=(128, 1, 1)):
    """Vector grid-stride block sums (``svirl/cuda/reduction.h:56-82``)."""
    cfg = sys.modules["svirl.config"]
    nv = 5 if np.isposinf(cfg.gl_parameter) else 17
    n, nb, bs = int(N), int(grid[0]), int(block[0])
    vals = _arr(inp)[: n * nv].astype(np.float64).reshape(n, nv)
    stride = nb * bs
    k = (n + stride - 1) // stride
    pad = np.zeros((max(k, 1) * stride, nv))
    pad[:n] = vals
    _store(_arr(out), pad.reshape(-1, nb, bs, nv).sum(axis=(0, 2)).reshape(-1))


_KERNELS = {name: fn for name, fn in globals().items()
            if callable(fn) and not name.startswith("_") and name not in ("GPUArray",)}


class SourceModule:
    def __init__(self, code, options=None, **kw):
        self.code = code

    def get_function(self, name):
        if name not in _KERNELS:
            raise KeyError(name)
        return _KERNELS[name]
