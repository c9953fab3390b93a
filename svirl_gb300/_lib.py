"""ctypes binding of libglgpu.so (the C ABI declared in include/glgpu.h).

The library is built in-tree (``svirl_gb300/_build/libglgpu.so``).  If it is
missing it is built here when nvcc is available; otherwise importing the
solver fails loudly: there is no CPU fallback.
"""
import ctypes as C
import os
import threading
import warnings

import numpy as np

from . import build as _build

GLGPU_OK = 0
GLGPU_E_ARG = -1
GLGPU_E_CUDA = -2
GLGPU_E_OOM = -3
GLGPU_E_TIMEOUT = -4
GLGPU_E_NAN = -5
GLGPU_E_NOROOT = -6


class Grid(C.Structure):
    _fields_ = [("Nx", C.c_int32), ("Ny", C.c_int32), ("dx", C.c_double), ("dy", C.c_double), ("dtype", C.c_int32)]


class Params(C.Structure):
    _fields_ = [("kappa", C.c_double), ("sigma", C.c_double), ("epsilon", C.c_double), ("H", C.c_double),
                ("stop_psi", C.c_double), ("stop_A", C.c_double), ("langevin_psi", C.c_double),
                ("langevin_A", C.c_double), ("rand_t", C.c_uint32), ("pad_", C.c_int32)]


class TDStats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("max_sweeps_psi", C.c_int32), ("max_sweeps_A", C.c_int32),
                ("last_sweeps_psi", C.c_int32), ("last_sweeps_A", C.c_int32), ("nan_seen", C.c_int32),
                ("total_sweeps_psi", C.c_int64), ("total_sweeps_A", C.c_int64), ("rand_t", C.c_uint32),
                ("used_graph", C.c_int32), ("sweep_launches", C.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_H = C.c_void_p
_P = C.c_void_p
_SIGNATURES = {
    "glgpu_version": (C.c_int, []),
    "glgpu_psi_sweeps_per_launch": (C.c_int, []),
    "glgpu_psi_strip_rows": (C.c_int, [_H]),
    "glgpu_set_psi_strip_rows": (C.c_int, [_H, C.c_int32]),
    "glgpu_set_psi_sweep_kernel": (C.c_int, [_H, C.c_int32]),
    "glgpu_set_psi_scheme": (C.c_int, [_H, C.c_int32]),
    "glgpu_set_irregular_vector_potential": (C.c_int, [_H, _P, C.c_int32]),
    "glgpu_get_irregular_vector_potential": (C.c_int, [_H, _P]),
    "glgpu_set_phase_lock": (C.c_int, [_H, _P, C.c_int32]),
    "glgpu_last_error": (C.c_char_p, [_H]),
    "glgpu_create": (C.c_int, [C.POINTER(Grid), C.c_int32, C.POINTER(_H)]),
    "glgpu_destroy": (C.c_int, [_H]),
    "glgpu_set_params": (C.c_int, [_H, C.POINTER(Params)]),
    "glgpu_get_params": (C.c_int, [_H, C.POINTER(Params)]),
    "glgpu_set_order_parameter": (C.c_int, [_H, _P]),
    "glgpu_get_order_parameter": (C.c_int, [_H, _P]),
    "glgpu_set_vector_potential": (C.c_int, [_H, _P]),
    "glgpu_get_vector_potential": (C.c_int, [_H, _P]),
    "glgpu_set_external_vector_potential": (C.c_int, [_H, _P]),
    "glgpu_set_material_tiling": (C.c_int, [_H, _P]),
    "glgpu_set_linear_coefficient_field": (C.c_int, [_H, _P]),
    "glgpu_td": (C.c_int, [_H, C.c_double, C.c_int32, C.c_int32, C.POINTER(TDStats)]),
    "glgpu_set_use_graphs": (C.c_int, [_H, C.c_int32]),
    "glgpu_set_loop_guard": (C.c_int, [_H, C.c_int32]),
    "glgpu_td_timed": (C.c_int, [_H, C.c_double, C.c_int32, C.c_int32, C.POINTER(TDStats), C.POINTER(C.c_double)]),
    "glgpu_time_sweeps": (C.c_int, [_H, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "glgpu_free_energy": (C.c_int, [_H, C.POINTER(C.c_double)]),
    "glgpu_magnetic_field": (C.c_int, [_H, _P]),
    "glgpu_current_density": (C.c_int, [_H, _P]),
    "glgpu_supercurrent_density": (C.c_int, [_H, _P]),
    "glgpu_vortex_candidates": (C.c_int, [_H, C.c_int32, C.POINTER(C.c_int32), _P, _P]),
    "glgpu_cg_reset_direction": (C.c_int, [_H]),
    "glgpu_cg_gradient": (C.c_int, [_H, C.c_int32]),
    "glgpu_cg_coefficients": (C.c_int, [_H, _P]),
    "glgpu_cg_update": (C.c_int, [_H, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "glgpu_jacobian": (C.c_int, [_H, _P, _P]),
    "glgpu_conjgrad_coef": (C.c_int, [_H, _P, _P, _P]),
    "glgpu_reduce_sum": (C.c_int, [_H, _P, C.c_int64, C.c_int32, _P]),
    "glgpu_free_energy_noalloc": (C.c_int, [C.POINTER(Grid), C.POINTER(Params), _P, _P, _P, _P, _P, _P]),
    "glgpu_batch_create": (C.c_int, [C.POINTER(_H), C.c_int32, C.POINTER(_H)]),
    "glgpu_batch_destroy": (C.c_int, [_H]),
    "glgpu_batch_last_error": (C.c_char_p, [_H]),
    "glgpu_batch_td": (C.c_int, [_H, C.c_double, C.c_int32, C.c_int32, C.POINTER(TDStats), C.POINTER(C.c_double)]),
    "glgpu_batch_set_use_graphs": (C.c_int, [_H, C.c_int32]),
    "glgpu_batch_set_loop_guard": (C.c_int, [_H, C.c_int32]),
    "glgpu_batch_set_energy_targets": (C.c_int, [_H, _P, C.c_double]),
    "glgpu_batch_set_cg_window": (C.c_int, [_H, C.c_int32, C.c_double]),
    "glgpu_batch_cg": (C.c_int, [_H, C.c_int32, C.c_double, C.c_double, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    # learned warm start (include/glgpu_nn.h)
    "glnn_set_conv_tma": (C.c_int, [C.c_int32]),
    "glnn_conv3x3_fwd": (C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int32, C.c_int32, _P, _P]),
    "glnn_relu_mask": (C.c_int, [_P, _P, _P, C.c_int64, _P]),
    "glnn_conv3x3_bwd_data": (C.c_int, [_P, _P, C.c_int32, _P, _P, C.c_int32, _P, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_int32, C.c_int32, _P, _P]),
    "glnn_conv3x3_bwd_weight_work": (C.c_int64, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "glnn_conv3x3_bwd_weight": (C.c_int, [_P, _P, C.c_int32, _P, C.c_int32, _P, C.c_int32, _P, _P, _P, C.c_int64,
                                          C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P]),
    "glnn_prep_weights": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, _P]),
    "glnn_pool2_fwd": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "glnn_pool2_bwd": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "glnn_up2_fwd": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "glnn_up2_bwd": (C.c_int, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "glnn_add": (C.c_int, [_P, _P, _P, C.c_int64, _P]),
    "glnn_mse": (C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P, _P, C.c_int64, _P]),
    "glnn_adam": (C.c_int, [_P, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                            C.c_int32, _P]),
    "glnn_f32_to_bf16": (C.c_int, [_P, _P, C.c_int64, _P]),
    "glnn_bf16_to_f32": (C.c_int, [_P, _P, C.c_int64, _P]),
}

_lib = None
_lock = threading.Lock()


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libglgpu.so, building it first if it is missing and nvcc exists."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise ImportError("libglgpu.so is not built; run svirl_gb300.build.build()")
            try:
                _build.build()
            except Exception as e:  # no nvcc / compile error: no fallback exists
                raise ImportError("libglgpu.so is missing and could not be built: %s" % e) from e
        lib = C.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class GLGPUError(RuntimeError):
    pass


def check(rc, h=None, what=""):
    if rc == GLGPU_OK:
        return
    msg = load().glgpu_last_error(h)
    msg = msg.decode() if msg else ""
    if rc == GLGPU_E_NAN:
        warnings.warn("glgpu: %s %s" % (what, msg), RuntimeWarning, stacklevel=3)
        return
    raise GLGPUError("glgpu error %d in %s: %s" % (rc, what, msg))


def ptr(a):
    """Data pointer of a C-contiguous NumPy array (or None -> NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


class Handle:
    """Owns one glgpu_handle (one GL instance on one GPU)."""

    def __init__(self, Nx, Ny, dx, dy, dtype, device=0):
        lib = load()
        self.lib = lib
        self.dtype = np.dtype(dtype)
        self.ctype = np.complex64 if self.dtype == np.float32 else np.complex128
        g = Grid(int(Nx), int(Ny), float(dx), float(dy), 4 if self.dtype == np.float32 else 8)
        h = _H()
        rc = lib.glgpu_create(C.byref(g), int(device), C.byref(h))
        if rc != GLGPU_OK:
            msg = lib.glgpu_last_error(None)
            raise GLGPUError("glgpu_create failed (%d): %s" % (rc, msg.decode() if msg else ""))
        self.h = h
        self.Nx, self.Ny = int(Nx), int(Ny)
        self.N = self.Nx * self.Ny
        self.Na = (self.Nx - 1) * self.Ny
        self.Nab = self.Na + self.Nx * (self.Ny - 1)
        self.Nc = (self.Nx - 1) * (self.Ny - 1)

    def close(self):
        if getattr(self, "h", None):
            self.lib.glgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # params / state ----------------------------------------------------------
    def get_params(self):
        p = Params()
        check(self.lib.glgpu_get_params(self.h, C.byref(p)), self.h, "get_params")
        return p

    def kappa_finite(self):
        k = float(self.get_params().kappa)
        return k > 0.0 and np.isfinite(k)

    def set_params(self, **kw):
        p = self.get_params()
        for k, v in kw.items():
            setattr(p, k, v)
        check(self.lib.glgpu_set_params(self.h, C.byref(p)), self.h, "set_params")

    def set_psi(self, psi_flat):
        a = np.ascontiguousarray(psi_flat, dtype=self.ctype)
        assert a.size == self.N
        check(self.lib.glgpu_set_order_parameter(self.h, ptr(a)), self.h, "set_order_parameter")

    def get_psi(self):
        a = np.empty(self.N, dtype=self.ctype)
        check(self.lib.glgpu_get_order_parameter(self.h, ptr(a)), self.h, "get_order_parameter")
        return a

    def set_ab(self, ab_flat):
        a = np.ascontiguousarray(ab_flat, dtype=self.dtype)
        assert a.size == self.Nab
        check(self.lib.glgpu_set_vector_potential(self.h, ptr(a)), self.h, "set_vector_potential")

    def get_ab(self):
        a = np.empty(self.Nab, dtype=self.dtype)
        check(self.lib.glgpu_get_vector_potential(self.h, ptr(a)), self.h, "get_vector_potential")
        return a

    def set_abei(self, abei_flat):
        a = None if abei_flat is None else np.ascontiguousarray(abei_flat, dtype=self.dtype)
        check(self.lib.glgpu_set_external_vector_potential(self.h, ptr(a)), self.h, "set_external_vector_potential")

    def set_mask(self, mt_flat):
        a = None if mt_flat is None else np.ascontiguousarray(mt_flat, dtype=np.uint8)
        check(self.lib.glgpu_set_material_tiling(self.h, ptr(a)), self.h, "set_material_tiling")

    def set_eps_field(self, eps_flat):
        a = None if eps_flat is None else np.ascontiguousarray(eps_flat, dtype=self.dtype)
        check(self.lib.glgpu_set_linear_coefficient_field(self.h, ptr(a)), self.h, "set_linear_coefficient_field")

    def set_irregular_vector_potential(self, vpi_flat, td_copy_only=False):
        a = None if vpi_flat is None else np.ascontiguousarray(vpi_flat, dtype=self.dtype)
        if a is not None:
            assert a.size == self.Nab
        check(self.lib.glgpu_set_irregular_vector_potential(self.h, ptr(a), 1 if td_copy_only else 0), self.h,
              "set_irregular_vector_potential")

    def get_irregular_vector_potential(self):
        a = np.empty(self.Nab, dtype=self.dtype)
        check(self.lib.glgpu_get_irregular_vector_potential(self.h, ptr(a)), self.h, "get_irregular_vector_potential")
        return a

    def set_phase_lock(self, nodes):
        a = np.ascontiguousarray([] if nodes is None else nodes, dtype=np.int32)
        check(self.lib.glgpu_set_phase_lock(self.h, ptr(a) if a.size else None, int(a.size)), self.h, "set_phase_lock")

    def psi_strip_rows(self):
        return int(self.lib.glgpu_psi_strip_rows(self.h))

    def set_psi_strip_rows(self, rows):
        check(self.lib.glgpu_set_psi_strip_rows(self.h, int(rows)), self.h, "set_psi_strip_rows")

    def set_psi_scheme(self, scheme):
        """psi time stepping: 0 backward Euler (the reference's), 1 Crank-Nicolson,
        2 the reference's Crank-Nicolson kernel as written."""
        check(self.lib.glgpu_set_psi_scheme(self.h, int(scheme)), self.h, "set_psi_scheme")

    def set_psi_sweep_kernel(self, select):
        """FP32 psi sweep kernel: 0 = register strip (default), 1 = bulk-copy ring."""
        check(self.lib.glgpu_set_psi_sweep_kernel(self.h, int(select)), self.h, "set_psi_sweep_kernel")

    def set_use_graphs(self, enable):
        check(self.lib.glgpu_set_use_graphs(self.h, 1 if enable else 0), self.h, "set_use_graphs")

    def set_loop_guard(self, launches):
        check(self.lib.glgpu_set_loop_guard(self.h, int(launches)), self.h, "set_loop_guard")

    # TD ------------------------------------------------------------------------
    def td(self, dt, Nt, eqn=0):
        st = TDStats()
        check(self.lib.glgpu_td(self.h, float(dt), int(Nt), int(eqn), C.byref(st)), self.h, "td")
        return st

    def td_timed(self, dt, Nt, eqn=0):
        st = TDStats()
        ms = C.c_double()
        check(self.lib.glgpu_td_timed(self.h, float(dt), int(Nt), int(eqn), C.byref(st), C.byref(ms)), self.h, "td_timed")
        return st, ms.value

    def time_sweeps(self, which=0, nrep=10):
        ms = C.c_double()
        check(self.lib.glgpu_time_sweeps(self.h, int(which), int(nrep), C.byref(ms)), self.h, "time_sweeps")
        return ms.value

    # observables ---------------------------------------------------------------
    def free_energy(self):
        e = C.c_double()
        check(self.lib.glgpu_free_energy(self.h, C.byref(e)), self.h, "free_energy")
        return e.value

    def _real_out(self, fn, n, what):
        a = np.empty(n, dtype=self.dtype)
        check(fn(self.h, ptr(a)), self.h, what)
        return a

    def magnetic_field(self):
        return self._real_out(self.lib.glgpu_magnetic_field, self.Nc, "magnetic_field")

    def current_density(self):
        return self._real_out(self.lib.glgpu_current_density, self.Nab, "current_density")

    def supercurrent_density(self):
        return self._real_out(self.lib.glgpu_supercurrent_density, self.Nab, "supercurrent_density")

    def vortex_candidates(self, cap=1024):
        while True:
            n = C.c_int32()
            cells = np.empty(max(cap, 1), dtype=np.int32)
            corners = np.empty((max(cap, 1), 12), dtype=self.dtype)
            check(self.lib.glgpu_vortex_candidates(self.h, cap, C.byref(n), ptr(cells), ptr(corners)), self.h,
                  "vortex_candidates")
            if n.value <= cap:
                m = n.value
                order = np.argsort(cells[:m], kind="stable")
                return cells[:m][order], corners[:m][order]
            cap = int(n.value) + 16

    # CG ------------------------------------------------------------------------
    def cg_reset_direction(self):
        check(self.lib.glgpu_cg_reset_direction(self.h), self.h, "cg_reset_direction")

    def cg_gradient(self, compute_beta):
        check(self.lib.glgpu_cg_gradient(self.h, 1 if compute_beta else 0), self.h, "cg_gradient")

    def cg_coefficients(self, nv):
        c = np.zeros(17, dtype=np.float64)
        check(self.lib.glgpu_cg_coefficients(self.h, ptr(c)), self.h, "cg_coefficients")
        return c[:nv]

    def cg_update(self, alpha_psi, alpha_A):
        e = C.c_double()
        check(self.lib.glgpu_cg_update(self.h, float(alpha_psi), float(alpha_A), C.byref(e)), self.h, "cg_update")
        return e.value

    def jacobian(self, want_A):
        gp = np.empty(self.N, dtype=self.ctype)
        gA = np.empty(self.Nab, dtype=self.dtype) if want_A else None
        check(self.lib.glgpu_jacobian(self.h, ptr(gp), ptr(gA)), self.h, "jacobian")
        return gp, gA

    def reduce_sum(self, x, nv):
        a = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(max(int(nv), 1), dtype=np.float64)
        check(self.lib.glgpu_reduce_sum(self.h, ptr(a), a.size // nv, int(nv), ptr(out)), self.h, "reduce_sum")
        return out

    def conjgrad_coef(self, dpsi_flat, dab_flat=None):
        d = np.ascontiguousarray(dpsi_flat, dtype=self.ctype)
        da = None if dab_flat is None else np.ascontiguousarray(dab_flat, dtype=self.dtype)
        c = np.zeros(17, dtype=np.float64)
        check(self.lib.glgpu_conjgrad_coef(self.h, ptr(d), ptr(da), ptr(c)), self.h, "conjgrad_coef")
        return c[:5] if da is None else c
