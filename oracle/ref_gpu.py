"""The reference's own CUDA kernels, run on the GPU as its host code runs them.

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` and the fixture script under
``tests/golden/`` use this module, as a checker; nothing in the product
(``svirl_gb300``) imports it.

``oracle/ref_build.py`` compiles ``svirl/cuda/*.h`` (the reference's kernels,
unchanged) into ``oracle/_ref/*.fatbin``; this module loads those fatbins with the
CUDA driver API (ctypes on ``libcuda``) and launches the kernels with the
reference's launch geometry: 1-D grids of 128-thread blocks, ``ceil(N/128)``
blocks for every field kernel (``svirl/parallel/startup.py:65-67``,
``svirl/solvers/td.py:185,298``, ``svirl/observables/observables.py:51-145``,
``svirl/solvers/cg.py:142-212``), and the two-pass ``sum`` / ``sum_v``
reductions of ``svirl/parallel/reduction.py:40-173``.  Device memory is held in
torch tensors (plumbing only).

``RefKernels`` offers the same functions, with the same signatures, as
``oracle/kernels_np.py``, so ``oracle.gl_oracle.GLOracle(kernels=RefKernels())``
runs the oracle's host loops (TD time and Jacobi loops with the reference's stop
rule, CG with its line searches) on the reference's kernel arithmetic.
"""
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BLOCK = 128

# argument kinds per kernel: r = real_t, p = pointer (None -> NULL), i = int32, u = uint32
SIGNATURES = {
    "iterate_order_parameter_jacobi_step": "rrppppppruurp",   # td.h:4-19
    "iterate_order_parameter_jacobi_step_CN": "rrppppppruurp",  # td.h:136-150 (commented out in the reference)
    "order_parameter_phase_lock": "pip",                        # td.h:295-300
    "iterate_vector_potential_jacobi_step": "rrrrppppppruurp",  # td.h:310-326
    "magnetic_field": "ppp",                                    # observables.h:4-9
    "current_density": "rrppp",                                 # observables.h:40-47
    "supercurrent_density": "ppppp",                            # observables.h:159-166
    "free_energy_pseudodensity": "rrprppppp",                   # observables.h:250-261
    "free_energy_jacobian_psi": "rrprppppp",                    # cg.h:15-26
    "free_energy_jacobian_A": "rrppppp",                       # cg.h:124-135
    "free_energy_conjgrad_coef_psi": "rrprpppppp",              # cg.h:314-326
    "free_energy_conjgrad_coef": "rrprppppppp",                 # cg.h:477-490
    "sum": "ppi",                                               # block_reduction.h:80-91
    "sum_v": "ppi",                                             # reduction.h:56-82
}


class RefUnavailable(RuntimeError):
    pass


_drv = None


def _driver():
    global _drv
    if _drv is not None:
        return _drv
    import torch
    if not torch.cuda.is_available():
        raise RefUnavailable("no CUDA device")
    torch.cuda.init()
    torch.empty(1, device="cuda")  # the runtime makes the primary context current
    try:
        lib = ctypes.CDLL("libcuda.so.1")
    except OSError as e:
        raise RefUnavailable(str(e))
    lib.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
    lib.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
    lib.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
    lib.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
        ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
    lib.cuCtxGetCurrent.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    ctx = ctypes.c_void_p()
    _check(lib, lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RefUnavailable("no current CUDA context")
    _drv = lib
    return lib


def _check(lib, rc, what):
    if rc != 0:
        s = ctypes.c_char_p()
        lib.cuGetErrorString(rc, ctypes.byref(s))
        raise RuntimeError("%s failed: %s (%d)" % (what, (s.value or b"?").decode(), rc))


def _manifest_file():
    p = os.path.join(REF_DIR, "manifest.json")
    if not os.path.exists(p):
        return {}
    with open(p) as fh:
        return json.load(fh)


def manifest():
    return _manifest_file().get("modules", {})


def check_signatures():
    """The launcher's argument kinds must equal those parsed from the reference's
    source when the modules were built: a wrong kind would pass a number where
    the kernel reads a pointer."""
    built = _manifest_file().get("signatures")
    if not built:
        raise RefUnavailable("manifest without kernel signatures: rebuild with python -m oracle.ref_build")
    bad = {k: (v, built.get(k)) for k, v in SIGNATURES.items() if built.get(k) != v}
    if bad:
        raise RuntimeError("launcher signatures differ from the reference source: %r" % bad)


def available(dtype, Nx, Ny, dx, dy, rvl=17):
    from oracle.ref_build import module_name
    name = module_name(dtype, Nx, Ny, dx, dy, rvl)
    return os.path.exists(os.path.join(REF_DIR, name + ".fatbin"))


class RefModule:
    """One compiled module of the reference (a dtype, a geometry, a reduction length)."""

    _cache = {}

    @classmethod
    def get(cls, dtype, Nx, Ny, dx, dy, rvl):
        from oracle.ref_build import module_name
        name = module_name(dtype, Nx, Ny, dx, dy, rvl)
        if name not in cls._cache:
            cls._cache[name] = cls(name, dtype)
        return cls._cache[name]

    def __init__(self, name, dtype):
        import torch
        check_signatures()
        self.torch = torch
        self.lib = _driver()
        path = os.path.join(REF_DIR, name + ".fatbin")
        if not os.path.exists(path):
            raise RefUnavailable("reference module %s not built (python -m oracle.ref_build)" % name)
        with open(path, "rb") as fh:
            self._image = ctypes.create_string_buffer(fh.read())
        self.mod = ctypes.c_void_p()
        _check(self.lib, self.lib.cuModuleLoadData(ctypes.byref(self.mod), self._image), "cuModuleLoadData")
        self.real = np.dtype(dtype).type
        self.fns = {}

    def _fn(self, name):
        if name not in self.fns:
            f = ctypes.c_void_p()
            _check(self.lib, self.lib.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()),
                   "cuModuleGetFunction(%s)" % name)
            self.fns[name] = f
        return self.fns[name]

    def launch(self, name, grid, block, *args):
        kinds = SIGNATURES[name]
        assert len(kinds) == len(args), (name, len(kinds), len(args))
        holders = []
        for k, a in zip(kinds, args):
            if k == "r":
                holders.append((ctypes.c_double if self.real is np.float64 else ctypes.c_float)(float(a)))
            elif k == "i":
                holders.append(ctypes.c_int32(int(a)))
            elif k == "u":
                holders.append(ctypes.c_uint32(int(a) & 0xFFFFFFFF))
            else:
                holders.append(ctypes.c_void_p(0 if a is None else a.data_ptr()))
        params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        stream = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        gx, gy = (grid if isinstance(grid, tuple) else (grid, 1))
        bx, by = (block if isinstance(block, tuple) else (block, 1))
        _check(self.lib, self.lib.cuLaunchKernel(self._fn(name), int(gx), int(gy), 1, int(bx), int(by), 1, 0, stream,
                                                 params, None), "cuLaunchKernel(%s)" % name)

    # device buffers -----------------------------------------------------------
    def real_t(self, x):
        return self.torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=self.real))).cuda()

    def complex_t(self, x):
        ct = np.complex64 if self.real is np.float32 else np.complex128
        return self.torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=ct))).cuda()

    def zeros_real(self, n):
        return self.torch.zeros(int(n), dtype=self.torch.float32 if self.real is np.float32 else self.torch.float64,
                                device="cuda")

    def zeros_complex(self, n):
        return self.torch.zeros(int(n), dtype=self.torch.complex64 if self.real is np.float32 else
                                self.torch.complex128, device="cuda")

    def mask(self, mt):
        return None if mt is None else self.torch.from_numpy(np.ascontiguousarray(np.asarray(mt, dtype=bool))).cuda()

    def opt_real(self, x):
        return None if x is None else self.real_t(x)

    # reductions (svirl/parallel/reduction.py) ---------------------------------------
    def gsum(self, ga_in, N):
        """``Reduction.gsum`` (``reduction.py:40-110``): first pass over ceil(N/128)
        blocks, second pass in one block of round_up(grid, 32) (at most 128) threads."""
        grid = (N + BLOCK - 1) // BLOCK
        s1 = self.zeros_real(grid)
        if grid == 1:
            self.launch("sum", 1, BLOCK, ga_in, s1, N)
            return s1
        self.launch("sum", grid, BLOCK, ga_in, s1, N)
        s2 = self.zeros_real(1)
        bs = BLOCK if BLOCK < grid else 32 * ((grid + 31) // 32)
        self.launch("sum", 1, bs, s1, s2, grid)
        return s2

    def gsum_v(self, ga_in, nv, ne):
        """``Reduction.gsum_v`` (``reduction.py:115-173``)."""
        if nv == 1:
            return ga_in.clone()
        grid = (nv + BLOCK - 1) // BLOCK
        v1 = self.zeros_real(grid * ne)
        self.launch("sum_v", grid, BLOCK, ga_in, v1, nv)
        if grid == 1:
            return v1
        v2 = self.zeros_real(ne)
        self.launch("sum_v", 1, BLOCK, v1, v2, grid)
        return v2


def _c128(t):
    return t.cpu().numpy().astype(np.complex128)


def _f64(t):
    return t.cpu().numpy().astype(np.float64)


class RefKernels:
    """``oracle/kernels_np.py``'s kernel functions, computed by the reference's
    compiled kernels.  Inputs and outputs are NumPy arrays (FP64 / complex128 on the
    host side, cast to the module's dtype on the device)."""

    def __init__(self, dtype=np.float64):
        self.dtype = np.dtype(dtype).type
        self._last = None

    def _m(self, g, rvl=17):
        m = RefModule.get(self.dtype, g.Nx, g.Ny, g.dx, g.dy, rvl)
        self._last = m
        return m

    @staticmethod
    def _grid(n):
        return (n + BLOCK - 1) // BLOCK

    # TDGL ---------------------------------------------------------------------
    def iterate_order_parameter_jacobi_step(self, g, dt, epsilon, epsilon_spatial, mt, ab_abi,
                                            psi_rhs, psi, langevin_c, jstep, rand_t, stop_eps):
        m = self._m(g)
        if ab_abi is None:  # the kernel reads ab_abi without a NULL test (td.h:91-101)
            ab_abi = np.zeros(g.Nab)
        rhs = m.complex_t(psi_rhs)
        nxt = m.zeros_complex(g.N)
        r2 = m.torch.zeros(1, dtype=m.torch.int32, device="cuda")
        m.launch("iterate_order_parameter_jacobi_step", self._grid(g.N), BLOCK, dt, epsilon,
                 m.opt_real(epsilon_spatial), m.mask(mt), m.opt_real(ab_abi), rhs, m.complex_t(psi), nxt,
                 langevin_c, jstep, rand_t, stop_eps, r2)
        psi_rhs[:] = _c128(rhs)
        return _c128(nxt), int(r2.cpu().item())

    def iterate_order_parameter_jacobi_step_cn(self, g, dt, epsilon, epsilon_spatial, mt, ab_abi,
                                               psi_rhs, psi, langevin_c, jstep, rand_t, stop_eps, as_written=True):
        """The reference's commented-out Crank-Nicolson kernel (``td.h:136-292``),
        compiled live by the recipe.  Its threads index (i, j) =
        (blockIdx.x*blockDim.x + threadIdx.x, blockIdx.y*blockDim.y + threadIdx.y);
        no host code of the reference launches it, so the launch is 16 x 8 blocks
        over the node grid.  Only the kernel as written exists in the reference."""
        if not as_written:
            raise RefUnavailable("the reference has only the Crank-Nicolson kernel as written")
        m = self._m(g)
        if ab_abi is None:  # read without a NULL test (td.h:239-251)
            ab_abi = np.zeros(g.Nab)
        rhs = m.complex_t(psi_rhs)
        nxt = m.zeros_complex(g.N)
        r2 = m.torch.zeros(1, dtype=m.torch.int32, device="cuda")
        m.launch("iterate_order_parameter_jacobi_step_CN", ((g.Nx + 15) // 16, (g.Ny + 7) // 8), (16, 8), dt, epsilon,
                 m.opt_real(epsilon_spatial), m.mask(mt), m.opt_real(ab_abi), rhs, m.complex_t(psi), nxt,
                 langevin_c, jstep, rand_t, stop_eps, r2)
        psi_rhs[:] = _c128(rhs)
        return _c128(nxt), int(r2.cpu().item())

    def order_parameter_phase_lock(self, psi, lock_ns):
        m = self._last
        p = m.complex_t(psi)
        ns = m.torch.from_numpy(np.ascontiguousarray(np.asarray(lock_ns, dtype=np.int32))).cuda()
        n = int(ns.numel())
        m.launch("order_parameter_phase_lock", (n + 1) // 2, 2, p, n, ns)  # td.py:207-216: blocks of 2
        psi[:] = _c128(p)

    def iterate_vector_potential_jacobi_step(self, g, dt, kappa2, rho, H, mt, psi, abi_ab_rhs, ab_rhs, ab,
                                             langevin_c, jstep, rand_t, stop_eps):
        m = self._m(g)
        for a in (psi, abi_ab_rhs, ab_rhs, ab):  # read without NULL tests (td.h:350-463)
            if a is None:
                raise ValueError("the A sweep needs psi, the supercurrent argument, the right-hand side and A")
        rhs = m.real_t(ab_rhs)
        nxt = m.zeros_real(g.Nab)
        r2 = m.torch.zeros(1, dtype=m.torch.int32, device="cuda")
        m.launch("iterate_vector_potential_jacobi_step", self._grid(g.N), BLOCK, dt, kappa2, rho, H, m.mask(mt),
                 m.complex_t(psi), m.real_t(abi_ab_rhs), rhs, m.real_t(ab), nxt, langevin_c, jstep, rand_t,
                 stop_eps, r2)
        ab_rhs[:] = _f64(rhs)
        return _f64(nxt), int(r2.cpu().item())

    # observables ------------------------------------------------------------------
    def magnetic_field(self, g, abei, ab):
        m = self._m(g)
        B = m.zeros_real(g.Nc)
        m.launch("magnetic_field", self._grid(g.N), BLOCK, m.opt_real(abei), m.opt_real(ab), B)
        return _f64(B)

    def current_density(self, g, kappa2, H, abei, ab):
        m = self._m(g)
        j = m.zeros_real(g.Nab)
        m.launch("current_density", self._grid(g.N), BLOCK, kappa2, H, m.opt_real(abei), m.opt_real(ab), j)
        return _f64(j)

    def supercurrent_density(self, g, mt, psi, abei, ab):
        m = self._m(g)
        js = m.zeros_real(g.Nab)
        m.launch("supercurrent_density", self._grid(g.N), BLOCK, m.mask(mt), m.complex_t(psi), m.opt_real(abei),
                 m.opt_real(ab), js)
        return _f64(js)

    def _pseudodensity(self, m, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
        grid = self._grid(g.N)
        G = m.zeros_real(grid)
        m.launch("free_energy_pseudodensity", grid, BLOCK, kappa2, epsilon, m.opt_real(epsilon_spatial), H,
                 m.mask(mt), m.complex_t(psi), m.opt_real(abei), m.opt_real(ab), G)
        return G, grid

    def free_energy_pseudodensity(self, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
        m = self._m(g, 17 if kappa2 > 0 else 5)
        G, _ = self._pseudodensity(m, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab)
        return _f64(G)

    def free_energy(self, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
        """``Observables.free_energy`` (``observables.py:124-149``): pseudodensity + gsum."""
        m = self._m(g, 17 if kappa2 > 0 else 5)
        G, grid = self._pseudodensity(m, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab)
        return float(_f64(m.gsum(G, grid))[0])

    # CG -------------------------------------------------------------------------
    def free_energy_jacobian_psi(self, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, abei, ab):
        m = self._m(g, 17 if kappa2 > 0 else 5)
        J = m.zeros_complex(g.N)  # "needs to be initialized to 0" (cg.h:25)
        m.launch("free_energy_jacobian_psi", self._grid(g.N), BLOCK, kappa2, epsilon, m.opt_real(epsilon_spatial), H,
                 m.mask(mt), m.complex_t(psi), m.opt_real(abei), m.opt_real(ab), J)
        return _c128(J)

    def free_energy_jacobian_A(self, g, kappa2, H, mt, psi, abei, ab):
        m = self._m(g, 17)
        J = m.zeros_real(g.Nab)
        m.launch("free_energy_jacobian_A", self._grid(g.N), BLOCK, kappa2, H, m.mask(mt), m.complex_t(psi),
                 m.opt_real(abei), m.opt_real(ab), J)
        return _f64(J)

    def free_energy_conjgrad_coef_psi_total(self, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, dpsi, abei, ab):
        """Kernel + ``gsum_v`` as ``CG._free_energy_conjgrad_coef_psi`` does (``cg.py:195-224``)."""
        m = self._m(g, 5)
        grid = self._grid(g.N)
        C = m.zeros_real(5 * grid)
        m.launch("free_energy_conjgrad_coef_psi", grid, BLOCK, kappa2, epsilon, m.opt_real(epsilon_spatial), H,
                 m.mask(mt), m.complex_t(psi), m.complex_t(dpsi), m.opt_real(abei), m.opt_real(ab), C)
        return _f64(m.gsum_v(C, grid, 5) if grid > 1 else C)[:5]

    def free_energy_conjgrad_coef_total(self, g, kappa2, epsilon, epsilon_spatial, H, mt, psi, dpsi, abei, ab, dab):
        """Kernel + ``gsum_v`` as ``CG._free_energy_conjgrad_coef`` does (``cg.py:330-375``)."""
        m = self._m(g, 17)
        grid = self._grid(g.N)
        C = m.zeros_real(17 * grid)
        m.launch("free_energy_conjgrad_coef", grid, BLOCK, kappa2, epsilon, m.opt_real(epsilon_spatial), H,
                 m.mask(mt), m.complex_t(psi), m.complex_t(dpsi), m.opt_real(abei), m.opt_real(ab),
                 m.real_t(dab), C)
        return _f64(m.gsum_v(C, grid, 17) if grid > 1 else C)[:17]


def reference_td(dtype, g, psi0, ab, mt, dt, warmup, steps, stop=1e-6, rand_t=1):
    """The reference's TD time loop at kappa = inf on its own kernels, driven as its
    host code drives them (``svirl/solvers/td.py:157-200,342-377``): per time step a
    device copy of psi into the right-hand side, then Jacobi sweeps, each preceded
    by zeroing the residual word and followed by reading it back (a 4-byte
    device-to-host copy, which synchronises), until ``1e-4*code < 1`` or 1024 sweeps;
    psi and psi_next swap after every sweep.  Buffers stay on the device.

    Returns the wall-clock seconds of ``steps`` steps after ``warmup`` untimed ones,
    the mean sweeps per timed step, and the mean device time of one sweep kernel
    (CUDA events around the timed steps' kernels)."""
    import time
    dt_ = np.dtype(dtype).type
    stop = max(float(stop), 1e-6 if dt_ is np.float32 else 1e-12)  # td.py:52-66
    m = RefModule.get(dt_, g.Nx, g.Ny, g.dx, g.dy, 5)
    torch = m.torch
    psi = m.complex_t(psi0)
    nxt = m.zeros_complex(g.N)
    rhs = m.zeros_complex(g.N)
    abd = m.real_t(ab)
    mtd = m.mask(mt)
    r2 = torch.zeros(1, dtype=torch.int32, device="cuda")
    grid = (g.N + BLOCK - 1) // BLOCK
    state = {"psi": psi, "nxt": nxt, "t": rand_t}
    ev = []

    def step(record):
        rhs.copy_(state["psi"])
        n = 0
        for j in range(1024):
            r2.zero_()
            if record:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
            m.launch("iterate_order_parameter_jacobi_step", grid, BLOCK, dt, 1.0, None, mtd, abd, rhs,
                     state["psi"], state["nxt"], 0.0, j, state["t"], stop, r2)
            if record:
                e1.record()
                ev.append((e0, e1))
            state["psi"], state["nxt"] = state["nxt"], state["psi"]
            n += 1
            if 1.0e-4 * dt_(int(r2.item())) < 1.0:
                break
        state["t"] = (state["t"] + 1) & 0xFFFFFFFF
        return n

    for _ in range(warmup):
        step(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sweeps = [step(True) for _ in range(steps)]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    kms = float(np.mean([a.elapsed_time(b) for a, b in ev])) if ev else 0.0
    return {"wall_s": wall, "steps": steps, "mean_sweeps": float(np.mean(sweeps)) if sweeps else 0.0,
            "sweep_kernel_ms": kms, "psi": state["psi"]}
