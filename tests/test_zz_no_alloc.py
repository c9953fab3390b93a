"""glgpu_free_energy_noalloc: the free energy of a caller-owned device state,
computed without the library allocating anything (its reduction scratch is a
static device array).  It exists for callers that cannot let a library call
cudaMalloc, e.g. a host whose own allocator or fixed pre-sized arena owns all
device memory.  Checked through the C ABI against the handle-based
glgpu_free_energy and against the oracle's energy of the same state, on two
calls in a row (the shared scratch keeps the previous call's contents), in FP64
and FP32; the second call must leave the device's free memory unchanged; plus
the size limit.  Kept in its own file, collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, against the handle path (the same kernel), as the FP64 observable parity tests
# relative, against the oracle's FP64 energy of the same stored state: FP64 as the
# parity tests; FP32 accumulates each node in FP32 (double-float partial sums)
ORACLE_TOL = {np.float64: 1e-12, np.float32: 1e-5}


def _state(dtype):
    from svirl_gb300 import GLSolver
    rng = np.random.default_rng(4)
    mt = np.ones((66, 52), dtype=bool)
    mt[rng.integers(0, 66, 400), rng.integers(0, 52, 400)] = False
    gl = GLSolver(Nx=67, Ny=53, dx=0.5, dy=0.45, order_parameter="random", random_seed=2, gl_parameter=3.0,
                  normal_conductivity=100.0, homogeneous_external_field=0.2, material_tiling=mt,
                  external_field=0.05, dtype=dtype)
    gl.solve.td(dt=0.1, Nt=3)
    return gl


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_noalloc_free_energy_matches_handle_path(dtype):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from svirl_gb300 import _lib
    lib = _lib.load()
    gl = _state(dtype)
    ref = gl.observables.free_energy
    h = gl._h
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    psi = torch.from_numpy(h.get_psi().view(dtype).copy()).to("cuda")
    ab = torch.from_numpy(h.get_ab().copy()).to("cuda")
    ev = gl.params.external_vector_potential
    abei = torch.from_numpy(np.concatenate([np.reshape(ev[0].T, -1), np.reshape(ev[1].T, -1)]).astype(dtype)).to("cuda")
    mt = torch.from_numpy(np.reshape(gl.mesh.material_tiling.T, -1).astype(np.uint8)).to("cuda")
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    assert psi.dtype == tdt
    grid = _lib.Grid(int(gl.cfg.Nx), int(gl.cfg.Ny), float(gl.cfg.dx), float(gl.cfg.dy), 8 if dtype == np.float64 else 4)
    params = h.get_params()
    # the oracle's energy of the same state (FP64 arithmetic on the stored values)
    from oracle import kernels_np as K
    g = K.Grid(int(gl.cfg.Nx), int(gl.cfg.Ny), float(gl.cfg.dx), float(gl.cfg.dy))
    E_orc = K.free_energy(g, float(params.kappa) ** 2, float(params.epsilon), None, float(params.H),
                          np.reshape(gl.mesh.material_tiling.T, -1), h.get_psi().astype(np.complex128),
                          abei.cpu().numpy().astype(np.float64), h.get_ab().astype(np.float64))
    free_after_first = None
    for call in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.glgpu_free_energy_noalloc(C.byref(grid), C.byref(params), C.c_void_p(psi.data_ptr()),
                                           C.c_void_p(ab.data_ptr()), C.c_void_p(abei.data_ptr()),
                                           C.c_void_p(mt.data_ptr()), C.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.glgpu_last_error(None)
        torch.cuda.synchronize()
        E = float(out.item())
        assert abs(E - ref) <= TOL * abs(ref), (E, ref)
        assert abs(E - E_orc) <= ORACLE_TOL[dtype] * abs(E_orc), (E, E_orc)
        if call == 0:
            # the first call may load the kernel's code (lazy module loading);
            # from then on the call takes no device memory
            free_after_first = torch.cuda.mem_get_info()[0]
    assert torch.cuda.mem_get_info()[0] == free_after_first


def test_noalloc_rejects_grids_beyond_its_scratch():
    from svirl_gb300 import _lib
    lib = _lib.load()
    grid = _lib.Grid(3000, 3000, 0.5, 0.5, 8)
    params = _lib.Params(float("inf"), 1.0, 1.0, 0.1, 1e-6, 1e-6, 0.0, 0.0, 1, 0)
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.glgpu_free_energy_noalloc(C.byref(grid), C.byref(params), one, one, None, None, one, None)
    assert rc == _lib.GLGPU_E_ARG
    assert b"maximum" in lib.glgpu_last_error(None)
