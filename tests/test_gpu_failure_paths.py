"""Failure paths of the device-side loops, exercised without faulting the GPU.

The Jacobi loops run on the device (a conditional CUDA graph, or a host loop that
reads the device's decision); each is bounded by a launch guard whose expiry is
reported as GLGPU_E_TIMEOUT (glgpu_set_loop_guard).  Here the guard is set to
two launches on a tiny grid, so it runs out in the first time step; the handle
must report the error, keep the state it had before the cut step, and then run
a normal TDGL that matches the oracle (1e-12, equal sweep counts).
"""
import numpy as np
import pytest

from svirl_gb300._lib import GLGPUError
from tests._pairs import gpu_state, make_pair, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("kappa", [np.inf, 4.0])
def test_loop_guard_reports_timeout_and_handle_recovers(graphs, kappa):
    gl, orc = make_pair(Nx=12, Ny=11, kappa=kappa, sigma=50.0, H=0.2, seed=3)
    gl._h.set_use_graphs(graphs)
    psi0, ab0 = gpu_state(gl)
    gl._h.set_loop_guard(2)
    with pytest.raises(GLGPUError, match="guard"):
        gl._h.td(0.1, 2, 0)
    psi1, ab1 = gpu_state(gl)
    assert np.array_equal(psi1, psi0) and np.array_equal(ab1, ab0)
    gl._h.set_loop_guard(0)
    st = gl._h.td(0.1, 3, 0)
    # the failed call advanced the Langevin counter by one per cut loop; without
    # noise it has no effect on the state
    orc.td(dt=0.1, Nt=3)
    psi, ab = gpu_state(gl)
    assert rel_err(psi, orc.psi) < 1e-12 and rel_err(ab, orc.ab) < 1e-12
    assert st.total_sweeps_psi == sum(orc.sweeps_psi)


def test_batch_loop_guard_reports_timeout():
    from svirl_gb300.batch import HandleBatch
    pairs = [make_pair(Nx=12 + k, Ny=11, kappa=np.inf, H=0.2, seed=k) for k in range(3)]
    b = HandleBatch([gl._h for gl, _ in pairs])
    b.set_loop_guard(2)
    with pytest.raises(GLGPUError, match="guard"):
        b.td_raw(0.1, 1)
    b.set_loop_guard(0)
    b.td_raw(0.1, 2)
    for gl, orc in pairs:
        orc.td(dt=0.1, Nt=2)
        psi, _ = gpu_state(gl)
        assert rel_err(psi, orc.psi) < 1e-12


def test_negative_guard_is_rejected():
    gl, _ = make_pair(Nx=8, Ny=8)
    with pytest.raises(GLGPUError):
        gl._h.set_loop_guard(-1)
