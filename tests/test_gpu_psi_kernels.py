"""The FP32 psi sweep's two kernels compute the same values bitwise: the
register-strip kernel (the default) and the bulk-copy kernel (inputs staged in
shared memory by TMA bulk copies, four strips per CTA).  Same TD states, same Jacobi
sweep counts, on domains at and around the strip and group widths (26 and 104
columns), with masks, Langevin noise and a spatial linear coefficient, in a single
handle and in a batch, through the graph and the host-driven loop."""
import numpy as np
import pytest

from tests._pairs import gpu_state, make_pair

pytestmark = pytest.mark.gpu


def _run(select, shape, mask, kappa, graphs=True, langevin=(0.0, 0.0), eps_field=False, rows=0):
    gl, _ = make_pair(Nx=shape[0], Ny=shape[1], kappa=kappa, sigma=50.0, H=0.2, mask=mask, seed=shape[0] + shape[1],
                      dtype=np.float32, langevin=langevin)
    if eps_field:
        x, y = gl.mesh.xy_grid
        gl.params.linear_coefficient = (1.0 - 0.3 * np.cos(0.7 * x) * np.sin(0.5 * y)).astype(np.float32)
    gl._h.set_psi_sweep_kernel(select)
    if rows:
        gl._h.set_psi_strip_rows(rows)
    gl._h.set_use_graphs(graphs)
    st = gl._h.td(0.1, 4, 0)
    psi, ab = gpu_state(gl)
    gl.close()
    return psi, ab, st.total_sweeps_psi, st.total_sweeps_A


@pytest.mark.parametrize("shape", [(4, 4), (27, 9), (105, 18), (131, 40), (235, 70), (300, 33)])
@pytest.mark.parametrize("mask", ["none", "holes"])
def test_bulk_and_register_kernels_agree_bitwise(shape, mask):
    for rows in (8, 17):
        a = _run(1, shape, mask, np.inf, rows=rows)
        b = _run(0, shape, mask, np.inf, rows=rows)
        assert np.array_equal(a[0], b[0]) and a[2] == b[2], (shape, rows)


@pytest.mark.parametrize("graphs", [True, False])
def test_bulk_kernel_with_langevin_spatial_eps_and_A(graphs):
    kw = dict(shape=(150, 61), mask="random30", kappa=3.0, graphs=graphs, langevin=(0.03, 0.01), eps_field=True)
    a = _run(1, **kw)
    b = _run(0, **kw)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2:] == b[2:]


def test_batch_matches_bulk_kernel_alone():
    from svirl_gb300.batch import HandleBatch
    shapes = [(64, 48), (130, 31), (27, 100)]
    pairs = [make_pair(Nx=s[0], Ny=s[1], kappa=np.inf, H=0.2, mask="holes", seed=q, dtype=np.float32)
             for q, s in enumerate(shapes)]
    alone = []
    for q, s in enumerate(shapes):
        gl, _ = make_pair(Nx=s[0], Ny=s[1], kappa=np.inf, H=0.2, mask="holes", seed=q, dtype=np.float32)
        gl._h.set_psi_sweep_kernel(1)
        gl._h.td(0.1, 5, 0)
        alone.append(gpu_state(gl)[0])
        gl.close()
    b = HandleBatch([gl._h for gl, _ in pairs])
    b.td_raw(0.1, 5, 0)
    b.close()
    for (gl, _), ref in zip(pairs, alone):
        assert np.array_equal(gpu_state(gl)[0], ref)
