"""The multi-process oracle used by the bench's reference arm (oracle/parallel_np.py)
computes the single-process oracle's kappa = inf TD trajectory bitwise, with the
same Jacobi sweep counts, on a masked domain split into row blocks."""
import numpy as np

from oracle import gl_oracle as O
from oracle import kernels_np as K
from oracle.parallel_np import SharedTD, timed_steps


def _workload(Nx=37, Ny=29, seed=3):
    rng = np.random.default_rng(seed)
    g = K.Grid(Nx, Ny, 0.5, 0.5)
    psi = O.random_order_parameter(g.N, 1.0, seed)
    a = -0.2 * np.repeat(np.arange(Ny) * 0.5, Nx - 1)
    ab = np.concatenate([a, np.zeros(g.Nb)])
    mt = np.ones((Ny - 1, Nx - 1), dtype=bool)  # [j, i]
    mt[rng.integers(0, Ny - 1, 80), rng.integers(0, Nx - 1, 80)] = False
    return g, psi, ab, mt.reshape(-1)


def test_row_block_processes_match_single_process_oracle():
    g, psi, ab, mt = _workload()
    orc = O.GLOracle(g.Nx, g.Ny, g.dx, g.dy, psi, ab, mt=mt, kappa=np.inf, H=0.2)
    orc.td(dt=0.1, Nt=5)
    td = SharedTD(g.Nx, g.Ny, g.dx, g.dy, psi, ab, mt=mt, dt=0.1, processes=3)
    try:
        wall = timed_steps(td, 2, 3)
        assert wall > 0
        assert td.sweeps == orc.sweeps_psi
        assert np.array_equal(td.psi(), orc.psi)
    finally:
        td.close()
