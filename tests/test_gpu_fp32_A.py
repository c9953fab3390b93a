"""FP32 TDGL at finite kappa where |A| is large: the A Jacobi loop must converge.

The reference's A loop stops when max |A^(k+1) - A^(k)| < 1e-6 (absolute,
svirl/solvers/td.py:53-57, td.h:408-462).  Iterated in FP32, A's iterates keep
differing by a unit in the last place once |A| > 8 (the Landau gauge reaches
H*Ly), so that rule is never met and every step runs to the 1024-sweep cap.  The
FP32 path iterates the offset from the step's start instead (k_A_sweep), the same
fixed-point iteration and stop quantity.  Here: kappa = 4, H = 0.3, 257^2 nodes
(|A| up to 38), 8 TD steps from the same start in FP32 and FP64.  Required: the
FP32 A loop takes at most twice the FP64 sweeps per step (far below the cap), and
the FP32 state stays within max |dpsi| <= 1e-3 and max |dA| <= 1e-5 max |A| of
the FP64 one (printed)."""
import numpy as np
import pytest

from tests._pairs import gpu_state, make_pair

pytestmark = pytest.mark.gpu


def _run(dtype, nt=8):
    gl, _ = make_pair(Nx=257, Ny=257, dx=0.5, dy=0.5, kappa=4.0, sigma=200.0, H=0.3, mask="holes", seed=5,
                      landau=True, dtype=dtype)
    st = gl._h.td(0.1, nt, 0)
    psi, ab = gpu_state(gl)
    gl.close()
    return psi, ab, st


def test_fp32_A_loop_converges_and_tracks_fp64():
    p32, a32, s32 = _run(np.float32)
    p64, a64, s64 = _run(np.float64)
    dpsi = float(np.max(np.abs(p32 - p64)))
    dA = float(np.max(np.abs(a32 - a64)))
    print("FP32 vs FP64 after 8 steps: |dpsi| %.2e, |dA| %.2e (max |A| %.1f); A sweeps per step FP32 %.1f, "
          "FP64 %.1f; psi sweeps FP32 %d, FP64 %d" % (dpsi, dA, np.max(np.abs(a64)), s32.total_sweeps_A / 8,
                                                     s64.total_sweeps_A / 8, s32.total_sweeps_psi,
                                                     s64.total_sweeps_psi))
    assert np.max(np.abs(a64)) > 30.0
    assert s32.max_sweeps_A < 1024 and s32.total_sweeps_A <= 2 * s64.total_sweeps_A
    assert dpsi <= 1e-3 and dA <= 1e-5 * np.max(np.abs(a64))
