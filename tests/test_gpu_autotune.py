"""The psi-sweep autotuner on a GPU: it measures every (kernel, strip height)
pair of an FP32 handle, applies the fastest, and the TDGL result of the tuned
handle is bitwise the default handle's."""
import numpy as np
import pytest

from tests._pairs import gpu_state, make_pair

pytestmark = pytest.mark.gpu


def test_tuned_handle_matches_default(tmp_path):
    from svirl_gb300 import autotune as AT
    path = str(tmp_path / "tune.json")
    gl, _ = make_pair(Nx=200, Ny=150, kappa=np.inf, H=0.2, mask="holes", seed=2, dtype=np.float32)
    ref, _ = make_pair(Nx=200, Ny=150, kappa=np.inf, H=0.2, mask="holes", seed=2, dtype=np.float32)
    c = AT.tune(gl._h, reps=3, path=path)
    assert not c["cached"] and len(c["measured"]) == 6 and min(c["measured"].values()) == c["us"] > 0
    assert gl._h.psi_strip_rows() == c["rows"]
    gl._h.td(0.1, 4, 0)
    ref._h.td(0.1, 4, 0)
    assert np.array_equal(gpu_state(gl)[0], gpu_state(ref)[0])
    again, _ = make_pair(Nx=200, Ny=150, kappa=np.inf, H=0.2, mask="none", seed=3, dtype=np.float32)
    assert AT.tune(again._h, path=path)["cached"]
