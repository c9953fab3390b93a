"""The psi-sweep autotuner's choice and cache logic, on a stand-in handle (CPU):
the fastest measured (kernel, strip height) pair is applied and stored under its
key; a second handle with the same key takes it from the cache without timing;
FP64 handles only try the register-strip kernel; force=True measures again."""
import json

import numpy as np

from svirl_gb300 import autotune as AT


class FakeHandle:
    def __init__(self, dtype, Nx=200, Ny=150, finite=True, times=None):
        self.dtype = np.dtype(dtype)
        self.Nx, self.Ny = Nx, Ny
        self._finite = finite
        self.kernel, self.rows = 0, 0
        self.timed = 0
        self.times = times or {}

    def kappa_finite(self):
        return self._finite

    def set_psi_sweep_kernel(self, k):
        self.kernel = k

    def set_psi_strip_rows(self, r):
        self.rows = r

    def time_sweeps(self, which, reps):
        self.timed += 1
        return self.times.get((self.kernel, self.rows), 0.1)


def test_fastest_pair_applied_and_cached(tmp_path):
    path = str(tmp_path / "tune.json")
    h = FakeHandle(np.float32, times={(0, 12): 0.05, (1, 8): 0.07})
    c = AT.tune(h, path=path)
    assert (c["kernel"], c["rows"], c["cached"]) == (0, 12, False)
    assert (h.kernel, h.rows) == (0, 12)
    assert len(c["measured"]) == len(AT.KERNELS_FP32) * len(AT.STRIP_ROWS)
    table = json.load(open(path))
    assert AT.key_of(h) in table and table[AT.key_of(h)]["rows"] == 12
    h2 = FakeHandle(np.float32, times={(1, 17): 0.01})
    c2 = AT.tune(h2, path=path)
    assert c2["cached"] and h2.timed == 0 and (h2.kernel, h2.rows) == (0, 12)
    c3 = AT.tune(h2, path=path, force=True)
    assert not c3["cached"] and (c3["kernel"], c3["rows"]) == (1, 17)


def test_fp64_tries_register_kernel_only_and_keys_differ(tmp_path):
    path = str(tmp_path / "tune.json")
    h = FakeHandle(np.float64, finite=False, times={(0, 8): 0.02})
    c = AT.tune(h, path=path)
    assert set(k.split("/")[0] for k in c["measured"]) == {"0"} and c["rows"] == 8
    assert AT.key_of(h) != AT.key_of(FakeHandle(np.float64, finite=True))
