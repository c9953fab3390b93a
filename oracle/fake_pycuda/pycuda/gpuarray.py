"""``pycuda.gpuarray`` over NumPy (device memory = a flat host array)."""

import numpy as np


class _DevPtr:
    """Stands in for ``GPUArray.gpudata``: the device allocation."""

    def __init__(self, owner):
        self.owner = owner

    def free(self):
        pass


class GPUArray:
    def __init__(self, n, dtype, data=None):
        self.dtype = np.dtype(dtype)
        n = int(np.prod(n)) if isinstance(n, (tuple, list)) else int(n)
        if data is None:
            data = np.empty(n, dtype=self.dtype)
            if self.dtype.kind in "fc":
                data.fill(np.nan)  # unwritten device memory must never be read
        self._a = data
        self.gpudata = _DevPtr(self)

    @property
    def size(self):
        return self._a.size

    @property
    def shape(self):
        return self._a.shape

    @property
    def nbytes(self):
        return self._a.nbytes

    def get(self):
        return self._a.copy()

    def fill(self, value):
        self._a.fill(value)
        return self

    def copy(self):
        return GPUArray(self.size, self.dtype, self._a.copy())


def zeros(n, dtype=np.float64):
    a = GPUArray(n, dtype)
    a._a.fill(0)
    return a


def empty(n, dtype=np.float64):
    return GPUArray(n, dtype)


def zeros_like(other):
    return zeros(other.size, other.dtype)


def empty_like(other):
    return empty(other.size, other.dtype)


def to_gpu(arr):
    arr = np.asarray(arr)
    return GPUArray(arr.size, arr.dtype, arr.reshape(-1).copy())


def sum(a):
    return to_gpu(np.array([a._a.sum()], dtype=a.dtype))
