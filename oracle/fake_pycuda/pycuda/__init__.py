"""NumPy stand-in for the subset of pycuda that svirl's host code uses.

TEST INFRASTRUCTURE ONLY: it lets the reference's unmodified Python host code
(``svirl/solvers``, ``svirl/observables``, ...) run on a machine without a GPU,
with every CUDA kernel replaced by its NumPy restatement in
``oracle/kernels_np.py``.  The API surface is exactly what svirl calls
(gpuarray.{zeros,empty,zeros_like,empty_like,to_gpu,sum}; driver.{init,Device,
memcpy_dtod,memcpy_htod,memcpy_dtoh}; compiler.SourceModule.get_function).
"""
