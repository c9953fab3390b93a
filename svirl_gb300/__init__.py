"""GB300-native (sm_103a) implementation of microsoft/svirl's 2D Ginzburg-Landau
hot path, behind svirl's ``GLSolver`` API.

    from svirl_gb300 import GLSolver
    gl = GLSolver(dx=0.5, dy=0.5, Lx=64, Ly=64, gl_parameter=5.0,
                  normal_conductivity=200.0, homogeneous_external_field=0.1)
    gl.solve.td(dt=0.1, Nt=1000)
    gl.solve.cg(n_iter=1000)
    vx, vy, vv = gl.vortex_detector.vortices

The numerics run in ``libglgpu.so`` (C ABI in ``include/glgpu.h``); there is no
CPU fallback.
"""
from .solver import GLSolver  # noqa: F401

__all__ = ["GLSolver"]
__version__ = "1.0.0"
