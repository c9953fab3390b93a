"""GLSolver argument checks, which run before any device work: the same
exception type as the reference's constructor (svirl/__init__.py:66-98) for
each invalid geometry or dtype.  The reference's own behaviour is read where its
sources are mounted; the expected types are also written out, so the test runs
without them."""
import os

import numpy as np
import pytest

INVALID = [
    (dict(Nx=3, Ny=8, dx=0.5, dy=0.5), AssertionError),            # Nx >= 4
    (dict(Nx=8, Ny=3, dx=0.5, dy=0.5), AssertionError),            # Ny >= 4
    (dict(Nx=8, Lx=5.0, dx=0.5, Ny=8, dy=0.5), AssertionError),   # Lx != dx (Nx - 1)
    (dict(Nx=8, Ny=8, dy=0.5), TypeError),                         # two of Nx, Lx, dx missing
    (dict(Nx=8, dx=0.5, Ly=4.0), TypeError),                       # two of Ny, Ly, dy missing
    (dict(Nx=8, Ny=8, dx=0.5, dy=0.5, dtype=np.float16), AssertionError),
    (dict(Nx=8, Ny=8, dx=-0.5, dy=0.5), AssertionError),           # Lx > 0
]


def _raised(fn):
    try:
        fn()
    except Exception as e:  # noqa: BLE001
        return type(e)
    return None


@pytest.mark.parametrize("kw,expected", INVALID)
def test_constructor_rejects_like_the_reference(kw, expected):
    from svirl_gb300 import GLSolver
    assert _raised(lambda: GLSolver(**kw)) is expected
    from tests import refshim
    from oracle.ref_build import reference_root
    if reference_root() is not None:  # the reference's own answer, where mounted
        assert _raised(lambda: refshim.load_reference().GLSolver(**kw)) is expected
