"""Load the reference package (microsoft/svirl) on top of the NumPy pycuda shim.

Only usable where the reference sources are mounted (the development
container).  Tests that need it skip elsewhere.
"""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_reference():
    from oracle.ref_build import reference_root
    REF = reference_root()
    if REF is None:
        pytest.skip("reference sources not mounted")
    sys.dont_write_bytecode = True
    shim = os.path.join(ROOT, "oracle", "fake_pycuda")
    for p in (shim, REF):
        if p not in sys.path:
            sys.path.insert(0, p)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        svirl = importlib.import_module("svirl")
    return svirl
