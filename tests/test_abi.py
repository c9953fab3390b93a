"""The C-ABI library builds, loads without a GPU, and exports every entry point
declared in include/glgpu.h and include/glgpu_nn.h; the Python binding
declares them all."""
import ctypes
import os
import re

from svirl_gb300 import _lib
from svirl_gb300 import build as B

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
HEADERS = [os.path.join(INCLUDE, f) for f in ("glgpu.h", "glgpu_nn.h")]


def declared_symbols():
    syms = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        syms |= set(re.findall(r"\b((?:glgpu|glnn)_[a-z0-9_]+)\s*\(", text))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "glgpu_create" in syms and "glgpu_td" in syms and "glgpu_cg_update" in syms
    assert "glnn_conv3x3_fwd" in syms and "glnn_adam" in syms
    assert len(syms) >= 40


def test_library_loads_and_exports_every_declared_symbol():
    path = B.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_symbols()) <= set(_lib._SIGNATURES)


def test_version_and_error_string_without_gpu():
    lib = _lib.load()
    assert lib.glgpu_version() >= 10000
    # a bad argument is rejected on the host, before any CUDA call
    g = _lib.Grid(3, 10, 0.5, 0.5, 8)
    h = ctypes.c_void_p()
    rc = lib.glgpu_create(ctypes.byref(g), 0, ctypes.byref(h))
    assert rc == _lib.GLGPU_E_ARG
    assert b">= 4" in lib.glgpu_last_error(None)
    g = _lib.Grid(8, 8, 0.5, 0.5, 3)
    assert lib.glgpu_create(ctypes.byref(g), 0, ctypes.byref(h)) == _lib.GLGPU_E_ARG
