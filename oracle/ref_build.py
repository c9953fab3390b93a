"""Recipe: compile the reference's own CUDA kernels into the checker under ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``svirl_gb300``) imports this
module or loads what it builds.

The reference compiles its kernels at run time (``svirl/parallel/startup.py:41-63``):
it concatenates ``svirl/cuda/{common,block_reduction,reduction,utils,observables,
td,cg}.h`` in that order, substitutes ``%(real)s``, ``%(complex)s``, ``%(Nx)s``,
``%(Ny)s``, ``%(dx)s``, ``%(dy)s`` and ``%(reduction_vector_length)s`` with Python's
``%`` operator (``dx``/``dy`` are ``cfg.dtype(dx)``, ``svirl/__init__.py:102``; the
vector length is 17 at finite kappa, 5 at kappa = inf), and hands the text to
pycuda's ``SourceModule`` with ``-std=c++11``, which wraps it in ``extern "C"``.
This recipe does the same, once per (dtype, geometry, vector length) in
``GEOMETRIES``, with our own ``oracle/refcuda/pycuda-complex.hpp`` standing in for
pycuda's header, and writes ``oracle/_ref/<name>.fatbin`` (sm_103a device code) plus
``oracle/_ref/manifest.json``.  It reads the reference sources where they lie and
copies nothing into the repository: ``oracle/_ref/`` is git-ignored.  The fatbins
are device code only, so one built on an x86 host loads on any host of the GPU.

    python -m oracle.ref_build [-v] [-f]

``reference_root()`` is the one place that names where the reference is mounted
(``$SVIRL_REFERENCE``, else the development container's mount point).
"""
import concurrent.futures as cf
import hashlib
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
INCLUDE = os.path.join(HERE, "refcuda")
FILES = ["common.h", "block_reduction.h", "reduction.h", "utils.h", "observables.h", "td.h", "cg.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (Nx, Ny, dx, dy): the golden cases, the default GPU parity geometry, two odd
# shapes, the 129^2 plain small workload and the 2049^2 large workload.
GEOMETRIES = [
    (12, 11, 0.5, 0.45),
    (10, 9, 0.5, 0.5),
    (13, 12, 0.5, 0.5),
    (14, 12, 0.5, 0.5),
    (33, 17, 0.5, 0.5),
    (40, 37, 0.4, 0.55),
    (129, 129, 0.5, 0.5),
    (2049, 2049, 0.5, 0.5),
]
DTYPES = (np.float64, np.float32)
VECTOR_LENGTHS = (5, 17)


def reference_root():
    """Directory holding the reference's ``svirl/`` package, or None."""
    for p in (os.environ.get("SVIRL_REFERENCE"), "/root/reference"):
        if p and os.path.isdir(os.path.join(p, "svirl", "cuda")):
            return p
    return None


def module_name(dtype, Nx, Ny, dx, dy, rvl):
    t = "f64" if np.dtype(dtype) == np.float64 else "f32"
    return "svirl_%s_%dx%d_%sx%s_v%d" % (t, Nx, Ny, str(np.dtype(dtype).type(dx)),
                                         str(np.dtype(dtype).type(dy)), rvl)


CN_MARK = "__global__ void iterate_order_parameter_jacobi_step_CN("


def live_cn(text):
    """The reference ships its Crank-Nicolson sweep commented out (``td.h:136-292``,
    every line prefixed with ``//``) and never launches it.  For the checker of
    this build's Crank-Nicolson option the recipe removes that prefix from the
    kernel's lines (from its signature to its closing brace) and changes nothing
    else, so the kernel compiles exactly as written: in the FP64 modules only, since
    as written it does not compile with real_t = float (it multiplies a
    complex<float> by a double, ``td.h:263``)."""
    lines = text.split("\n")
    out, inside = [], False
    for ln in lines:
        if not inside and ln.startswith("//") and CN_MARK in ln:
            inside = True
        if inside:
            body = ln[2:]
            body = body[1:] if body.startswith(" ") else body
            out.append(body)
            if body.rstrip() == "}":
                inside = False
        else:
            out.append(ln)
    return "\n".join(out)


def source(ref, dtype, Nx, Ny, dx, dy, rvl):
    """The text the reference hands to SourceModule (``startup.py:41-63``), wrapped
    in ``extern "C"`` as SourceModule does by default, with the commented-out
    Crank-Nicolson kernel made live (``live_cn``)."""
    dt = np.dtype(dtype).type
    template = ""
    for f in FILES:
        with open(os.path.join(ref, "svirl", "cuda", f)) as fh:
            text = fh.read()
            template += (live_cn(text) if f == "td.h" and dt is np.float64 else text) + "\n"
    subst = {
        "real": "float" if dt is np.float32 else "double",
        "complex": "pycuda::complex<float>" if dt is np.float32 else "pycuda::complex<double>",
        "Nx": np.int32(Nx), "Ny": np.int32(Ny),
        "dx": dt(dx), "dy": dt(dy),
        "reduction_vector_length": rvl,
    }
    return 'extern "C" {\n' + (template % subst) + "\n}\n"


def kernel_signatures(ref):
    """Argument kinds of every ``__global__`` function of the reference's source:
    r = real_t, p = pointer, i = int32_t, u = uint32_t (the launcher checks its own
    table against these before any launch)."""
    import re
    text = ""
    for f in FILES:
        with open(os.path.join(ref, "svirl", "cuda", f)) as fh:
            t = fh.read()
            text += (live_cn(t) if f == "td.h" else t) + "\n"
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    sigs = {}
    for m in re.finditer(r"__global__\s+void\s+(\w+)\s*\(([^)]*)\)", text):
        kinds = ""
        for a in m.group(2).split(","):
            a = a.strip()
            if not a:
                continue
            if "*" in a:
                kinds += "p"
            elif a.startswith("real_t"):
                kinds += "r"
            elif a.startswith("int32_t"):
                kinds += "i"
            elif a.startswith("uint32_t"):
                kinds += "u"
            else:
                raise ValueError("unknown argument type in %s: %r" % (m.group(1), a))
        sigs[m.group(1)] = kinds
    return sigs


def _nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src_text, out_path, verbose=False):
    tmp = out_path + ".cu"
    with open(tmp, "w") as fh:
        fh.write(src_text)
    cmd = [_nvcc()] + ARCH + ["-std=c++11", "-fatbin", "-I" + INCLUDE, "-o", out_path, tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    os.remove(tmp)
    if verbose or r.returncode:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode:
        raise RuntimeError("nvcc failed for " + os.path.basename(out_path))


def build(geometries=GEOMETRIES, dtypes=DTYPES, vector_lengths=VECTOR_LENGTHS, verbose=False, force=False):
    """Compile every module that is missing or stale; return the manifest dict.
    Returns None (and builds nothing) when the reference sources are absent."""
    ref = reference_root()
    if ref is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    hdr = open(os.path.join(INCLUDE, "pycuda-complex.hpp")).read()
    man_path = os.path.join(OUT, "manifest.json")
    old = {}
    if os.path.exists(man_path):
        with open(man_path) as fh:
            old = json.load(fh).get("modules", {})
    mods, jobs = {}, []
    for dtype in dtypes:
        for (Nx, Ny, dx, dy) in geometries:
            for rvl in vector_lengths:
                name = module_name(dtype, Nx, Ny, dx, dy, rvl)
                text = source(ref, dtype, Nx, Ny, dx, dy, rvl)
                digest = hashlib.sha256((text + hdr).encode()).hexdigest()[:16]
                path = os.path.join(OUT, name + ".fatbin")
                mods[name] = {"dtype": np.dtype(dtype).name, "Nx": Nx, "Ny": Ny, "dx": dx, "dy": dy,
                              "rvl": rvl, "sha": digest, "file": name + ".fatbin"}
                if force or not os.path.exists(path) or old.get(name, {}).get("sha") != digest:
                    jobs.append((text, path))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(lambda j: _compile(j[0], j[1], verbose), jobs))
    with open(man_path, "w") as fh:
        json.dump({"modules": mods, "files": FILES, "signatures": kernel_signatures(ref)}, fh, indent=1)
    return mods


if __name__ == "__main__":
    m = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print("reference sources not found" if m is None else "%d modules in %s" % (len(m), OUT))
