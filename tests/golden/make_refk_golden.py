"""Generate tests/golden/refk_*.npz: outputs of the reference's own CUDA kernels.

Runs on a machine with a GPU, after ``python -m oracle.ref_build`` has compiled
the reference's kernels (``svirl/cuda/*.h``) into ``oracle/_ref/`` where the
reference sources are mounted.  For every committed case fixture
(``case_*.npz``, ``fv_*.npz``: inputs made by the reference's host code) and for
the 129x129 plain workload, the oracle's host loops run on the reference's
kernels (``oracle.ref_gpu.RefKernels``) and the fixture keeps what those kernels
computed: free energy, B, j, js, dF/dpsi, dF/dA and the line-search coefficients
at the initial state; psi, A and the Jacobi sweep counts after TDGL; the CG
energies.  ``tests/test_golden_refk.py`` then checks the NumPy oracle against
them on the CPU, and ``tests/test_gpu_reference_kernels.py`` checks libglgpu.

    python tests/golden/make_refk_golden.py [out_dir]
"""
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import gl_oracle as O  # noqa: E402
from oracle import kernels_np as K  # noqa: E402
from oracle.ref_gpu import RefKernels  # noqa: E402

C1 = dict(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=5.0, sigma=200.0, H=0.1, seed=1, td_steps=50, cg_iters=20)
C1_INF = dict(Nx=129, Ny=129, dx=0.5, dy=0.5, kappa=np.inf, sigma=1.0, H=0.1, seed=2, td_steps=20, cg_iters=60)


WORKLOADS = {"c1_k5_129": C1, "c1_kinf_129": C1_INF}


def direction(g, seed):
    """The seeded line-search direction the coefficients are recorded for."""
    rng = np.random.default_rng(seed + 40)
    dpsi = rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N)
    return dpsi, 0.1 * rng.standard_normal(g.Nab)


def _opt(x):
    x = np.asarray(x)
    return None if x.size == 0 else x


def landau_ab(g, H):
    """A = (-H y, 0): a[i + Nxa*j] = -H * j * dy."""
    a = -H * np.repeat(np.arange(g.Nya) * g.dy, g.Nxa)
    return np.concatenate([a, np.zeros(g.Nb)])


def record(orc, R, dpsi=None, dab=None, td_steps=0, cg_iters=0, fv=False):
    g = orc.g
    out = {}
    f = (orc.kappa2, orc.epsilon, orc.epsilon_spatial, orc.H, orc.mt, orc.psi, orc.abei, orc.ab)
    out["F0"] = R.free_energy(g, *f)
    out["B0"] = R.magnetic_field(g, orc.abei, orc.ab)
    out["js0"] = R.supercurrent_density(g, orc.mt, orc.psi, orc.abei, orc.ab)
    out["gpsi0"] = R.free_energy_jacobian_psi(g, *f)
    if orc.solveA:
        out["j0"] = R.current_density(g, orc.kappa2, orc.H, orc.abei, orc.ab)
        out["gA0"] = R.free_energy_jacobian_A(g, orc.kappa2, orc.H, orc.mt, orc.psi, orc.abei, orc.ab)
    if dpsi is not None:
        if orc.solveA:
            out["coef"] = R.free_energy_conjgrad_coef_total(g, *f[:6], dpsi, orc.abei, orc.ab, dab)
        else:
            out["coef"] = R.free_energy_conjgrad_coef_psi_total(g, *f[:6], dpsi, orc.abei, orc.ab)
    if td_steps:
        orc.td(dt=0.1, Nt=td_steps)
        out["psi_td"], out["ab_td"] = orc.psi.copy(), orc.ab.copy()
        out["sweeps_psi"], out["sweeps_A"] = np.array(orc.sweeps_psi), np.array(orc.sweeps_A)
        out["F_td"] = orc.free_energy()
        if fv:
            out["vpi_td"] = orc.vpi.copy()
    if cg_iters:
        orc.cg(n_iter=cg_iters)
        out["cg_energies"] = np.array(orc.cg_energies)
        out["psi_cg"] = orc.psi.copy()
    return out


def case_oracle(d, kernels):
    return O.GLOracle(int(d["Nx"]), int(d["Ny"]), float(d["dx"]), float(d["dy"]), d["psi0"], d["ab0"],
                      mt=_opt(d["mt"]), abei=_opt(d["abei"]), kappa=float(d["kappa"]), sigma=float(d["sigma"]),
                      H=float(d["H"]), rand_t=int(d["seed"]), kernels=kernels,
                      vpi=_opt(d["ai0"]) if "ai0" in d.files else None,
                      lock_ns=_opt(d["lock"]) if "lock" in d.files else None)


def workload_oracle(spec, kernels):
    g = K.Grid(spec["Nx"], spec["Ny"], spec["dx"], spec["dy"])
    psi0 = O.random_order_parameter(g.N, 1.0, spec["seed"])
    return O.GLOracle(g.Nx, g.Ny, g.dx, g.dy, psi0, landau_ab(g, spec["H"]), kappa=spec["kappa"],
                      sigma=spec["sigma"], H=spec["H"], rand_t=spec["seed"], kernels=kernels)


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(out_dir, exist_ok=True)
    R = RefKernels(np.float64)
    for path in sorted(glob.glob(os.path.join(HERE, "case_*.npz")) + glob.glob(os.path.join(HERE, "fv_*.npz"))):
        d = np.load(path)
        name = os.path.basename(path)[:-4]
        fv = name.startswith("fv_")
        orc = case_oracle(d, R)
        steps = int(d["steps"][0]) if fv else int(d["td_steps"])
        rec = record(orc, R, None if fv else d["dpsi"], d["dab"] if "dab" in d.files else None,
                     td_steps=steps, cg_iters=0 if fv else int(d["cg_iters"]), fv=fv)
        np.savez_compressed(os.path.join(out_dir, "refk_%s.npz" % name), **rec)
        print("wrote refk_%s.npz" % name)
    for tag, spec in WORKLOADS.items():
        orc = workload_oracle(spec, R)
        dpsi, dab = direction(orc.g, spec["seed"])
        rec = record(orc, R, dpsi, dab, td_steps=spec["td_steps"], cg_iters=spec["cg_iters"])
        np.savez_compressed(os.path.join(out_dir, "refk_%s.npz" % tag), **rec)
        print("wrote refk_%s.npz" % tag)


if __name__ == "__main__":
    main()
