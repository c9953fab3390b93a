"""Benchmark: TDGL node-steps/s on the large single-domain workload.

Workload (the metric's large single-domain configuration): Nx = Ny = 2049
(Lx = Ly = 1024, dx = dy = 0.5), kappa = inf (A fixed in the Landau gauge
Ax = -H*y, Ay = 0, H = 0.05), material tiling with circular holes of radius 4
at seeded uniform positions covering >= 5% of the cells, random order parameter
(seeded), TDGL dt = 0.1.  A step is one TDGL time step (one backward-Euler
Jacobi solve) of the whole domain.  Synthetic, seeded inputs.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--dtype fp32|fp64] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun each rank runs an independent
replica on its own GPU (the single domain is not decomposed across GPUs).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SIDE = 2049
DX = 0.5
H_FIELD = 0.05
DT = 0.1
HOLE_R = 4.0
HOLE_FRAC = 0.05
METRIC = "TDGL node-steps/s (2049x2049, kappa=inf, 5% holes, dt=0.1)"


def holes_mask(n_side, dx, radius, frac, seed):
    """Cells (Nxc x Nyc, [i, j]) outside circular holes at uniform positions,
    holes added until at least `frac` of the cells are removed."""
    nc = n_side - 1
    L = dx * (n_side - 1)
    mt = np.ones((nc, nc), dtype=bool)
    rng = np.random.default_rng(seed)
    xc = (np.arange(nc) + 0.5) * dx
    r_cells = int(np.ceil(radius / dx)) + 1
    removed = 0
    target = frac * nc * nc
    while removed < target:
        cx, cy = rng.random(2) * L
        i0, j0 = int(cx / dx), int(cy / dx)
        i_lo, i_hi = max(0, i0 - r_cells), min(nc, i0 + r_cells + 1)
        j_lo, j_hi = max(0, j0 - r_cells), min(nc, j0 + r_cells + 1)
        sub = (xc[i_lo:i_hi, None] - cx) ** 2 + (xc[None, j_lo:j_hi] - cy) ** 2 < radius * radius
        before = mt[i_lo:i_hi, j_lo:j_hi].sum()
        mt[i_lo:i_hi, j_lo:j_hi] &= ~sub
        removed += before - mt[i_lo:i_hi, j_lo:j_hi].sum()
    return mt


def make_solver(n_side=N_SIDE, dtype=np.float32, seed=0, device=0, kappa=np.inf):
    """The workload's solver; a finite `kappa` (normal conductivity 200) adds the
    vector-potential equation (used to profile the A sweep on the same domain)."""
    from svirl_gb300 import GLSolver
    mt = holes_mask(n_side, DX, HOLE_R, HOLE_FRAC, seed)
    gl = GLSolver(Nx=n_side, Ny=n_side, dx=DX, dy=DX, order_parameter="random", random_seed=seed,
                  gl_parameter=kappa, normal_conductivity=200.0, homogeneous_external_field=H_FIELD,
                  material_tiling=mt, dtype=dtype, device_id=device)
    ya = gl.mesh.xy_a_grid[1]
    gl.vars.vector_potential = ((-H_FIELD * ya).astype(dtype), np.zeros((n_side, n_side - 1), dtype=dtype))
    return gl


def fp32_errors(g32, g64):
    """Every result of a solver pair that ran the same steps in FP32 and FP64:
    max |x32 - x64| and max |x64| of psi, A, the magnetic field B, the current
    density j and the supercurrent density js, and the relative free-energy
    difference."""
    def pair(get):
        a, b = get(g32), get(g64)
        a = np.concatenate([np.ravel(x) for x in a]) if isinstance(a, tuple) else np.ravel(a)
        b = np.concatenate([np.ravel(x) for x in b]) if isinstance(b, tuple) else np.ravel(b)
        return {"max_abs_err": float(np.max(np.abs(a.astype(b.dtype) - b))), "max_abs": float(np.max(np.abs(b)))}
    out = {"psi": pair(lambda g: g.vars.order_parameter), "A": pair(lambda g: g.vars.vector_potential),
           "B": pair(lambda g: g.observables.magnetic_field), "j": pair(lambda g: g.observables.current_density),
           "js": pair(lambda g: g.observables.supercurrent_density)}
    f32, f64 = float(g32.observables.free_energy), float(g64.observables.free_energy)
    out["F"] = {"rel_err": abs(f32 - f64) / abs(f64), "F64": f64}
    return out


def precision_check(n_side, steps=20, seed=0):
    """FP32 against FP64 on the same workload: the same initial state (the FP64
    state rounded to FP32), `steps` TD steps each; the errors of every result
    after them (fp32_errors), plus the summary keys of earlier lines."""
    g32 = make_solver(n_side, np.float32, seed=seed)
    g64 = make_solver(n_side, np.float64, seed=seed)
    try:
        g32.solve.td(dt=DT, Nt=steps)
        g64.solve.td(dt=DT, Nt=steps)
        err = fp32_errors(g32, g64)
    finally:
        g32.close()
        g64.close()
    return {"steps": steps, "max_abs_dpsi": err["psi"]["max_abs_err"], "max_abs_psi": err["psi"]["max_abs"],
            "rel_dF": err["F"]["rel_err"], "per_result": err}


def make_oracle(n_side, seed=0):
    """The same workload for the CPU oracle (FP64), on an n_side x n_side domain."""
    from oracle import gl_oracle as O
    from oracle import kernels_np as K
    mt = holes_mask(n_side, DX, HOLE_R, HOLE_FRAC, seed)
    g = K.Grid(n_side, n_side, DX, DX)
    psi = O.random_order_parameter(g.N, 1.0, seed)
    nm = O.node_mask(g, O.flatten_ij(mt)).reshape(-1)
    ya = np.linspace(0.0, DX * (n_side - 1), n_side)
    a = np.repeat((-H_FIELD * ya)[:, None], n_side - 1, axis=1).reshape(-1)  # a[j, i] = -H y_j
    ab = np.concatenate([a, np.zeros(g.Nb)])
    del nm
    return O.GLOracle(n_side, n_side, DX, DX, psi, ab, mt=O.flatten_ij(mt), kappa=np.inf, H=H_FIELD, rand_t=seed)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r.strip().split(",") for r in self.tmp.read().strip().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, name in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------

def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(dtype_name, fuse, rows):
    """DRAM bytes per psi-sweep launch from the committed ncu summary of the same
    kernel build (same sweeps per launch and strip height), or None."""
    p = os.path.join(ROOT, "profiles", "psi_sweep_%s_2049.md" % dtype_name)
    if not os.path.exists(p):
        return None
    vals = {}
    for line in open(p):
        if ":" in line and line.split(":", 1)[0] in ("traffic_bytes_per_launch", "sweeps_per_launch", "strip_rows"):
            k, v = line.split(":", 1)
            try:
                vals[k] = float(v.strip())
            except ValueError:
                return None
    if int(vals.get("sweeps_per_launch", 1)) != fuse or int(vals.get("strip_rows", 0)) != rows:
        return None
    return vals.get("traffic_bytes_per_launch")


def cpu_baseline(mean_sweeps, budget_s=20.0, n_side=N_SIDE):
    """The oracle (NumPy FP64, one thread) on the same 2049^2 workload, bounded: psi
    Jacobi sweeps of the workload's state for about `budget_s` seconds.  A TD step
    is a number of such sweeps (the stop rule decides how many; the GPU run
    measured `mean_sweeps` per step over its timed steps), so the oracle's
    node-steps/s = its node-sweeps/s / mean_sweeps."""
    from oracle import kernels_np as K
    orc = make_oracle(n_side, seed=0)
    rhs = orc.psi.copy()
    cur = orc.psi
    t0 = time.perf_counter()
    sweeps = 0
    while time.perf_counter() - t0 < budget_s:
        cur, _ = K.iterate_order_parameter_jacobi_step(orc.g, DT, 1.0, None, orc.mt, orc.ab, rhs, cur, 0.0,
                                                       sweeps, 1, 1e-6)
        sweeps += 1
    dt = time.perf_counter() - t0
    node_sweeps = n_side * n_side * sweeps / dt
    return {"value": node_sweeps / mean_sweeps, "unit": "node-steps/s", "cores": 1, "kind": "port",
            "node_sweeps_per_s": node_sweeps,
            "sample": "oracle (NumPy FP64, 1 thread) on the same %dx%d domain: %d psi Jacobi sweeps in %.1f s, "
                      "per step %.2f sweeps (the GPU run's mean over its timed steps)"
                      % (n_side, n_side, sweeps, dt, mean_sweeps)}


def run_reference(args):
    """The reference's computation on the host cores.  The reference has no CPU
    implementation of this path (its kernels are CUDA only), so its arithmetic is
    timed through the oracle (NumPy FP64 restatement of its kernels and host
    loop), on the same 2049^2 workload and trajectory as the GPU run: one domain
    split into row blocks over all host cores (oracle/parallel_np.py, bitwise the
    single-process result), `warmup` untimed TD steps, then `steps` timed ones
    (steps warmup+1 .. warmup+steps, as the GPU run times); value = nodes x steps /
    wall time of the timed steps.  A run stays within a few minutes: at most 20
    warm-up and 100 timed steps (about 0.8 s each on 16 cores) are run, a bounded
    sample of the GPU run's steps; the line states the sample and its mean sweeps
    per step, and node-sweeps/s beside node-steps/s."""
    from oracle.parallel_np import SharedTD, timed_steps
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = len(os.sched_getaffinity(0))
    orc = make_oracle(N_SIDE, seed=0)
    td = SharedTD(N_SIDE, N_SIDE, DX, DX, orc.psi, orc.ab, mt=orc.mt, dt=DT, processes=cores)
    del orc
    warm, steps = min(args.warmup, 20), min(args.steps, 100)
    try:
        wall = timed_steps(td, warm, steps)
        sweeps = td.sweeps[warm:]
    finally:
        td.close()
    value = N_SIDE * N_SIDE * steps / wall
    line = {"metric": METRIC, "value": value, "unit": "node-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": "tdgl_2049_kinf_holes5", "Nx": N_SIDE, "Ny": N_SIDE, "same_config": True,
                       "processes": td.P, "mean_sweeps_per_step": float(np.mean(sweeps)),
                       "timed_steps": steps, "warmup_steps": warm,
                       "node_sweeps_per_s": N_SIDE * N_SIDE * float(np.sum(sweeps)) / wall},
            "cpu_baseline": {"value": value, "unit": "node-steps/s", "cores": td.P, "kind": "port",
                             "sample": "the whole %dx%d workload (seed 0), one trajectory, %d untimed then %d timed "
                                       "TD steps (steps %d..%d; at most 20 + 100 of the requested %d + %d); NumPy "
                                       "FP64 oracle split into %d row blocks, one process per core"
                                       % (N_SIDE, N_SIDE, warm, steps, warm + 1, warm + steps, args.warmup,
                                          args.steps, td.P)},
            "e2e": {"value": value, "unit": "node-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    try:
        line["reference_kernels_gb300"] = reference_kernels_gpu(args)
    except Exception as e:  # noqa: BLE001 - an extra measurement; the line prints regardless
        line["reference_kernels_gb300"] = {"unavailable": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(line), flush=True)


def reference_kernels_gpu(args, dtype=np.float32):
    """The reference's own CUDA kernels (svirl/cuda/*.h compiled unchanged into
    oracle/_ref) on this GPU, driven the way its host code drives them
    (oracle.ref_gpu.reference_td): the same workload, `warmup` then `steps` TD steps."""
    import torch
    from oracle import ref_gpu
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    orc = make_oracle(N_SIDE, seed=0)
    r = ref_gpu.reference_td(dtype, orc.g, orc.psi, orc.ab, orc.mt, DT, args.warmup, min(args.steps, 50))
    N = N_SIDE * N_SIDE
    return {"value": N * r["steps"] / r["wall_s"], "unit": "node-steps/s", "dtype": "f32",
            "ms_per_step": 1e3 * r["wall_s"] / r["steps"], "mean_sweeps_per_step": r["mean_sweeps"],
            "sweep_kernel_ms": r["sweep_kernel_ms"], "steps": r["steps"],
            "how": "svirl's iterate_order_parameter_jacobi_step compiled unchanged for sm_103a, launched as "
                   "svirl/solvers/td.py:157-200 does (per sweep: zero the residual word, launch ceil(N/128) "
                   "blocks of 128, read the word back); wall clock around the timed steps"}


# ---------------------------------------------------------------------------
# states/s: relaxed GL states per second, batched device CG vs the plain solver
# ---------------------------------------------------------------------------

STATES_METRIC = "GL states/s to dF/F<=1e-6 (batched FP32 device CG vs plain single-instance FP64 CG)"
STATE_SIZES = (129, 193, 257, 385, 513)  # Lx = Ly in {64, 96, 128, 192, 256}, dx = 0.5


def states_instances(count, first_seed=1000):
    """Instance k: its own generator default_rng(first_seed + k): size, H ~ U[0.02, 0.5], kappa = 4,
    hole fraction U[0, 0.05] with radii U[2, 6], random psi (seeded)."""
    from svirl_gb300 import learned as L
    out = []
    for k in range(count):
        rng = np.random.default_rng(first_seed + k)
        n = STATE_SIZES[int(rng.integers(len(STATE_SIZES)))]
        out.append(L.Instance.sample(n, rng, H_range=(0.02, 0.5), kappa_range=(4.0, 4.0), hole_frac=(0.0, 0.05),
                                     radius=(2.0, 6.0)))
    return out


def states_instances_bounded(count, max_side, first_seed=1000):
    """The first `count` instances of the field sweep (instance k drawn exactly as
    states_instances draws it) whose side is at most `max_side`."""
    from svirl_gb300 import learned as L
    out, k = [], 0
    while len(out) < count:
        rng = np.random.default_rng(first_seed + k)
        n = STATE_SIZES[int(rng.integers(len(STATE_SIZES)))]
        if n <= max_side:
            out.append(L.Instance.sample(n, rng, H_range=(0.02, 0.5), kappa_range=(4.0, 4.0), hole_frac=(0.0, 0.05),
                                         radius=(2.0, 6.0)))
        k += 1
    return out


def measure_states(insts, cg_iters, gtol, plain_sample, fp64_arm=True):
    """The batched pipeline (FP32 stencils, FP64 reductions, exact-boundary gradient,
    device-decided steps) on `insts`, timed with its loads and fetches, against F*
    from a tight FP64 relaxation of the same instances from the same start (untimed);
    the plain single-instance CG (one instance at a time, FP64, the same device CG and
    stop rule) timed on the first `plain_sample` instances.  A state counts when
    |F - F*|/|F*| <= 1e-6 (`value`, `speedup_vs_plain`); under the strict criterion
    (`strict`) it must also meet the absolute gradient tolerance, evaluated in FP64
    on the fetched state.  An FP32 state cannot meet it (the gradient of its own
    rounding is above 1e-4), so with `fp64_arm` the same batched CG also runs in FP64
    (timed), the batched arm for the strict criterion."""
    from svirl_gb300 import relax as RX
    cache = RX.HandleCache()
    strict = {}
    try:
        # warm-up: a few small instances through the same path
        RX.relax(states_instances(4, first_seed=1), cache, np.float32, n_iter=50, gtol=1e-3)
        t0 = time.perf_counter()
        out, states, _ = RX.relax(insts, cache, np.float32, n_iter=cg_iters, gtol=gtol)
        wall = time.perf_counter() - t0
        ref, _, _ = RX.relax(insts, cache, np.float64, n_iter=2 * cg_iters, gtol=gtol * 1e-2, fetch=False)
        Estar = ref["energy"]

        def criteria(sts, idx=None):
            ii = np.arange(len(insts)) if idx is None else np.asarray(idx)
            its = [insts[q] for q in ii]
            E = RX.energies_fp64(its, sts, cache)
            rel = (E - Estar[ii]) / np.abs(Estar[ii])
            e_ok = np.abs(rel) <= 1e-6
            g_ok = RX.gradient_ok_fp64(its, sts, cache, gtol)
            return rel, e_ok, g_ok

        rel, ok, gok = criteria(states)
        value = float(ok.sum()) / wall
        strict["fp32_batched"] = {"states_ok": int((ok & gok).sum()), "gradient_ok": int(gok.sum()),
                                  "states_per_s": float((ok & gok).sum()) / wall}
        if fp64_arm:
            t0 = time.perf_counter()
            out64, states64, _ = RX.relax(insts, cache, np.float64, n_iter=cg_iters, gtol=gtol)
            wall64 = time.perf_counter() - t0
            _, ok64, gok64 = criteria(states64)
            strict["fp64_batched"] = {"states_ok": int((ok64 & gok64).sum()), "energy_ok": int(ok64.sum()),
                                      "wall_s": wall64, "states_per_s": float((ok64 & gok64).sum()) / wall64,
                                      "cg_iters_median": float(np.median(out64["iters"]))}
        sample = insts[:plain_sample]
        t_plain, ok_plain, ok_plain_g = 0.0, 0, 0
        for q, it in enumerate(sample):
            t1 = time.perf_counter()
            o1, st1, _ = RX.relax([it], cache, np.float64, n_iter=cg_iters, gtol=gtol)
            t_plain += time.perf_counter() - t1
            _, e1, g1 = criteria(st1, [q])
            ok_plain += int(e1[0])
            ok_plain_g += int(e1[0] and g1[0])
    finally:
        cache.close()
    plain_rate = ok_plain / t_plain if t_plain > 0 else 0.0
    plain_strict = ok_plain_g / t_plain if t_plain > 0 else 0.0
    strict["plain"] = {"states_ok": ok_plain_g, "states_per_s": plain_strict}
    for k in ("fp32_batched", "fp64_batched"):
        if k in strict:
            strict[k]["speedup_vs_plain"] = strict[k]["states_per_s"] / plain_strict if plain_strict > 0 else None
    strict["criterion"] = ("|F - F*|/|F*| <= 1e-6 and |grad F| <= %g (absolute, exact-boundary gradient, evaluated "
                           "in FP64 on the fetched state)" % gtol)
    return {"value": value, "wall_s": wall, "states_ok": int(ok.sum()), "instances": len(insts),
            "states_lower_energy": int((rel < -1e-6).sum()),
            "rel_err_quantiles": np.quantile(rel, [0, 0.5, 0.9, 1]).tolist(),
            "cg_device_ms": out["ms"], "cg_iters": {"mean": float(out["iters"].mean()), "max": int(out["iters"].max())},
            "plain": {"states_per_s": plain_rate, "sample": len(sample), "met_criterion": ok_plain, "wall_s": t_plain,
                      "how": "the same device CG on one instance at a time, FP64, no batching"},
            "speedup_vs_plain": value / plain_rate if plain_rate > 0 else None,
            "strict": strict,
            "h2d_bytes": int(sum(it.n * it.n * 4 * 4 for it in insts))}


STATES_CRITERION = ("|F - F*|/|F*| <= 1e-6, F* = FP64 relaxation of the same instance from the same start "
                    "(gradient tolerance gtol/100, twice the iteration cap)")


def run_states(args):
    """States/s of the batched field sweep (`args.instances` instances) against the
    plain single-instance CG (measure_states)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    insts = states_instances(args.instances)
    nodes = sum(it.n * it.n for it in insts)
    m = measure_states(insts, args.cg_iters, args.gtol, args.plain_sample, fp64_arm=args.states_fp64_arm)
    value = m["value"]
    line = {"metric": STATES_METRIC, "value": value, "unit": "states/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * m["wall_s"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 stencils, f64 reductions", "data": "synthetic (seeded)",
            "config": {"workload": "batched_field_sweep", "instances": len(insts), "sizes": list(STATE_SIZES),
                       "kappa": 4.0, "H": "U[0.02,0.5]", "holes": "fraction U[0,0.05], radius U[2,6]",
                       "nodes_total": nodes, "cg_iters_cap": args.cg_iters, "gtol_abs": args.gtol,
                       "criterion": STATES_CRITERION},
            "states_ok": m["states_ok"], "states_lower_energy": m["states_lower_energy"], "strict": m["strict"],
            "rel_err_quantiles": m["rel_err_quantiles"], "cg_device_ms": m["cg_device_ms"], "cg_iters": m["cg_iters"],
            "plain": m["plain"], "speedup_vs_plain": m["speedup_vs_plain"],
            "e2e": {"value": value, "unit": "states/s", "h2d_bytes_per_step": m["h2d_bytes"],
                    "d2h_bytes_per_step": m["h2d_bytes"],
                    "how": "wall time of load (H2D) + batched CG + fetch (D2H) of every instance"}}
    print(json.dumps(line), flush=True)


def states_sample_line(count=48, max_side=257, cg_iters=12000, gtol=1e-4, plain_sample=8):
    """A bounded sample of the states/s comparison for the default bench line: the
    first `count` instances of the field sweep with side <= `max_side` (the larger
    sides take minutes in the FP64 validation), the field sweep's cap and stop rule."""
    insts = states_instances_bounded(count, max_side)
    m = measure_states(insts, cg_iters, gtol, plain_sample)
    m.update({"metric": STATES_METRIC, "unit": "states/s", "criterion": STATES_CRITERION,
              "sample": "the first %d instances of the seeded field sweep with side <= %d (sides %s), cap %d, "
                        "absolute gradient %g" % (count, max_side, sorted({it.n for it in insts}), cg_iters, gtol)})
    return m


def run_cg(args):
    """Batched device CG iterations of the field sweep's first `instances`
    instances (FP32 stencils, FP64 reductions, exact-boundary gradient), `steps`
    iterations from the random start with every stop test off: device time per
    iteration and node-iterations/s.  Algorithmic bytes per node-iteration (FP32):
    gradient (read psi 8, A 8, write g 16), direction and line-search sums (read g
    16, previous direction 16, psi 8, A 8, write the direction 16), update and
    energy (read psi 8, A 8, direction 16, write psi 8, A 8) = 144 B."""
    from svirl_gb300 import relax as RX
    if int(os.environ.get("RANK", "0")) != 0:
        return
    insts = states_instances(args.instances)
    nodes = sum(it.n * it.n for it in insts)
    cache = RX.HandleCache()
    RX.relax(insts, cache, np.float32, n_iter=max(args.warmup, 3), gtol=0.0, fetch=False, graphs=not args.no_graphs)
    out, _, _ = RX.relax(insts, cache, np.float32, n_iter=args.steps, gtol=0.0, fetch=False, graphs=not args.no_graphs)
    cache.close()
    ms_it = out["ms"] / args.steps
    peak, peak_kind = peaks()
    alg = nodes * 144 / (ms_it * 1e-3) / 1e9
    line = {"metric": "batched CG node-iterations/s (FP32, field sweep)", "value": nodes / (ms_it * 1e-3),
            "unit": "node-iterations/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms_it, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 stencils, f64 reductions", "data": "synthetic (seeded)",
            "config": {"workload": "batched_cg_iterations", "instances": len(insts), "nodes_total": nodes,
                       "graphs": not args.no_graphs},
            "roofline": {"bound": "hbm", "achieved": alg, "peak": peak, "unit": "GB/s", "frac": alg / peak,
                         "bytes_per_node_iteration": 144, "peak_kind": peak_kind, "traffic": None}}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Poisson-arriving requests (mean 200/s), n ~ U{64..512}, kappa finite or inf,
    fp32 or fp64, TDGL 500 steps then CG; throughput and latency percentiles."""
    from svirl_gb300 import serve as S
    if int(os.environ.get("RANK", "0")) != 0:
        return
    reqs = S.poisson_requests(args.requests, 200.0, seed=7)
    warm = S.Engine(td_steps=10, td_chunk=10, cg_chunk=50, cg_cap=100)
    warm.run(S.poisson_requests(4, 1000.0, seed=1, sizes=(64, 96)), max_wall_s=60)
    warm.close()
    eng = S.Engine(td_steps=500)
    done, wall = eng.run(reqs, max_wall_s=args.serve_seconds)
    summ = S.summarize(done, wall)
    eng.close()
    line = {"metric": "GL solve requests/s (serving loop)", "value": summ["throughput_per_s"], "unit": "requests/s",
            "n_gpus": 1, "steps": len(done), "warmup": 1, "ms_per_step": 1e3 * wall / max(len(done), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 mix",
            "data": "synthetic (seeded)",
            "config": {"workload": "serving", "arrivals": "Poisson, mean 200/s", "requests_offered": len(reqs),
                       "sizes": "U{64..512}^2", "kappa": "U[2,10] or inf (50/50)", "dtype": "fp32/fp64 (50/50)",
                       "td_steps": 500, "cg": "energy ratio < 1e-6, cap 4000", "wall_limit_s": args.serve_seconds},
            "latency_s": summ["latency_s"], "completed": summ["completed"], "mean_cg_iters": summ["mean_cg_iters"]}
    print(json.dumps(line), flush=True)


def run_c1(args):
    """The plain small configuration: 129x129 (Lx = Ly = 64, dx = dy = 0.5), FP64,
    kappa = 5, sigma = 200, H = 0.1, A in the Landau gauge, full domain, seeded
    random psi; td(dt=0.1, Nt=1000) then cg(n_iter=1000) through GLSolver (the
    reference's API and decisions); the oracle times the same TD on one core."""
    from svirl_gb300 import GLSolver
    if int(os.environ.get("RANK", "0")) != 0:
        return

    def c1_solver(dtype):
        g = GLSolver(dx=0.5, dy=0.5, Lx=64, Ly=64, order_parameter="random", random_seed=0, gl_parameter=5.0,
                     normal_conductivity=200.0, homogeneous_external_field=0.1, dtype=dtype)
        ya = g.mesh.xy_a_grid[1]
        g.vars.vector_potential = ((-0.1 * ya).astype(dtype), np.zeros((129, 128), dtype=dtype))
        return g

    # FP32 against FP64 from the same start after the same TD steps and CG (untimed)
    g32, g64 = c1_solver(np.float32), c1_solver(np.float64)
    g32.solve.td(dt=0.1, Nt=args.steps)
    g64.solve.td(dt=0.1, Nt=args.steps)
    prec = {"after_td_steps": args.steps, "td": fp32_errors(g32, g64)}
    g32.solve.cg(n_iter=200)
    g64.solve.cg(n_iter=200)
    prec["after_cg_200"] = fp32_errors(g32, g64)
    g32.close()
    g64.close()
    gl = c1_solver(np.float64)
    gl.solve.td(dt=0.1, Nt=5)  # warm-up: graph build
    st, ms = gl._h.td_timed(0.1, args.steps, 0)
    t0 = time.perf_counter()
    gl.solve.cg(n_iter=1000)
    t_cg = time.perf_counter() - t0
    n_cg = len(gl.solve._cg.cg_energies)
    N = 129 * 129
    value = N * args.steps / (ms * 1e-3)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import gl_oracle as O
        psi, ab = gl._h.get_psi().astype(np.complex128), gl._h.get_ab().astype(np.float64)
        orc = O.GLOracle(129, 129, 0.5, 0.5, psi, ab, kappa=5.0, sigma=200.0, H=0.1)
        t1 = time.perf_counter()
        k = 0
        while time.perf_counter() - t1 < 20.0:
            orc.td(dt=0.1, Nt=1)
            k += 1
        tc = time.perf_counter() - t1
        cpu = {"value": N * k / tc, "unit": "node-steps/s", "cores": 1, "kind": "port",
               "sample": "oracle (NumPy FP64, 1 thread), %d TD steps of the same 129x129 state" % k}
    line = {"metric": "TDGL node-steps/s (129x129, kappa=5, FP64) and CG wall time", "value": value,
            "unit": "node-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": 5, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": "plain_small_129", "kappa": 5.0, "sigma": 200.0, "H": 0.1, "gauge": "Landau",
                       "mean_sweeps_psi": st.total_sweeps_psi / args.steps,
                       "mean_sweeps_A": st.total_sweeps_A / args.steps},
            "cg": {"iterations": n_cg, "wall_s": t_cg, "ms_per_iteration": 1e3 * t_cg / max(n_cg, 1),
                   "how": "GLSolver.solve.cg(n_iter=1000): GPU phases, step length on the host (reference decisions)"},
            "fp32_vs_fp64": prec,
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def run_conv(args):
    """The learned warm start's hottest kernels on a 32 x 128 x 128 x 64 -> 64 layer,
    timed with CUDA events: the tcgen05 3x3 convolution forward (TMA operands; the
    value) and its backward as the library's autograd wrapper runs it (dy masked once
    by the ReLU derivative, the data gradient and the weight gradient from the masked
    dy, TMA operands), beside the thread-gather forward and data gradient and the
    mma.sync weight gradient; FLOP rate against the measured bf16 peak."""
    import ctypes as C
    import torch
    from svirl_gb300 import learned as L
    if int(os.environ.get("RANK", "0")) != 0:
        return
    lib = L._lib_nn()
    n, h, w, cin, cout = 32, 128, 128, 64, 64
    g = torch.Generator(device="cpu").manual_seed(0)
    x = torch.randn((n, h, w, cin), generator=g).to("cuda", torch.bfloat16)
    W = (0.05 * torch.randn((cout, 3, 3, cin), generator=g)).cuda()
    b = torch.zeros(cout, device="cuda")
    wb = torch.empty(W.shape, dtype=torch.bfloat16, device="cuda")
    wt = torch.empty((3, 3, cin, cout), dtype=torch.bfloat16, device="cuda")
    y = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    dy = torch.randn((n, h, w, cout), generator=g).to("cuda", torch.bfloat16)
    dym = torch.empty_like(dy)
    dx = torch.empty_like(x)
    dw = torch.empty_like(W)
    db = torch.empty_like(b)
    nwork = int(lib.glnn_conv3x3_bwd_weight_work(n, h, w, cin, cout))
    work = torch.empty(nwork, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = L._stream()
    P = L._ptr
    assert lib.glnn_prep_weights(P(W), P(wb), P(wt), cout, cin, s) == 0
    flop = 2.0 * n * h * w * 9 * cin * cout

    def timed(fn, reps):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    f = lambda: lib.glnn_conv3x3_fwd(P(x), cin, None, 0, P(wb), P(b), P(y), n, h, w, cout, 1, P(err), s)
    mk = lambda: lib.glnn_relu_mask(P(dy), P(y), P(dym), dy.numel(), s)
    bd_gather = lambda: lib.glnn_conv3x3_bwd_data(P(dy), P(y), 1, P(wt), P(dx), cin, None, 0, n, h, w, cout, P(err), s)
    bd = lambda: lib.glnn_conv3x3_bwd_data(P(dym), None, 0, P(wt), P(dx), cin, None, 0, n, h, w, cout, P(err), s)
    bw = lambda: lib.glnn_conv3x3_bwd_weight(P(dym), None, 0, P(x), cin, None, 0, P(dw), P(db), P(work), nwork, n, h,
                                            w, cout, P(err), s)
    f(); mk()
    lib.glnn_set_conv_tma(0)
    ms_f_gather = timed(f, args.steps)
    ms_d_gather = timed(bd_gather, args.steps)
    ms_w_mma = timed(bw, args.steps)
    lib.glnn_set_conv_tma(1)
    ms_f_tile, ms_d_tile = timed(f, args.steps), timed(bd, args.steps)
    lib.glnn_set_conv_tma(2)
    ms_f, ms_mk, ms_d, ms_w = timed(f, args.steps), timed(mk, args.steps), timed(bd, args.steps), timed(bw, args.steps)
    assert int(err.item()) == 0
    peak = 1922.0
    pth = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pth):
        peak = float(json.load(open(pth))["bf16_tflops"])
    tf = flop / (ms_f * 1e-3) / 1e12
    line = {"metric": "3x3 conv TFLOP/s (tcgen05 forward with TMA operands, persistent CTAs, 32x128x128x64->64, bf16 in, fp32 accumulate)",
            "value": tf,
            "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": 3, "ms_per_step": ms_f,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic (seeded)",
            "config": {"workload": "conv3x3_layer", "n": n, "h": h, "w": w, "cin": cin, "cout": cout},
            "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                         "peak_kind": "measured bf16 burst"},
            "forward_gather": {"ms": ms_f_gather, "tflops": flop / (ms_f_gather * 1e-3) / 1e12,
                               "kernel": "tcgen05, operands gathered by the threads"},
            "forward_tma_per_tile": {"ms": ms_f_tile, "tflops": flop / (ms_f_tile * 1e-3) / 1e12,
                                     "kernel": "tcgen05, TMA operands, one output tile per CTA"},
            "data_grad_tma_per_tile": {"ms": ms_d_tile, "tflops": flop / (ms_d_tile * 1e-3) / 1e12},
            "relu_mask": {"ms": ms_mk, "kernel": "dy * relu'(y), once per backward"},
            "data_grad": {"ms": ms_d, "tflops": flop / (ms_d * 1e-3) / 1e12,
                          "kernel": "tcgen05, operands loaded by TMA (masked dy)"},
            "data_grad_gather": {"ms": ms_d_gather, "tflops": flop / (ms_d_gather * 1e-3) / 1e12,
                                 "kernel": "tcgen05, operands gathered by the threads (ReLU derivative while gathering)"},
            "weight_grad": {"ms": ms_w, "tflops": flop / (ms_w * 1e-3) / 1e12,
                            "kernel": "tcgen05, MN-major operands loaded by TMA, split-K (with the bias gradient)"},
            "weight_grad_mma": {"ms": ms_w_mma, "tflops": flop / (ms_w_mma * 1e-3) / 1e12, "kernel": "mma.sync"},
            "layer_fwd_bwd_ms": ms_f + ms_mk + ms_d + ms_w}
    print(json.dumps(line), flush=True)


def run_learned(args):
    """Learned CG warm start: relaxed 128^2 states generated by the batched device CG
    (kappa ~ U[2, 10], H ~ U[0.02, 0.5], hole masks), the network trained on them by
    the library's BF16 kernels; then, on held-out instances at 128^2 and 256^2,
    (1) relaxed states/s of the learned + batched method (prediction, batched FP32
    device CG) against the plain single-instance FP64 CG from the random start, one
    stop rule and one criterion for both (`learned.states_throughput`), and
    (2) CG iterations to F* within 1e-6 from the random start and from the
    prediction (`learned.evaluate`)."""
    import torch
    from svirl_gb300 import learned as L
    from svirl_gb300.relax import HandleCache
    if int(os.environ.get("RANK", "0")) != 0:
        return
    t0 = time.perf_counter()
    x, y, _ = L.generate(args.train_states, n=128, seed=0, pool_size=256, n_iter=3000, gtol=1e-4)
    t_gen = time.perf_counter() - t0
    net = L.WarmStartNet(seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = L.train(net, x, y, epochs=args.epochs, batch=32, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    steps = args.epochs * (x.shape[0] // 32)
    del x, y
    evals, thr = {}, {}
    for n, count in ((128, 64), (256, 24)):
        rng = np.random.default_rng(777 + n)
        insts = [L.Instance.sample(n, rng) for _ in range(count)]
        cache = HandleCache()
        try:
            Estar = L.reference_energies(insts, cache)  # untimed validation
            thr["%d" % n] = L.states_throughput(net, insts, Estar, cache, cap=args.learned_cap, gtol=args.gtol,
                                                plain_sample=args.plain_sample)
            evals["%d" % n] = L.evaluate(net, insts, cache=cache, Estar=Estar)
        finally:
            cache.close()
    t = thr["128"]["by_dtype"]["float32"]
    nodes = 128 * 128 * 64
    line = {"metric": "GL states/s to dF/F<=1e-6, learned warm start + batched FP32 CG (128^2, 64 instances)",
            "value": t["states_per_s"], "unit": "states/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * t["wall_s"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 net (f32 accumulate), f32 CG stencils, f64 reductions (the f64 CG arm under "
                     "throughput.*.by_dtype.float64)",
            "data": "synthetic (solver-generated)",
            "config": {"workload": "learned_warm_start", "train_states": args.train_states, "epochs": args.epochs,
                       "params": net.n_params(), "levels": list(L.LEVELS), "target_mode": "amplitude",
                       "train_loss_first_last": [hist[0], hist[-1]], "gen_s": t_gen, "train_s": t_train,
                       "cg_cap": args.learned_cap, "gtol_abs": args.gtol, "plain": thr["128"]["plain"],
                       "criterion": "|F - F*|/|F*| <= 1e-6, F* = FP64 relaxation (gradient norm 1e-7, 20000 "
                                    "iterations) of the same instance from the same initial state: the random start "
                                    "(plain arm), the prediction (learned arm)"},
            "speedup_vs_plain": t["speedup_vs_plain"], "throughput": thr, "eval": evals,
            "e2e": {"value": t["states_per_s"], "unit": "states/s", "h2d_bytes_per_step": nodes * 8 * 2,
                    "d2h_bytes_per_step": nodes * 4 * 4,
                    "how": "wall time of features to the device, prediction, decoding to host, states into the "
                           "handles, batched CG, states back"}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--dtype", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=N_SIDE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kappa", type=float, default=float("inf"),
                    help="GL parameter of the TDGL workload (inf: the headline workload; finite: adds the A step)")
    ap.add_argument("--psi-kernel", type=int, choices=[0, 1], default=None,
                    help="FP32 psi sweep kernel (0 register strip, 1 bulk-copy ring); default: the autotuner's choice")
    ap.add_argument("--no-graphs", action="store_true",
                    help="host-driven Jacobi loop (same kernels); ncu cannot profile kernels inside conditional graphs")
    ap.add_argument("--workload", choices=["tdgl", "states", "serve", "learned", "c1", "conv", "cg"], default="tdgl",
                    help="tdgl: node-steps/s on the 2049^2 domain; states: relaxed states/s of a batched sweep; "
                         "serve: the serving loop; learned: the learned CG warm start")
    ap.add_argument("--train-states", type=int, default=20000)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--cg-iters", type=int, default=12000)
    ap.add_argument("--gtol", type=float, default=1e-4)
    ap.add_argument("--plain-sample", type=int, default=8)
    ap.add_argument("--states-fp64-arm", action="store_true",
                    help="--workload states: also time the batched CG in FP64 (for the strict criterion)")
    ap.add_argument("--no-states-sample", action="store_true",
                    help="leave out the bounded states/s sample of the default line")
    ap.add_argument("--learned-cap", type=int, default=4000,
                    help="CG iteration cap of both arms of the learned + batched states/s comparison")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "states":
        run_states(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload == "learned":
        run_learned(args)
        return
    if args.workload == "c1":
        run_c1(args)
        return
    if args.workload == "conv":
        run_conv(args)
        return
    if args.workload == "cg":
        run_cg(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    dtype = np.float32 if args.dtype == "fp32" else np.float64
    kinf = not np.isfinite(args.kappa)
    gl = make_solver(args.size, dtype=dtype, seed=rank, device=local, kappa=args.kappa)
    h = gl._h
    # the psi sweep's launch shape: measured (or read from the tuning cache),
    # or the kernel forced by --psi-kernel (at the model's strip height)
    from svirl_gb300 import autotune
    if args.psi_kernel is None:
        tuned = autotune.tune(h)
    else:
        h.set_psi_sweep_kernel(args.psi_kernel)
        tuned = {"kernel": args.psi_kernel, "rows": h.psi_strip_rows(), "cached": False, "measured": None}
    if args.no_graphs:
        h.set_use_graphs(False)
    N = args.size * args.size
    h.td(DT, args.warmup, 0)

    def barrier():
        if dist is not None:
            dist.barrier()

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    st, ms = h.td_timed(DT, args.steps, 0)
    clk = clocks.stop()
    barrier()
    if dist is not None:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    sweeps = int(st.total_sweeps_psi)
    value = world * N * args.steps / (ms * 1e-3)

    # roofline of the dominant kernel (the psi Jacobi sweep), timed alone.  One
    # launch does `fuse` sweeps.  Algorithmic bytes per node-sweep: read psi^(k),
    # the right-hand side and two link values of A, write psi^(k+1) (32 B FP32,
    # 64 B FP64), +1 B for the material mask.
    fuse = int(h.lib.glgpu_psi_sweeps_per_launch())
    rows = int(h.lib.glgpu_psi_strip_rows(h.h))
    sweep_ms = h.time_sweeps(0, 20)
    bytes_per_node_sweep = (32 if dtype == np.float32 else 64) + 1
    alg_bytes = N * bytes_per_node_sweep * fuse
    peak, peak_kind = peaks()
    achieved = alg_bytes / (sweep_ms * 1e-3) / 1e9
    # finite kappa: the A sweep timed alone as well (pairs of sweeps 0 and 1, L2
    # flushed before each pair); algorithmic bytes per node-sweep: psi, the
    # right-hand side, the supercurrent argument, A^(k), the write (8 B each in FP32,
    # 16 B in FP64, two links per node), +1 B mask
    a_sweep = None
    if not kinf:
        a_ms = h.time_sweeps(1, 10)
        a_bytes = (40 if dtype == np.float32 else 80) + 1
        a_gbs = N * a_bytes / (a_ms * 1e-3) / 1e9
        a_sweep = {"kernel": "k_A_sweep", "launch_ms": a_ms, "bytes_per_node_sweep": a_bytes,
                   "achieved_GBps": a_gbs, "frac": a_gbs / peak}

    # end to end through the C ABI with pinned host buffers: H2D psi, one TD step, D2H psi
    import torch
    ctype = np.complex64 if dtype == np.float32 else np.complex128
    pin_in = torch.empty(2 * N, dtype=torch.float32 if dtype == np.float32 else torch.float64, pin_memory=True)
    pin_out = torch.empty_like(pin_in).pin_memory()
    psi_in = pin_in.numpy().view(ctype)
    psi_out = pin_out.numpy().view(ctype)
    psi_in[:] = h.get_psi()
    e2e_steps = max(10, min(args.steps // 10, 200))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h.set_psi(psi_in)
        h.td(DT, 1, 0)
        out = h.lib.glgpu_get_order_parameter(h.h, psi_out.ctypes.data_as(__import__("ctypes").c_void_p))
        assert out == 0
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_value = world * N * e2e_steps / e2e_s
    # where the end-to-end step's time goes: the same three calls timed apart
    t_parts = [0.0, 0.0, 0.0]
    dev_ms = 0.0
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        h.set_psi(psi_in)
        t2 = time.perf_counter()
        dev_ms += h.td_timed(DT, 1, 0)[1]
        t3 = time.perf_counter()
        assert h.lib.glgpu_get_order_parameter(h.h, psi_out.ctypes.data_as(__import__("ctypes").c_void_p)) == 0
        t4 = time.perf_counter()
        t_parts[0] += t2 - t1
        t_parts[1] += t3 - t2
        t_parts[2] += t4 - t3
    e2e_parts = {"h2d_ms": 1e3 * t_parts[0] / e2e_steps, "td_step_ms": 1e3 * t_parts[1] / e2e_steps,
                 "td_step_graph_ms": dev_ms / e2e_steps,
                 "d2h_ms": 1e3 * t_parts[2] / e2e_steps,
                 "h2d_GBps": psi_in.nbytes / (t_parts[0] / e2e_steps) / 1e9,
                 "d2h_GBps": psi_out.nbytes / (t_parts[2] / e2e_steps) / 1e9}

    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline(sweeps / args.steps)
        prec = None
        if dtype == np.float32 and not args.no_cpu_baseline and kinf:
            try:  # a side measurement: the bench line prints whatever happens here
                prec = precision_check(args.size)
            except Exception as e:  # noqa: BLE001
                prec = {"error": "%s: %s" % (type(e).__name__, e)}
        # sweep launches counted on the device, plus per step the link table, the
        # loop begin/end and step-end kernels, plus the final copy and reset
        launches = int(st.sweep_launches) + 4 * args.steps + 3
        line = {
            "metric": METRIC if kinf else METRIC.replace("kappa=inf", "kappa=%g" % args.kappa),
            "value": value, "unit": "node-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if dtype == np.float32 else "f64", "data": "synthetic (seeded)",
            "config": {"workload": "tdgl_2049_kinf_holes5" if kinf else "tdgl_2049_k%g_holes5" % args.kappa,
                       "Nx": args.size, "Ny": args.size, "dx": DX,
                       "kappa": "inf" if kinf else args.kappa, "H": H_FIELD, "dt": DT, "hole_radius": HOLE_R, "hole_fraction": HOLE_FRAC,
                       "parallelism": "replica per GPU" if world > 1 else "single GPU",
                       "l2": "working set %.0f MB > 129 MB L2 (no flush between steps); sweep timing flushes L2"
                             % (N * (3 * (8 if dtype == np.float32 else 16) + (8 if dtype == np.float32 else 16)) / 1e6),
                       "mean_sweeps_per_step": sweeps / args.steps,
                       "mean_A_sweeps_per_step": st.total_sweeps_A / args.steps,
                       "psi_sweep_shape": {"kernel": ["register strip", "bulk-copy ring"][tuned["kernel"]],
                                           "strip_rows": tuned["rows"], "from_cache": tuned["cached"],
                                           "measured_us": tuned["measured"]}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": ncu_traffic(args.dtype, fuse, rows) if tuned["kernel"] == 0 else None,
                         "kernel": "k_psi_sweep" if tuned["kernel"] == 0 else "k_psi_sweep_bulk",
                         "sweeps_per_launch": fuse, "strip_rows": rows,
                         "bytes_per_node_sweep": bytes_per_node_sweep, "bytes_per_launch": alg_bytes,
                         "launch_ms": sweep_ms, "peak_kind": peak_kind},
            "e2e": {"value": e2e_value, "unit": "node-steps/s",
                    "h2d_bytes_per_step": int(psi_in.nbytes), "d2h_bytes_per_step": int(psi_out.nbytes),
                    "how": "per step: H2D psi from pinned memory, glgpu_td (1 step), D2H psi, via the C ABI",
                    "parts": e2e_parts},
            "gpu_launches": launches,
            "clocks": clk,
            "cpu_baseline": cpu,
            "fp32_vs_fp64": prec,
        }
        if a_sweep is not None:
            line["A_sweep"] = a_sweep
        if dtype == np.float32 and kinf and not args.no_states_sample:
            try:  # a side measurement after the timed region, like fp32_vs_fp64
                line["states_sample"] = states_sample_line()
            except Exception as e:  # noqa: BLE001
                line["states_sample"] = {"error": "%s: %s" % (type(e).__name__, e)}
        print(json.dumps(line), flush=True)
    gl.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
