"""Generate the golden fixtures of tests/golden/ (run in a checkout where the
reference sources are available; the fixtures are committed, the GPU tests only
read them).

For each case the unmodified reference (microsoft/svirl's host code) runs on the
NumPy pycuda shim (oracle/fake_pycuda) from its own seeded initial state: the
fixture keeps the inputs (psi0, A0, mask, external vector potential, parameters)
and the reference's outputs (free energy, B, j, js, dF/dpsi, dF/dA and the 5/17
line-search coefficients for a seeded direction at the initial state; psi, A and
the Jacobi sweep counts after TDGL; the CG energies and state after a few
iterations; the vortex list of the final state).  The oracle recomputes every
output from the inputs and must agree before a fixture is written.

    python tests/golden/make_golden.py [reference_dir]      (GOLDEN_ONLY=cases|fv|api: one group)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import gl_oracle as O  # noqa: E402

CASES = {
    # name: (Nx, Ny, dx, dy, kappa, sigma, H, external_field, mask_kind, seed, td_steps, cg_iters)
    "k5_full": (12, 11, 0.5, 0.45, 5.0, 200.0, 0.1, 0.0, "none", 1, 6, 6),
    "k2_random_ext": (10, 9, 0.5, 0.5, 2.0, 10.0, 0.3, 0.05, "random30", 2, 5, 5),
    "kinf_holes": (13, 12, 0.5, 0.5, np.inf, 1.0, 0.2, 0.0, "holes", 3, 6, 8),
}


def mask_of(kind, nxc, nyc, rng):
    if kind == "none":
        return None
    mt = np.ones((nxc, nyc), dtype=bool)
    if kind == "random30":
        k = int(0.3 * nxc * nyc)
        mt[rng.integers(0, nxc, k), rng.integers(0, nyc, k)] = False
    elif kind == "holes":
        mt[2:5, 3:6] = False
        mt[nxc - 4:nxc - 2, 1:3] = False
    return mt


def flat(x):
    return O.flatten_ij(np.asarray(x))


def close(x, y, tol):
    x, y = np.asarray(x), np.asarray(y)
    return np.max(np.abs(x - y)) <= tol * max(np.max(np.abs(y)), 1e-300)


def make_case(svirl, name, spec):
    Nx, Ny, dx, dy, kappa, sigma, H, ext, kind, seed, nt, ncg = spec
    rng = np.random.default_rng(100 + seed)
    mt = mask_of(kind, Nx - 1, Ny - 1, rng)
    kw = dict(Nx=Nx, Ny=Ny, dx=dx, dy=dy, order_parameter="random", random_seed=seed, gl_parameter=kappa,
              normal_conductivity=sigma, homogeneous_external_field=H)
    if mt is not None:
        kw["material_tiling"] = mt
    if ext:
        kw["external_field"] = ext
    gl = svirl.GLSolver(**kw)
    psi0 = flat(gl.vars.order_parameter)
    a, b = gl.vars.vector_potential
    ab0 = np.concatenate([flat(a), flat(b)])
    ei = gl.params.external_irregular_vector_potential
    abei = None if ei is None else np.concatenate([flat(ei[0]), flat(ei[1])])
    orc = O.GLOracle(Nx, Ny, dx, dy, psi0, ab0, mt=None if mt is None else flat(mt), abei=abei, kappa=kappa,
                     sigma=sigma, H=H, rand_t=seed)
    out = {"Nx": Nx, "Ny": Ny, "dx": dx, "dy": dy, "kappa": kappa, "sigma": sigma, "H": H, "ext": ext, "seed": seed,
           "td_steps": nt, "cg_iters": ncg, "psi0": psi0, "ab0": ab0,
           "mt": np.zeros(0, bool) if mt is None else flat(mt), "abei": np.zeros(0) if abei is None else abei}
    # observables, gradients and coefficients at the initial state
    out["F0"] = gl.observables.free_energy
    out["B0"] = flat(gl.observables.magnetic_field)
    jx, jy = gl.observables.current_density
    out["j0"] = np.concatenate([flat(jx), flat(jy)])
    sx, sy = gl.observables.supercurrent_density
    out["js0"] = np.concatenate([flat(sx), flat(sy)])
    gl.solve._init_cg()
    out["gpsi0"] = np.asarray(gl.solve._cg._free_energy_jacobian_psi.get()).reshape(-1)
    drng = np.random.default_rng(7 + seed)
    dpsi = drng.standard_normal(Nx * Ny) + 1j * drng.standard_normal(Nx * Ny)
    out["dpsi"] = dpsi
    if np.isfinite(kappa):
        out["gA0"] = np.asarray(gl.solve._cg._free_energy_jacobian_A.get()).reshape(-1)
        dab = 0.1 * drng.standard_normal(orc.g.Nab)
        out["dab"] = dab
        out["coef"] = np.asarray(orc.coef(dpsi, dab))
        ref_c = np.asarray(gl.solve._cg._free_energy_conjgrad_coef(svirl_gpu(dpsi), svirl_gpu(dab)))
        ref_c = np.concatenate([ref_c[0, :], ref_c[1, :], ref_c[2, :], [ref_c[3, 0], ref_c[4, 0]]])
        assert close(out["coef"], ref_c, 1e-12), name
    else:
        out["coef"] = np.asarray(orc.coef_psi(dpsi))
        ref_c = np.asarray(gl.solve._cg._free_energy_conjgrad_coef_psi(svirl_gpu(dpsi)))
        assert close(out["coef"], ref_c, 1e-12), name
    assert abs(orc.free_energy() - out["F0"]) <= 1e-13 * abs(out["F0"]), name
    assert close(orc.magnetic_field(), out["B0"], 1e-12) and close(orc.current_density(), out["j0"], 1e-12)
    assert close(orc.supercurrent_density(), out["js0"], 1e-12) and close(orc.jacobian_psi(), out["gpsi0"], 1e-12)
    if np.isfinite(kappa):
        assert close(orc.jacobian_A(), out["gA0"], 1e-12), name
    # TDGL
    gl.solve.td(dt=0.1, Nt=nt)
    orc.td(dt=0.1, Nt=nt)
    out["psi_td"] = flat(gl.vars.order_parameter)
    a, b = gl.vars.vector_potential
    out["ab_td"] = np.concatenate([flat(a), flat(b)])
    out["sweeps_psi"] = np.array(orc.sweeps_psi)
    out["sweeps_A"] = np.array(getattr(orc, "sweeps_A", []))
    assert close(orc.psi, out["psi_td"], 1e-13) and close(orc.ab, out["ab_td"], 1e-13), name
    # CG
    gl.solve.cg(n_iter=ncg)
    orc.cg(n_iter=ncg)
    out["cg_energies"] = np.array(gl.solve._cg.cg_energies)
    out["psi_cg"] = flat(gl.vars.order_parameter)
    a, b = gl.vars.vector_potential
    out["ab_cg"] = np.concatenate([flat(a), flat(b)])
    tol = 1e-13 if np.isinf(kappa) else 1e-8
    assert close(orc.cg_energies, out["cg_energies"], tol), name
    # vortex detector on the final state
    vx, vy, vv = gl.vortex_detector.vortices
    out["vx"], out["vy"], out["vv"] = np.asarray(vx), np.asarray(vy), np.asarray(vv)
    ox, oy, ov = O.detect_vortices(orc.g, out["psi_cg"], out["ab_cg"], H)
    assert np.array_equal(ox, out["vx"]) and np.array_equal(ov, out["vv"]), name
    np.savez_compressed(os.path.join(HERE, "case_%s.npz" % name), **out)
    return out


FV_CASES = {
    # name: (Nx, Ny, dx, dy, kappa, sigma, H, mask_kind, seed, vortices (x, y, v), lock_radius, steps (td, psi, A))
    "fv_k3": (14, 12, 0.5, 0.5, 3.0, 200.0, 0.1, "none", 4, ([2.1, 4.3], [2.4, 3.1], [1, -1]), 0.8, (4, 3, 2)),
    "fv_kinf_holes": (13, 12, 0.5, 0.5, np.inf, 1.0, 0.2, "holes", 5, ([3.0], [2.0], [2]), 1.0, (4, 3, 0)),
}


def make_fv_case(svirl, name, spec):
    """Fixed vortices: the irregular vector potential and phase lock as the
    reference sets them, then TDGL in the combined, psi-only and A-only modes
    (td.py:120-154,204-223,252-325) and the vortex list."""
    Nx, Ny, dx, dy, kappa, sigma, H, kind, seed, vort, radius, (n0, n1, n2) = spec
    rng = np.random.default_rng(200 + seed)
    mt = mask_of(kind, Nx - 1, Ny - 1, rng)
    kw = dict(Nx=Nx, Ny=Ny, dx=dx, dy=dy, order_parameter="random", random_seed=seed, gl_parameter=kappa,
              normal_conductivity=sigma, homogeneous_external_field=H, fixed_vortices=vort,
              fixed_vortices_correction="cell centers", phase_lock_radius=radius)
    if mt is not None:
        kw["material_tiling"] = mt
    gl = svirl.GLSolver(**kw)
    fvs = gl.params.fixed_vortices
    psi0 = flat(gl.vars.order_parameter)
    a, b = gl.vars.vector_potential
    ab0 = np.concatenate([flat(a), flat(b)])
    ai, bi = fvs.irregular_vector_potential
    ai0 = np.concatenate([flat(ai), flat(bi)])
    ei = gl.params.external_irregular_vector_potential
    abei = None if ei is None else np.concatenate([flat(ei[0]), flat(ei[1])])
    lock = fvs._phase_lock_ns.get_d_obj().get().astype(np.int64) if fvs._phase_lock_ns is not None else np.zeros(0, int)
    orc = O.GLOracle(Nx, Ny, dx, dy, psi0, ab0, mt=None if mt is None else flat(mt), abei=abei, kappa=kappa,
                     sigma=sigma, H=H, rand_t=seed, vpi=ai0, lock_ns=lock)
    fx, fy, fv = fvs.fixed_vortices
    out = {"Nx": Nx, "Ny": Ny, "dx": dx, "dy": dy, "kappa": kappa, "sigma": sigma, "H": H, "seed": seed,
           "vort_in": np.array(vort, dtype=float), "lock_radius": radius, "steps": np.array([n0, n1, n2]),
           "fv": np.stack([fx, fy, fv]), "psi0": psi0, "ab0": ab0, "ai0": ai0, "lock": lock,
           "mt": np.zeros(0, bool) if mt is None else flat(mt), "abei": np.zeros(0) if abei is None else abei}

    def device_vpi():
        return np.asarray(fvs._vpi.get_d_obj().get()).reshape(-1)

    def snap(tag):
        out["psi_" + tag] = flat(gl.vars.order_parameter)
        # A from the device: after psi-only steps the reference's host mirror of A is
        # not refreshed, though its device A has changed by the A_irr subtractions
        out["ab_" + tag] = np.asarray(gl.vars._vp.get_d_obj().get()).reshape(-1)
        out["vpi_" + tag] = device_vpi()
        assert close(orc.psi, out["psi_" + tag], 1e-13) and close(orc.ab, out["ab_" + tag], 1e-13), (name, tag)
        assert close(orc.vpi, out["vpi_" + tag], 1e-13), (name, tag)

    gl.solve.td(dt=0.1, Nt=n0)
    orc.td(dt=0.1, Nt=n0)
    snap("td")
    gl.solve.td(dt=0.1, Nt=n1, eqn="order_parameter")
    orc.td(dt=0.1, Nt=n1, eqn="order_parameter")
    snap("psi")
    if n2:
        gl.solve.td(dt=0.1, Nt=n2, eqn="vector_potential")
        orc.td(dt=0.1, Nt=n2, eqn="vector_potential")
        snap("A")
    out["sweeps_psi"] = np.array(orc.sweeps_psi)
    out["sweeps_A"] = np.array(orc.sweeps_A)
    out["F"] = gl.observables.free_energy
    assert abs(orc.free_energy() - out["F"]) <= 1e-12 * abs(out["F"]), name
    vx, vy, vv = gl.vortex_detector.vortices
    out["vx"], out["vy"], out["vv"] = np.asarray(vx), np.asarray(vy), np.asarray(vv)
    # the detector reads the host mirror of A (not refreshed by the A_irr kernels)
    a, b = gl.vars.vector_potential
    out["ab_host"] = np.concatenate([flat(a), flat(b)])
    ai_bi = (ai, bi)
    ox, oy, ov = O.detect_vortices(orc.g, orc.psi, out["ab_host"], H, ai_bi=ai_bi)
    assert np.array_equal(ox, out["vx"]) and np.array_equal(oy, out["vy"]) and np.array_equal(ov, out["vv"]), name
    np.savez_compressed(os.path.join(HERE, "%s.npz" % name), **out)
    return out


API_CASE = dict(Nx=12, Ny=10, dx=0.5, dy=0.5, kappa=4.0, sigma=30.0, H=0.1, ext=0.03, eps=0.9, seed=5, level=0.7,
                level2=0.5, seed2=8, dH=0.05, H_reset=0.2, dt=0.08, Nt=6)


def api_material(x, y):
    """Material tiling of the API case as a callable of the cell centres
    (svirl/mesh/grid.py:102-120): the domain minus a disc and a strip."""
    return ((x - 3.1) ** 2 + (y - 2.2) ** 2 > 1.2 ** 2) & ~((x > 4.0) & (y < 0.8))


def make_api_case(svirl):
    """The GLSolver surface around the hot path: a callable material tiling,
    random_level / random_seed at construction, randomize_order_parameter, homogeneous_external_field_delta
    and _reset (the vector potential they set), td with T given, and the
    observables normalcurrent_density and superfluid_density."""
    c = API_CASE
    gl = svirl.GLSolver(Nx=c["Nx"], Ny=c["Ny"], dx=c["dx"], dy=c["dy"], order_parameter="random",
                        random_seed=c["seed"], random_level=c["level"], gl_parameter=c["kappa"],
                        normal_conductivity=c["sigma"], linear_coefficient=c["eps"],
                        homogeneous_external_field=c["H"], external_field=c["ext"], material_tiling=api_material)
    out = {k: np.asarray(v) for k, v in c.items()}
    out["mt"] = flat(gl.mesh.material_tiling)
    assert 0 < out["mt"].sum() < out["mt"].size

    def ab():
        a, b = gl.vars.vector_potential
        return np.concatenate([flat(a), flat(b)])

    out["psi0"], out["ab0"] = flat(gl.vars.order_parameter), ab()
    ei = gl.params.external_irregular_vector_potential
    out["abei"] = np.concatenate([flat(ei[0]), flat(ei[1])])
    gl.vars.randomize_order_parameter(level=c["level2"], seed=c["seed2"])
    out["psi1"] = flat(gl.vars.order_parameter)
    gl.params.homogeneous_external_field_delta = c["dH"]
    out["H2"], out["ab2"] = np.float64(gl.params.homogeneous_external_field), ab()
    gl.params.homogeneous_external_field_reset = c["H_reset"]
    out["H3"], out["ab3"] = np.float64(gl.params.homogeneous_external_field), ab()
    try:
        gl.solve.td(dt=c["dt"], Nt=c["Nt"], T=c["dt"] * c["Nt"] + 1.0)
        raise RuntimeError("td accepted an end time that disagrees with dt * Nt")
    except AssertionError:
        pass
    gl.solve.td(dt=c["dt"], Nt=c["Nt"], T=c["dt"] * c["Nt"])
    out["psi4"], out["ab4"] = flat(gl.vars.order_parameter), ab()
    out["F4"] = gl.observables.free_energy
    out["B4"] = flat(gl.observables.magnetic_field)
    jx, jy = gl.observables.current_density
    out["j4"] = np.concatenate([flat(jx), flat(jy)])
    sx, sy = gl.observables.supercurrent_density
    out["js4"] = np.concatenate([flat(sx), flat(sy)])
    nx_, ny_ = gl.observables.normalcurrent_density
    out["jn4"] = np.concatenate([flat(nx_), flat(ny_)])
    out["rho4"] = flat(gl.observables.superfluid_density)
    # the oracle from the state after the field reset reproduces the TD step and the observables
    orc = O.GLOracle(c["Nx"], c["Ny"], c["dx"], c["dy"], out["psi1"], out["ab3"], mt=out["mt"], abei=out["abei"],
                     kappa=c["kappa"], sigma=c["sigma"], epsilon=c["eps"], H=float(out["H3"]), rand_t=c["seed"])
    orc.td(dt=c["dt"], Nt=c["Nt"])
    assert close(orc.psi, out["psi4"], 1e-13) and close(orc.ab, out["ab4"], 1e-13)
    assert abs(orc.free_energy() - out["F4"]) <= 1e-13 * abs(out["F4"])
    assert close(orc.magnetic_field(), out["B4"], 1e-12) and close(orc.current_density(), out["j4"], 1e-12)
    assert close(orc.supercurrent_density(), out["js4"], 1e-12)
    assert close(orc.current_density() - orc.supercurrent_density(), out["jn4"], 1e-12)
    assert close(np.abs(orc.psi) ** 2, out["rho4"], 1e-13)
    np.savez_compressed(os.path.join(HERE, "api_k4.npz"), **out)
    return out


def svirl_gpu(x):
    from pycuda import gpuarray  # the shim's
    return gpuarray.to_gpu(np.ascontiguousarray(x))


def main():
    from oracle.ref_build import reference_root
    ref = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if ref is None:
        raise SystemExit("reference sources not found: pass their directory or set SVIRL_REFERENCE")
    for p in (os.path.join(ROOT, "oracle", "fake_pycuda"), ref):
        sys.path.insert(0, p)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import svirl
        only = os.environ.get("GOLDEN_ONLY")  # e.g. "api": write that fixture alone
        if only in (None, "cases"):
            for name, spec in CASES.items():
                make_case(svirl, name, spec)
                print("wrote case_%s.npz" % name)
        if only in (None, "fv"):
            for name, spec in FV_CASES.items():
                make_fv_case(svirl, name, spec)
                print("wrote %s.npz" % name)
        if only in (None, "api"):
            make_api_case(svirl)
            print("wrote api_k4.npz")


if __name__ == "__main__":
    main()
