"""Build a GLSolver (GPU) and a GLOracle (CPU) on the same initial state."""
import numpy as np

from oracle import gl_oracle as O


def flat(x):
    return np.reshape(np.asarray(x).T, -1)


def random_mask(rng, nxc, nyc, kind="random30"):
    mt = np.ones((nxc, nyc), dtype=bool)
    if kind == "full":
        return mt
    if kind == "none":
        return None
    if kind == "empty":
        mt[:] = False
        return mt
    if kind == "q1":
        mt[: nxc // 2, : nxc // 2] = False
        return mt
    if kind == "holes":
        xs = np.arange(nxc)[:, None]
        ys = np.arange(nyc)[None, :]
        for _ in range(max(1, nxc * nyc // 60)):
            cx, cy, r = rng.integers(nxc), rng.integers(nyc), 1.5 + 2 * rng.random()
            mt[(xs - cx) ** 2 + (ys - cy) ** 2 < r * r] = False
        return mt
    p = int(kind[6:]) / 100.0
    k = int(p * nxc * nyc)
    mt[rng.integers(0, nxc, k), rng.integers(0, nyc, k)] = False
    return mt


def make_pair(Nx=12, Ny=11, dx=0.5, dy=0.45, kappa=np.inf, sigma=1.0, H=0.1, mask="none", seed=0,
              dtype=np.float64, external_field=0.0, langevin=(0.0, 0.0), landau=False, stop=1e-6, **kw):
    from svirl_gb300 import GLSolver
    rng = np.random.default_rng(seed)
    mt = random_mask(rng, Nx - 1, Ny - 1, mask)
    gl = GLSolver(Nx=Nx, Ny=Ny, dx=dx, dy=dy, order_parameter="random", random_seed=seed,
                  gl_parameter=kappa, normal_conductivity=sigma, homogeneous_external_field=H,
                  material_tiling=mt, dtype=dtype, external_field=external_field,
                  order_parameter_Langevin_coefficient=langevin[0],
                  vector_potential_Langevin_coefficient=langevin[1],
                  stop_criterion_order_parameter=stop, stop_criterion_vector_potential=stop, **kw)
    if landau:
        ya = gl.mesh.xy_a_grid[1]
        a = (-H * ya).astype(dtype)
        b = np.zeros((Nx, Ny - 1), dtype=dtype)
        gl.vars.vector_potential = (a, b)
    orc = oracle_of(gl, rand_t=seed)
    return gl, orc


def oracle_of(gl, rand_t=1, kernels=None):
    c = gl.cfg
    psi = flat(gl.vars.order_parameter).astype(np.complex128)
    a, b = gl.vars.vector_potential
    ab = np.concatenate([flat(a), flat(b)]).astype(np.float64)
    mt = flat(gl.mesh.material_tiling) if gl.mesh.have_material_tiling() else None
    ev = gl.params.external_vector_potential
    abei = None if ev is None else np.concatenate([flat(ev[0]), flat(ev[1])]).astype(np.float64)
    if abei is not None and not np.any(abei):
        abei = None
    return O.GLOracle(int(c.Nx), int(c.Ny), float(c.dx), float(c.dy), psi, ab, mt=mt, abei=abei,
                      kappa=float(gl.params.gl_parameter), sigma=float(gl.params.normal_conductivity),
                      epsilon=float(np.asarray(gl.params._epsilon)) if np.ndim(gl.params._epsilon) == 0 else 0.0,
                      epsilon_spatial=(None if np.ndim(gl.params._epsilon) == 0
                                       else flat(gl.params._epsilon).astype(np.float64)),
                      H=float(gl.params.homogeneous_external_field),
                      stop_psi=float(c.stop_criterion_order_parameter), stop_A=float(c.stop_criterion_vector_potential),
                      rand_t=rand_t, langevin_psi=float(gl.params.order_parameter_Langevin_coefficient),
                      langevin_A=float(gl.params.vector_potential_Langevin_coefficient),
                      convergence_rtol=c.convergence_rtol, dtype=c.dtype, kernels=kernels)


def gpu_state(gl):
    return gl._h.get_psi().astype(np.complex128), gl._h.get_ab().astype(np.float64)


def rel_err(x, y):
    x, y = np.asarray(x), np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))
