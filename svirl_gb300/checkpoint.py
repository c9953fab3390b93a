"""Checkpoint / resume of a solver, and a dataset format for relaxed states.

A checkpoint is one ``.npz`` file holding everything the next TDGL step or CG
iteration depends on: the grid, the dtype, the model parameters, the material
tiling, psi, A, the external vector potential and the Langevin counter
``rand_t`` (``svirl/solvers/td.py:35-37``: the noise of step t is a hash of the
node index and t, so restoring t continues the same noise sequence).  A run
restored from a checkpoint continues bit for bit as the run that wrote it.
The reference keeps its state only in memory (``svirl/vars/vars.py:53-127``);
the file layout here is this project's.

    from svirl_gb300 import checkpoint
    checkpoint.save(gl, "state.npz")
    gl2 = checkpoint.load("state.npz")          # a new GLSolver
    checkpoint.restore(gl, "state.npz")         # into an existing one (same grid)

Datasets (the learned warm start's training data): ``save_dataset`` /
``load_dataset`` store sampled instances (n, dx, H, kappa, sigma, cell mask,
psi0) with their relaxed (psi, A).
"""
import numpy as np

FORMAT = 1


def _state(gl):
    c, p = gl.cfg, gl.params
    a, b = gl.vars.vector_potential
    ext = p.external_vector_potential
    mt = gl.mesh._mt  # None: the full domain
    return dict(
        format=np.int32(FORMAT),
        Nx=np.int32(c.Nx), Ny=np.int32(c.Ny), dx=np.float64(c.dx), dy=np.float64(c.dy),
        dtype=np.str_(np.dtype(c.dtype).name),
        gl_parameter=np.float64(p.gl_parameter),
        normal_conductivity=np.float64(p.normal_conductivity),
        linear_coefficient=np.asarray(p._epsilon),  # 0-d when uniform
        homogeneous_external_field=np.float64(p.homogeneous_external_field),
        langevin_psi=np.float64(p.order_parameter_Langevin_coefficient),
        langevin_A=np.float64(p.vector_potential_Langevin_coefficient),
        stop_psi=np.float64(c.stop_criterion_order_parameter),
        stop_A=np.float64(c.stop_criterion_vector_potential),
        convergence_rtol=np.float64(c.convergence_rtol),
        rand_t=np.uint32(gl._h.get_params().rand_t),
        material_tiling=np.zeros((0, 0), bool) if mt is None else np.asarray(mt, bool),
        psi=np.asarray(gl.vars.order_parameter),
        a=np.asarray(a), b=np.asarray(b),
        ext_a=np.zeros((0, 0)) if ext is None else np.asarray(ext[0]),
        ext_b=np.zeros((0, 0)) if ext is None else np.asarray(ext[1]),
        fv=np.stack(p.fixed_vortices.fixed_vortices) if p.fixed_vortices.fixed_vortices_x.size else np.zeros((3, 0)),
        fv_lock_radius=np.float64(np.nan if p.fixed_vortices.phase_lock_radius is None
                                  else p.fixed_vortices.phase_lock_radius),
        fv_td=(gl._h.get_irregular_vector_potential() if p.fixed_vortices.fixed_vortices_x.size
               else np.zeros(0)),
        # the external + irregular potential in use (set when the external potential was)
        vpei_a=np.zeros((0, 0)) if p._vpei is None else np.asarray(p._vpei[0]),
        vpei_b=np.zeros((0, 0)) if p._vpei is None else np.asarray(p._vpei[1]),
    )


def save(gl, path):
    """Write the solver's state to `path` (``.npz``)."""
    np.savez(path, **_state(gl))


def _read(path):
    with np.load(path, allow_pickle=False) as f:
        d = {k: f[k] for k in f.files}
    if int(d.get("format", -1)) != FORMAT:
        raise ValueError("%s: not a checkpoint of format %d" % (path, FORMAT))
    return d


def _apply(gl, d):
    c, p = gl.cfg, gl.params
    if (int(d["Nx"]), int(d["Ny"])) != (int(c.Nx), int(c.Ny)) or str(d["dtype"]) != np.dtype(c.dtype).name:
        raise ValueError("checkpoint grid or dtype (%d x %d, %s) differs from the solver's (%d x %d, %s)"
                         % (int(d["Nx"]), int(d["Ny"]), str(d["dtype"]), c.Nx, c.Ny, np.dtype(c.dtype).name))
    mt = d["material_tiling"]
    gl.mesh.material_tiling = None if mt.size == 0 else mt
    p.gl_parameter = float(d["gl_parameter"])
    p.normal_conductivity = float(d["normal_conductivity"])
    eps = d["linear_coefficient"]
    p.linear_coefficient = float(eps) if eps.ndim == 0 else eps
    p.homogeneous_external_field = float(d["homogeneous_external_field"])
    fv = d["fv"]
    r = float(d["fv_lock_radius"])
    p.fixed_vortices.phase_lock_radius = None if np.isnan(r) else r
    p.fixed_vortices.fixed_vortices = None if fv.shape[1] == 0 else (fv[0], fv[1], fv[2])
    if fv.shape[1]:  # the TD step's copy of A_irr, changed by A loops since it was set
        gl._h.set_irregular_vector_potential(d["fv_td"], td_copy_only=True)
    p.external_vector_potential = None if d["ext_a"].size == 0 else (d["ext_a"], d["ext_b"])
    p._vpei = None if d["vpei_a"].size == 0 else (d["vpei_a"], d["vpei_b"])
    if p._vpei is None:
        gl._h.set_abei(None)
    else:
        flat = np.concatenate([d["vpei_a"].T.reshape(-1), d["vpei_b"].T.reshape(-1)]).astype(c.dtype)
        gl._h.set_abei(None if not np.any(flat) else flat)
    p.order_parameter_Langevin_coefficient = float(d["langevin_psi"])
    p.vector_potential_Langevin_coefficient = float(d["langevin_A"])
    gl.vars.order_parameter = d["psi"]
    gl.vars.vector_potential = (d["a"], d["b"])
    gl._h.set_params(rand_t=int(d["rand_t"]), stop_psi=float(d["stop_psi"]), stop_A=float(d["stop_A"]))
    c.stop_criterion_order_parameter = c.dtype(d["stop_psi"])
    c.stop_criterion_vector_potential = c.dtype(d["stop_A"])
    c.convergence_rtol = float(d["convergence_rtol"])


def restore(gl, path):
    """Load the state in `path` into `gl` (same grid and dtype)."""
    _apply(gl, _read(path))


def load(path, device_id=0):
    """A new GLSolver with the state in `path`."""
    from .solver import GLSolver
    d = _read(path)
    gl = GLSolver(Nx=int(d["Nx"]), Ny=int(d["Ny"]), dx=float(d["dx"]), dy=float(d["dy"]),
                  dtype=np.dtype(str(d["dtype"])).type, order_parameter=1.0, device_id=device_id,
                  convergence_rtol=float(d["convergence_rtol"]))
    _apply(gl, d)
    return gl


def save_dataset(path, insts, states):
    """Instances (``learned.Instance``, one size) and their relaxed [(psi, ab)]."""
    n = insts[0].n
    if any(it.n != n for it in insts):
        raise ValueError("a dataset holds instances of one size")
    np.savez(path, format=np.int32(FORMAT), n=np.int32(n), dx=np.float64(insts[0].dx),
             H=np.array([it.H for it in insts]), kappa=np.array([it.kappa for it in insts]),
             sigma=np.array([it.sigma for it in insts]), mt=np.stack([it.mt for it in insts]),
             psi0=np.stack([it.psi0 for it in insts]), psi=np.stack([np.asarray(s[0]) for s in states]),
             ab=np.stack([np.asarray(s[1]) for s in states]))


def load_dataset(path):
    """(instances, [(psi, ab)]) written by ``save_dataset``."""
    from .learned import Instance
    with np.load(path, allow_pickle=False) as f:
        if int(f["format"]) != FORMAT:
            raise ValueError("%s: not a dataset of format %d" % (path, FORMAT))
        n, dx = int(f["n"]), float(f["dx"])
        insts = [Instance(n, dx, float(H), float(k), mt, p0, sigma=float(s))
                 for H, k, s, mt, p0 in zip(f["H"], f["kappa"], f["sigma"], f["mt"], f["psi0"])]
        states = list(zip(f["psi"], f["ab"]))
    return insts, states
