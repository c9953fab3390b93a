"""Multi-rank layouts of the hot path on CPU ranks (gloo, 127.0.0.1): instance
sharding with a result gather, and the row-block decomposition of one domain
with halo exchange and a MAX all-reduce of the Jacobi residual, which must give
exactly the single-domain TDGL result (same values, same sweep counts).  The
per-block compute is the oracle's sweep; on GPUs it is the library's."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from oracle import gl_oracle as O
from oracle import kernels_np as K
from svirl_gb300 import domain as D


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(world, fn, *args):
    ctx = mp.get_context("spawn")
    port = _free_port()
    q = ctx.Queue()
    ps = [ctx.Process(target=_entry, args=(r, world, port, fn, args, q)) for r in range(world)]
    for p in ps:
        p.start()
    out = [q.get(timeout=240) for _ in range(world)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    return dict(out)


def _entry(rank, world, port, fn, args, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, fn(rank, world, dist, *args)))
    finally:
        dist.destroy_process_group()


# --------------------------------------------------------------------------
def _case(seed, Nx=13, Ny=17, H=0.15):
    rng = np.random.default_rng(seed)
    g = K.Grid(Nx, Ny, 0.5, 0.45)
    mt = rng.random((Nx - 1) * (Ny - 1)) > 0.2
    psi = (1.0 - 0.5 * rng.random(g.N)) * np.exp(1j * np.pi * (2 * rng.random(g.N) - 1))
    ab = 0.1 * rng.standard_normal(g.Nab)
    return g, mt, psi, ab


def test_shard_instances_is_a_balanced_partition():
    sizes = [129 ** 2, 513 ** 2, 193 ** 2, 257 ** 2, 385 ** 2, 129 ** 2, 257 ** 2, 513 ** 2]
    for world in (1, 2, 3, 4):
        owner = D.shard_instances(sizes, world)
        assert owner == D.shard_instances(sizes, world)
        load = np.bincount(owner, weights=sizes, minlength=world)
        assert load.sum() == sum(sizes) and load.max() - load.min() <= max(sizes)


def _shard_worker(rank, world, dist, seeds):
    owner = D.shard_instances([_case(s)[0].N for s in seeds], world)
    mine = {}
    for q, s in enumerate(seeds):
        if owner[q] == rank:
            g, mt, psi, ab = _case(s)
            mine[q] = float(K.free_energy(g, 25.0, 1.0, None, 0.15, mt, psi, None, ab))
    parts = [None] * world
    dist.all_gather_object(parts, mine)
    allres = {}
    for p in parts:
        allres.update(p)
    return [allres[q] for q in range(len(seeds))]


def test_instance_shards_gather_equals_serial():
    seeds = list(range(7))
    res = _run(2, _shard_worker, seeds)
    serial = []
    for s in seeds:
        g, mt, psi, ab = _case(s)
        serial.append(float(K.free_energy(g, 25.0, 1.0, None, 0.15, mt, psi, None, ab)))
    assert res[0] == serial and res[1] == serial


def _domain_worker(rank, world, dist, seed, steps, dt, stop):
    g, mt, psi, ab = _case(seed)
    Nx, Ny = g.Nx, g.Ny
    B = D.RowBlocks(Nx, Ny, world, rank)
    ny = B.n_local_rows
    gl = K.Grid(Nx, ny, g.dx, g.dy)
    mt_l = B.local_cells(mt.reshape(Ny - 1, Nx - 1)).reshape(-1)
    a_l, b_l = B.local_links(g.a2(ab), g.b2(ab))
    ab_l = np.concatenate([a_l.reshape(-1), b_l.reshape(-1)])
    psi_l = B.local_nodes(psi.reshape(Ny, Nx)).copy()
    own = B.owned()
    sweeps = []

    def converged(code):
        return 1.0e-4 * float(code) < 1.0

    for _ in range(steps):
        rhs = psi_l.reshape(-1).copy()

        def sweep(cur):
            nxt, _ = K.iterate_order_parameter_jacobi_step(gl, dt, 1.0, None, mt_l, ab_l, rhs.copy(), cur.reshape(-1),
                                                           0.0, 1, 0, stop)
            nxt = nxt.reshape(ny, Nx)
            c = cur.reshape(ny, Nx)
            r = np.fmax(np.abs(nxt.real - c.real), np.abs(nxt.imag - c.imag))[own]
            return nxt, float(K.residual_code(r, stop).max())

        psi_l, k = D.jacobi_solve(B, sweep, psi_l, converged, dist)
        sweeps.append(k)
    return psi_l[own].reshape(-1).tolist(), sweeps


@pytest.mark.parametrize("world", [2, 3])
def test_row_blocks_reproduce_single_domain_td(world):
    seed, steps, dt, stop = 3, 4, 0.1, 1e-9
    res = _run(world, _domain_worker, seed, steps, dt, stop)
    g, mt, psi, ab = _case(seed)
    orc = O.GLOracle(g.Nx, g.Ny, g.dx, g.dy, psi, ab, mt=mt, kappa=np.inf, H=0.15, stop_psi=stop)
    orc.td(dt=dt, Nt=steps, eqn="order_parameter")
    full = np.concatenate([np.array(res[r][0]) for r in range(world)])
    assert np.array_equal(full, orc.psi)
    for r in range(world):
        assert res[r][1] == orc.sweeps_psi
