"""Multi-GPU layout of the hot path (host-side logic).

Two ways the work splits across ranks (one process per GPU):

* Instances (batched sweeps, serving): independent instances are partitioned
  across ranks by node count (longest-processing-time greedy), each rank runs
  its share through the batched engine, and only results are gathered: no
  collective on the data path.  ``shard_instances``.

* One large domain: rows of nodes are split into contiguous blocks, each rank
  holds its rows plus one halo row on each side.  Every Jacobi sweep of the psi
  step updates the owned rows, takes the maximum residual over ranks
  (all-reduce MAX) for the reference's stop rule, and exchanges the halo rows
  with the neighbours.  Each node's update reads only its four neighbours, so
  the decomposed iteration computes exactly the single-domain values and stops
  after the same sweep.  ``RowBlocks`` + ``jacobi_solve``; the per-block sweep
  is supplied by the caller (on a GPU, the library's sweep on the block).

Every GPU in this build's test machines stands alone, so the multi-rank paths
are exercised on CPU ranks (gloo) in the tests.
"""
import numpy as np


def shard_instances(node_counts, world):
    """Rank of each instance: instances sorted by size, each given to the rank
    with the fewest nodes so far (ties: lowest rank).  Deterministic."""
    load = [0] * world
    owner = [0] * len(node_counts)
    for q in sorted(range(len(node_counts)), key=lambda q: (-node_counts[q], q)):
        r = min(range(world), key=lambda k: (load[k], k))
        owner[q] = r
        load[r] += node_counts[q]
    return owner


class RowBlocks:
    """Contiguous blocks of node rows j in [j0, j1) per rank, with one halo row on
    each interior side: the local array holds rows [lo, hi)."""

    def __init__(self, Nx, Ny, world, rank):
        if Ny < 2 * world:
            raise ValueError("fewer than two rows per rank")
        self.Nx, self.Ny, self.world, self.rank = Nx, Ny, world, rank
        edges = [round(k * Ny / world) for k in range(world + 1)]
        self.j0, self.j1 = edges[rank], edges[rank + 1]
        self.lo = max(0, self.j0 - 1)
        self.hi = min(Ny, self.j1 + 1)

    @property
    def n_local_rows(self):
        return self.hi - self.lo

    def owned(self):
        """Slice of the local rows this rank owns."""
        return slice(self.j0 - self.lo, self.j1 - self.lo)

    def local_nodes(self, field_rows):
        """Rows [lo, hi) of a (Ny, Nx) node field."""
        return np.ascontiguousarray(field_rows[self.lo:self.hi])

    def local_cells(self, cells_rows):
        """Cells between the local node rows: rows [lo, hi-1) of a (Ny-1, Nx-1) cell field."""
        return np.ascontiguousarray(cells_rows[self.lo:self.hi - 1])

    def local_links(self, a_rows, b_rows):
        """x links on the local rows and y links between them."""
        return np.ascontiguousarray(a_rows[self.lo:self.hi]), np.ascontiguousarray(b_rows[self.lo:self.hi - 1])

    def exchange_halo(self, local, dist, group=None):
        """Send the first and last owned rows to the neighbours and receive their
        rows into the halo rows (torch.distributed point-to-point, CPU tensors)."""
        import torch
        reqs = []
        t = torch.from_numpy(local.view(np.float64) if local.dtype == np.complex128 else local)
        own = self.owned()
        if self.rank > 0:
            reqs.append(dist.isend(t[own.start].contiguous(), self.rank - 1, group=group))
            buf_lo = torch.empty_like(t[0])
            reqs.append(dist.irecv(buf_lo, self.rank - 1, group=group))
        if self.rank < self.world - 1:
            reqs.append(dist.isend(t[own.stop - 1].contiguous(), self.rank + 1, group=group))
            buf_hi = torch.empty_like(t[0])
            reqs.append(dist.irecv(buf_hi, self.rank + 1, group=group))
        for r in reqs:
            r.wait()
        if self.rank > 0:
            t[0] = buf_lo
        if self.rank < self.world - 1:
            t[-1] = buf_hi


def allreduce_max(x, dist, group=None):
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def jacobi_solve(blocks, sweep, psi_local, converged, dist, max_sweeps=1024, group=None):
    """The Jacobi loop of one psi step on a row block: `sweep(psi_local)` returns
    (new local psi, max residual over the owned rows); the loop stops when
    `converged(global max residual)` or after `max_sweeps` sweeps, exactly as
    the single-domain loop.  Returns (psi_local, sweeps)."""
    k = 0
    while True:
        psi_local, r = sweep(psi_local)
        k += 1
        blocks.exchange_halo(psi_local, dist, group)
        if converged(allreduce_max(r, dist, group)) or k >= max_sweeps:
            return psi_local, k
