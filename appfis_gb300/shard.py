"""Multi-rank decomposition of the hot path: slabs of a padded field with a halo exchange per
sweep (or one exchange of a deeper halo per several sweeps), scalar all-reduces, and the
assignment of independent flood domains to ranks.

The reference partitions every grid into Cartesian blocks, one per MPI rank
(Appfis/Common.hpp:197-226: n // blocks points per rank, the first n % blocks ranks one more),
and refreshes ghost layers after every sweep with two Sendrecv's per axis — low face to the low
neighbour while receiving the high ghost, then high face to the high neighbour while receiving
the low ghost (Appfis/Communication.hpp:612-678), with wrap-around neighbours when the
topology is periodic.  Reductions end in an MPI_Allreduce (Communication.hpp:752-789).

Here one process drives one GPU and the field is split along its slowest axis only: each
rank's slab is then one contiguous block of rows/planes, its faces are contiguous slices, and
the exchange is a pair of point-to-point transfers of whole faces (torch.distributed: NCCL
between GPUs, gloo between host processes) with no packing kernels.  The sweep itself is a
callable (a C-ABI kernel on the rank's device buffers), so the same driver runs every
workload.  Flood domains are independent units: they are dealt to ranks by their cell counts
(longest first onto the least-loaded rank) and need no exchange at all.
"""
import torch
import torch.distributed as dist


def partition(n, parts, index):
    """(start, count) of block `index` of `parts` over n points: n // parts each, the first
    n % parts blocks one more (Appfis/Common.hpp:216-224)."""
    if parts < 1 or not 0 <= index < parts:
        raise ValueError("partition: bad parts/index %d/%d" % (parts, index))
    if n < parts:
        raise ValueError("partition: %d ranks for %d points" % (parts, n))
    base, rem = divmod(n, parts)
    start = index * base + min(index, rem)
    return start, base + (1 if index < rem else 0)


class Slab:
    """This rank's block of the slowest axis of a padded field.

    n: interior extent of the slowest axis; ghost: ghost width; periodic: wrap-around
    neighbours.  The local field holds count + 2*ghost entries on that axis: ghost layers,
    the rank's interior block, ghost layers (the reference's sub-grid layout)."""

    def __init__(self, n, ghost, periodic=False, rank=None, world=None, group=None):
        self.group = group
        self.rank = dist.get_rank(group) if rank is None else rank
        self.world = dist.get_world_size(group) if world is None else world
        self.n, self.ghost, self.periodic = n, ghost, periodic
        self.start, self.count = partition(n, self.world, self.rank)
        if self.count < ghost:
            raise ValueError("slab of %d layers is thinner than the ghost width %d" % (self.count, ghost))
        lo, hi = self.rank - 1, self.rank + 1
        if periodic:
            lo %= self.world
            hi %= self.world
        self.low = lo if 0 <= lo < self.world else None    # neighbour owning the layers below
        self.high = hi if 0 <= hi < self.world else None   # neighbour owning the layers above

    def local_extent(self):
        return self.count + 2 * self.ghost

    def interior(self, field):
        """View of this rank's interior layers of a local field."""
        return field[self.ghost:self.ghost + self.count]

    def scatter(self, full_padded):
        """This rank's local padded slab cut from a full padded field (every rank holds it)."""
        g = self.ghost
        return full_padded[self.start:self.start + self.count + 2 * g].clone()

    def exchange(self, field):
        """Refreshes the ghost layers of `field` (local padded slab, slowest axis first) from the
        neighbours' interior faces; ghost layers without a neighbour keep their values."""
        g, c = self.ghost, self.count
        low_face, high_face = field[g:2 * g], field[c:c + g]
        low_ghost, high_ghost = field[0:g], field[c + g:c + 2 * g]
        # phase 1: low face -> low neighbour, high ghost <- high neighbour
        self._sendrecv(low_face, self.low, high_ghost, self.high, tag=0)
        # phase 2: high face -> high neighbour, low ghost <- low neighbour
        self._sendrecv(high_face, self.high, low_ghost, self.low, tag=1)
        return field

    def _sendrecv(self, send, dst, recv, src, tag):
        if dst is None and src is None:
            return
        if dst == self.rank and src == self.rank:  # one rank, periodic: wrap in place
            recv.copy_(send)
            return
        ops = []
        sbuf = send.contiguous()
        rbuf = recv if recv.is_contiguous() else torch.empty_like(recv)
        if dst is not None:
            ops.append(dist.P2POp(dist.isend, sbuf, self._global(dst), group=self.group, tag=tag))
        if src is not None:
            ops.append(dist.P2POp(dist.irecv, rbuf, self._global(src), group=self.group, tag=tag))
        for req in dist.batch_isend_irecv(ops):
            req.wait()
        if src is not None and rbuf is not recv:
            recv.copy_(rbuf)

    def _global(self, r):
        return r if self.group is None else dist.get_global_rank(self.group, r)

    def gather(self, field, dst=0):
        """Interior layers of every rank, concatenated along the slowest axis, on rank `dst`
        (None elsewhere)."""
        mine = self.interior(field).contiguous()
        parts = None
        if self.rank == dst:
            parts = [torch.empty((partition(self.n, self.world, r)[1],) + tuple(mine.shape[1:]), dtype=mine.dtype,
                                 device=mine.device) for r in range(self.world)]
        if self.world == 1:
            return mine.clone()
        # gather with uneven blocks: point-to-point from every rank to dst
        if self.rank == dst:
            for r in range(self.world):
                if r == dst:
                    parts[r].copy_(mine)
                else:
                    dist.recv(parts[r], self._global(r), group=self.group)
            return torch.cat(parts, 0)
        dist.send(mine, self._global(dst), group=self.group)
        return None


def iterate(slab, cur, nxt, iters, sweep):
    """`iters` sweeps of the slab: ghost refresh of the current buffer, then sweep(cur, nxt),
    then swap (the reference's Execute*D with GridsToUpdate, Runtime.hpp:306-369).  Returns the
    buffer holding the newest state."""
    for _ in range(iters):
        slab.exchange(cur)
        sweep(cur, nxt)
        cur, nxt = nxt, cur
    return cur


def iterate_blocked(slab, cur, nxt, iters, sweep_layers, depth):
    """`iters` sweeps of a radius-1 stencil with one ghost exchange per `depth` sweeps (temporal
    blocking across ranks; slab.ghost >= depth): after an exchange the rank advances its whole
    local slab except the outermost layer on each side that faces a neighbour by up to `depth`
    sweeps.  The stale outer layer corrupts one more layer per sweep, so after k <= ghost
    sweeps the rank's own layers are exact, and the next exchange replaces the corrupted ghost
    layers.  On a side without a neighbour (non-periodic edge) all ghost layers stay fixed, as
    the reference's boundary does.  This lets a kernel that does several sweeps per launch on
    chip (the time-blocked heat and GameOfLife kernels) run on a slab.

    sweep_layers(cur, nxt, k, lo, hi) advances layers lo .. hi-1 of `cur` (slowest axis) by k
    sweeps, reading the layers outside that range as a fixed boundary, and returns the buffer
    holding the result (cur or nxt; its layers outside lo .. hi-1 must equal cur's).  Returns
    the buffer holding the newest state."""
    if not 1 <= depth <= slab.ghost:
        raise ValueError("iterate_blocked: depth %d must be in 1 .. ghost width %d" % (depth, slab.ghost))
    lo = 1 if slab.low is not None else slab.ghost
    hi = slab.local_extent() - (1 if slab.high is not None else slab.ghost)
    done = 0
    while done < iters:
        k = min(depth, iters - done)
        slab.exchange(cur)
        if sweep_layers(cur, nxt, k, lo, hi) is nxt:
            cur, nxt = nxt, cur
        done += k
    return cur


def allreduce(value, op="sum", device="cpu", group=None):
    """A scalar reduced over all ranks (the reference's AllReduce after Execute*DReduce)."""
    t = torch.tensor([value], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op={"sum": dist.ReduceOp.SUM, "max": dist.ReduceOp.MAX, "min": dist.ReduceOp.MIN}[op],
                        group=group)
    return float(t.item())


def assign_units(costs, world):
    """Deals independent units (flood domains, by cell count) to `world` ranks: longest first
    onto the least-loaded rank (ties to the lower rank).  Returns one list of unit indices per
    rank, each in increasing order; deterministic, so every rank computes the same plan."""
    load = [0] * world
    plan = [[] for _ in range(world)]
    for u in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        plan[r].append(u)
        load[r] += costs[u]
    return [sorted(p) for p in plan]
