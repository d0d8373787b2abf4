"""Multi-rank path on host ranks (gloo, 2 and 3 processes): the reference's block partition,
the two-phase ghost exchange (periodic and not), sharded heat runs (one exchange per sweep, and
one exchange of a 3-deep halo per 1-3 sweeps) gathered and compared bit-for-bit with the
whole-grid oracle, scalar all-reduce, and the flood domain plan.

The per-rank sweep in these tests is the oracle's one-iteration step (no GPU here); on GPUs the
same driver calls the C-ABI sweep (tests/test_shard_gpu.py)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from appfis_gb300 import shard
from appfis_gb300 import workloads as W


def test_partition_follows_reference_rule():
    # n // parts each, the first n % parts blocks one more (Appfis/Common.hpp:216-224)
    assert [shard.partition(10, 3, r) for r in range(3)] == [(0, 4), (4, 3), (7, 3)]
    assert [shard.partition(8, 4, r) for r in range(4)] == [(0, 2), (2, 2), (4, 2), (6, 2)]
    for n in (5, 17, 1024, 16384):
        for parts in (q for q in (1, 2, 3, 5, 8) if q <= n):
            blocks = [shard.partition(n, parts, r) for r in range(parts)]
            assert blocks[0][0] == 0 and sum(c for _, c in blocks) == n
            assert all(blocks[r][0] + blocks[r][1] == blocks[r + 1][0] for r in range(parts - 1))
    with pytest.raises(ValueError):
        shard.partition(2, 3, 0)


def test_assign_units_balanced_and_deterministic():
    costs = [W.triton_sizes(32, 512, 3072, 42)[k][0] * W.triton_sizes(32, 512, 3072, 42)[k][1] for k in range(32)]
    for world in (1, 2, 3, 8):
        plan = shard.assign_units(costs, world)
        assert sorted(u for p in plan for u in p) == list(range(32))
        loads = [sum(costs[u] for u in p) for p in plan]
        assert max(loads) - min(loads) <= max(costs)  # greedy bound
        assert plan == shard.assign_units(costs, world)
    assert shard.assign_units([5, 5, 5], 5)[3:] == [[], []]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, case, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = case(rank, world)
        if rank == 0:
            out.put(res)
    finally:
        dist.destroy_process_group()


def _spawn(case, world):
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    mp.start_processes(_worker, args=(world, _free_port(), case, q), nprocs=world, join=True, start_method="spawn")
    return q.get()


def _case_exchange(rank, world):
    """Interior rows labelled with their global index; ghosts -1.  Returns per-rank checks."""
    ok = []
    for periodic in (False, True):
        n, g = 11, 2
        s = shard.Slab(n, g, periodic=periodic)
        f = torch.full((s.local_extent(), 3), -1.0)
        s.interior(f)[:] = torch.arange(s.start, s.start + s.count, dtype=torch.float32)[:, None]
        s.exchange(f)
        lo = [(s.start - g + i) for i in range(g)]
        hi = [(s.start + s.count + i) for i in range(g)]
        want_lo = [float(v % n) if periodic or 0 <= v < n else -1.0 for v in lo]
        want_hi = [float(v % n) if periodic or 0 <= v < n else -1.0 for v in hi]
        ok.append(f[:g, 0].tolist() == want_lo and f[-g:, 0].tolist() == want_hi)
    t = torch.tensor([1.0 if all(ok) else 0.0])
    dist.all_reduce(t, op=dist.ReduceOp.MIN)
    return t.item()


def _case_heat(rank, world):
    from oracle import oracle as O
    c = dict(nx=37, ny=29, iters=9, r=0.2)
    full = torch.from_numpy(W.heat2d_padded(c["nx"], c["ny"], 1.0, 7))
    s = shard.Slab(c["ny"], 1)
    a = s.scatter(full)
    b = a.clone()

    def sweep(cur, nxt):  # one iteration on the local padded slab
        nxt.copy_(torch.from_numpy(O.heat2d(cur.numpy(), 1, c["r"], threads=1)))

    cur = shard.iterate(s, a, b, c["iters"], sweep)
    got = s.gather(cur)
    total = shard.allreduce(float(s.interior(cur)[:, 1:-1].double().sum()), "sum")
    if rank != 0:
        return None
    ref = O.heat2d(full.numpy(), c["iters"], c["r"], threads=1)
    return bool(np.array_equal(got.numpy(), ref[1:-1])), total, float(ref[1:-1, 1:-1].astype(np.float64).sum())


def _case_heat_blocked(rank, world):
    """Ghost width 3, one exchange per `depth` sweeps, 10 sweeps (the last block shorter)."""
    from oracle import oracle as O
    c = dict(nx=37, ny=29, iters=10, r=0.2)
    out = []
    for depth in (1, 2, 3):
        g = 3
        core = W.heat2d_padded(c["nx"], c["ny"], 1.0, 7)
        # the global field with g ghost rows on each side (the Dirichlet row next to the interior)
        full = torch.from_numpy(np.concatenate([np.repeat(core[:1], g - 1, 0), core, np.repeat(core[-1:], g - 1, 0)]))
        s = shard.Slab(c["ny"], g)
        a = s.scatter(full)
        b = a.clone()

        def sweep_layers(cur, nxt, k, lo, hi):  # rows lo .. hi-1, rows lo-1 and hi as the fixed ring
            sub = cur[lo - 1:hi + 1].numpy()
            nxt.copy_(cur)
            nxt[lo - 1:hi + 1] = torch.from_numpy(O.heat2d(sub, k, c["r"], threads=1))
            return nxt

        cur = shard.iterate_blocked(s, a, b, c["iters"], sweep_layers, depth)
        got = s.gather(cur)
        if rank == 0:
            ref = O.heat2d(core, c["iters"], c["r"], threads=1)
            out.append(bool(np.array_equal(got.numpy(), ref[1:-1])))
    return out if rank == 0 else None


@pytest.mark.parametrize("world", [2, 3])
def test_blocked_exchange_heat_matches_whole_grid_gloo(world):
    assert _spawn(_case_heat_blocked, world) == [True, True, True]


def test_blocked_depth_checked():
    s = shard.Slab(10, 2, rank=0, world=1)
    with pytest.raises(ValueError):
        shard.iterate_blocked(s, torch.zeros(14), torch.zeros(14), 3, lambda *a: None, 3)


@pytest.mark.parametrize("world", [2, 3])
def test_exchange_gloo(world):
    assert _spawn(_case_exchange, world) == 1.0


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_heat_matches_whole_grid_gloo(world):
    same, total, ref_total = _spawn(_case_heat, world)
    assert same
    assert total == pytest.approx(ref_total, rel=1e-12)


def test_single_rank_periodic_wraps_in_place():
    s = shard.Slab(6, 1, periodic=True, rank=0, world=1)
    f = torch.arange(8, dtype=torch.float32)
    s.exchange(f)
    assert f.tolist() == [6.0, 1, 2, 3, 4, 5, 6, 1.0]
    s = shard.Slab(6, 1, periodic=False, rank=0, world=1)
    f = torch.arange(8, dtype=torch.float32)
    s.exchange(f)
    assert f.tolist() == list(range(8))
