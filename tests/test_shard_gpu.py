"""The sharded driver on one GPU: the slab iteration with the C-ABI heat sweep reproduces the
oracle bit-for-bit, and the single-rank periodic exchange equals the library's periodic ghost
refresh along the slowest axis."""
import ctypes

import numpy as np
import pytest

from appfis_gb300 import shard
from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_slab_iteration_with_device_sweep(gb, torch_cuda):
    torch = torch_cuda
    nx, ny, iters, r = 45, 33, 12, 0.2
    full = W.heat2d_padded(nx, ny, 1.0, 3)
    s = shard.Slab(ny, 1, rank=0, world=1)
    a = s.scatter(torch.from_numpy(full)).cuda()
    b = a.clone()

    def sweep(cur, nxt):
        gb.call("appfis_gb_heat2d_sweep", cur.data_ptr(), nxt.data_ptr(), nx, ny, nx + 2, r, r,
                torch.cuda.current_stream().cuda_stream)

    cur = shard.iterate(s, a, b, iters, sweep)
    assert np.array_equal(cur.cpu().numpy(), O.heat2d(full, iters, r))


def test_single_rank_periodic_exchange_matches_library(gb, torch_cuda):
    torch = torch_cuda
    nz, ny, nx, g = 9, 5, 6, 1
    f = torch.rand((nz + 2, ny + 2, nx + 2), device="cuda")
    a = f.clone()
    shard.Slab(nz, g, periodic=True, rank=0, world=1).exchange(a)
    b = f.clone()
    dims = (ctypes.c_int * 3)(nx + 2, ny + 2, nz + 2)
    gb.call("appfis_gb_ghost_periodic", b.data_ptr(), 4, 3, dims, g, None)
    torch.cuda.synchronize()
    # the library refreshes every axis; compare the z ghost planes' interior rows/columns
    assert torch.equal(a[0, g:-g, g:-g], b[0, g:-g, g:-g]) and torch.equal(a[-1, g:-g, g:-g], b[-1, g:-g, g:-g])
