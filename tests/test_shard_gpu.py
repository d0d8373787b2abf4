"""The sharded driver on one GPU: the slab iteration with the C-ABI heat sweep (one exchange per
sweep, and one per 8 sweeps with the time-blocked kernel) reproduces the oracle bit-for-bit, and
the single-rank periodic exchange equals the library's periodic ghost refresh along the slowest
axis."""
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


def test_blocked_slab_iteration_with_time_blocked_kernel(gb, torch_cuda):
    """iterate_blocked with an 8-deep halo and the heat kernel that does several sweeps per launch
    on chip (appfis_gb_heat2d, 8 per launch): one exchange per 8 sweeps, bit-identical to the
    oracle."""
    torch = torch_cuda
    nx, ny, iters, r, g = 45, 33, 20, 0.2, 8
    core = W.heat2d_padded(nx, ny, 1.0, 3)
    full = np.concatenate([np.repeat(core[:1], g - 1, 0), core, np.repeat(core[-1:], g - 1, 0)])
    s = shard.Slab(ny, g, rank=0, world=1)
    a = s.scatter(torch.from_numpy(full)).cuda()
    b = a.clone()
    ci = ctypes.c_int(-1)

    def sweep_layers(cur, nxt, k, lo, hi):
        nxt.copy_(cur)
        x, y = cur[lo - 1:], nxt[lo - 1:]
        gb.call("appfis_gb_heat2d", x.data_ptr(), y.data_ptr(), nx, hi - lo, nx + 2, k, r, r, ctypes.byref(ci),
                torch.cuda.current_stream().cuda_stream)
        return cur if ci.value == 0 else nxt

    cur = shard.iterate_blocked(s, a, b, iters, sweep_layers, g)
    assert np.array_equal(cur.cpu().numpy()[g - 1:g + ny + 1], O.heat2d(core, iters, r))


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
