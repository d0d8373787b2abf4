"""2-D heat kernels vs the oracle and the reference's golden outputs: bit-identical fields
(same rounding sequence), time-blocked launches equal one-sweep launches, job stats."""
import ctypes
import glob
import os

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def dev_pair(torch, padded, pitch=None):
    ny2, nx2 = padded.shape
    pitch = pitch or nx2
    host = np.zeros((ny2, pitch), dtype=np.float32)
    host[:, :nx2] = padded
    a = torch.from_numpy(host).cuda()
    return a, a.clone(), pitch


def run_blocked(gb, torch, padded, iters, pitch=None, r=0.2):
    ny, nx = padded.shape[0] - 2, padded.shape[1] - 2
    a, b, pitch = dev_pair(torch, padded, pitch)
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_heat2d", a.data_ptr(), b.data_ptr(), nx, ny, pitch, iters, r, r, ctypes.byref(ci), None)
    torch.cuda.synchronize()
    return (a if ci.value == 0 else b).cpu().numpy()[:, : nx + 2]


def run_sweeps(gb, torch, padded, iters, r=0.2):
    ny, nx = padded.shape[0] - 2, padded.shape[1] - 2
    a, b, pitch = dev_pair(torch, padded)
    for _ in range(iters):
        gb.call("appfis_gb_heat2d_sweep", a.data_ptr(), b.data_ptr(), nx, ny, pitch, r, r, None)
        a, b = b, a
    torch.cuda.synchronize()
    return a.cpu().numpy()


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "heat2d_*.npz"))), ids=os.path.basename)
def test_golden_bit_exact(gb, torch_cuda, f):
    g = np.load(f)
    out = run_blocked(gb, torch_cuda, g["padded"], int(g["iters"]))
    assert np.array_equal(out, g["out"])
    assert np.array_equal(run_sweeps(gb, torch_cuda, g["padded"], int(g["iters"])), g["out"])


@pytest.mark.parametrize("nx,ny,iters,pitch", [(1, 1, 5, None), (3, 70, 9, None), (100, 37, 23, 128), (130, 65, 8, None),
                                               (64, 32, 1, None), (257, 129, 17, 288)])
def test_vs_oracle(gb, torch_cuda, nx, ny, iters, pitch):
    f = W.heat2d_padded(nx, ny, 1.0, nx + ny)
    f[:, 0] = 0.25  # a LEFT face value too
    ref = O.heat2d(f, iters, 0.2)
    assert np.array_equal(run_blocked(gb, torch_cuda, f, iters, pitch), ref)


def test_full_size_job_bit_exact(gb, torch_cuda):
    """The benchmark case (1024^2, 1000 iterations) through the host-buffer job: bit-identical
    to the oracle, and the MAX/MIN/SUM stats agree (SUM within double-vs-float accumulation)."""
    c = W.HEAT2D
    f = W.heat2d_padded(c["nx"], c["ny"], c["top"], c["seed"])
    ref = O.heat2d(f, c["iters"], c["r"])
    out = f.copy()
    stats = (ctypes.c_double * 3)()
    gb.call("appfis_gb_heat2d_job", out.ctypes.data, c["nx"], c["ny"], c["iters"], c["r"], c["r"], stats)
    assert np.array_equal(out, ref)
    box = (1, c["nx"] + 1, 1, c["ny"] + 1)
    assert stats[0] == O.reduce(ref, box, "max")
    assert stats[1] == O.reduce(ref, box, "min")
    np.testing.assert_allclose(stats[2], ref[1:-1, 1:-1].astype(np.float64).sum(), rtol=1e-12)
