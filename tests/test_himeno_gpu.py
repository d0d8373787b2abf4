"""Himeno kernels vs the oracle: the FP32 plain form bit-identical to the reference's CPU path
(golden fixture + random coefficient fields), gosa within 1e-12 of the oracle's double sum;
the FP16 defect-correction form within its stated error of the FP64 oracle."""
import ctypes
import glob
import os

import numpy as np
import pytest

from appfis_gb300 import _lib
from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def job(gb, coef, p, iters, form=0, period=20, omega=0.8):
    nz, ny, nx = p.shape[0] - 2, p.shape[1] - 2, p.shape[2] - 2
    out = np.ascontiguousarray(p, dtype=np.float32).copy()
    c = np.ascontiguousarray(coef, dtype=np.float32)
    gosa = np.zeros(max(iters, 1), dtype=np.float64)
    gb.call("appfis_gb_himeno_job", c.ctypes.data, out.ctypes.data, nx, ny, nz, iters, omega, form, period,
            gosa.ctypes.data)
    return out, gosa[:iters]


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "himeno_*.npz"))), ids=os.path.basename)
def test_golden_bit_exact(gb, torch_cuda, f):
    g = np.load(f)
    out, gosa = job(gb, g["coef"], g["p"], int(g["iters"]))
    assert np.array_equal(out, g["out"])
    np.testing.assert_allclose(gosa, g["gosa"], rtol=1e-12)


@pytest.mark.parametrize("nx,ny,nz,iters", [(1, 1, 1, 3), (33, 5, 40, 6), (70, 41, 9, 4), (257, 9, 65, 3)])
def test_random_vs_oracle(gb, torch_cuda, nx, ny, nz, iters):
    coef = W.himeno_coef(nx, ny, nz, seed=nx + ny + nz)
    p = W.himeno_p(nx, ny, nz)
    p[1:-1, 1:-1, 1:-1] += W.uniform(3, nx * ny * nz).reshape(nz, ny, nx).astype(np.float32)
    out, gosa = job(gb, coef, p, iters)
    ref, rgosa = O.himeno(coef, p, iters, 0.8)
    assert np.array_equal(out, ref)
    np.testing.assert_allclose(gosa, rgosa, rtol=1e-12)


def test_device_entry_two_buffers(gb, torch_cuda):
    torch = torch_cuda
    nx, ny, nz, iters = 40, 30, 20, 5
    coef = W.himeno_coef(nx, ny, nz)
    p = W.himeno_p(nx, ny, nz)
    dc = torch.from_numpy(coef).cuda()
    ptrs = (ctypes.c_void_p * 12)(*[dc[k].data_ptr() for k in range(12)])
    pitch = 64  # a padded pitch different from nx+2
    hp = np.zeros((nz + 2, ny + 2, pitch), dtype=np.float32)
    hp[:, :, : nx + 2] = p
    hc = np.zeros((12, nz + 2, ny + 2, pitch), dtype=np.float32)
    hc[..., : nx + 2] = coef
    dc = torch.from_numpy(hc).cuda()
    ptrs = (ctypes.c_void_p * 12)(*[dc[k].data_ptr() for k in range(12)])
    a = torch.from_numpy(hp).cuda()
    b = a.clone()
    g = torch.zeros(iters, dtype=torch.float64, device="cuda")
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_himeno", ptrs, a.data_ptr(), b.data_ptr(), nx, ny, nz, pitch, iters, 0.8, g.data_ptr(),
            ctypes.byref(ci), None)
    out = (a if ci.value == 0 else b).cpu().numpy()[:, :, : nx + 2]
    ref, rg = O.himeno(coef, p, iters, 0.8)
    assert np.array_equal(out, ref)
    np.testing.assert_allclose(g.cpu().numpy(), rg, rtol=1e-12)


def test_mixed_defect_correction_error(gb, torch_cuda):
    """FP16-storage defect correction vs the FP64 oracle on the benchmark's coefficient set:
    p within 2.5e-4 absolute (p is O(1); the plain FP32 form is within 1e-5), gosa within 1%
    relative, per sweep."""
    nx, ny, nz, iters = 65, 65, 129, 60
    coef32 = W.himeno_coef(nx, ny, nz)
    p32 = W.himeno_p(nx, ny, nz)
    p64, g64 = O.himeno(W.himeno_coef(nx, ny, nz, dtype=np.float64), W.himeno_p(nx, ny, nz, dtype=np.float64), iters, 0.8,
                        dtype=np.float64)
    plain, gp = job(gb, coef32, p32, iters, form=0)
    mixed, gm = job(gb, coef32, p32, iters, form=1, period=20)
    err_plain = np.abs(plain - p64).max()
    err_mixed = np.abs(mixed - p64).max()
    assert err_plain < 1e-5
    assert err_mixed < 2.5e-4, err_mixed
    np.testing.assert_allclose(gm, g64, rtol=1e-2)
    np.testing.assert_allclose(gp, g64, rtol=1e-4)


def device_run(gb, torch, coef, p, iters, pitch, form=0, period=20, omega=0.8, spp=0):
    """Runs the device entry point on fields whose rows are padded to `pitch` elements (spp: the
    mixed form's inner sweeps per launch, 0 = its default of one)."""
    nz, ny, nx = p.shape[0] - 2, p.shape[1] - 2, p.shape[2] - 2
    hp = np.zeros((nz + 2, ny + 2, pitch), dtype=np.float32)
    hp[:, :, : nx + 2] = p
    hc = np.zeros((12, nz + 2, ny + 2, pitch), dtype=np.float32)
    hc[..., : nx + 2] = coef
    dc = torch.from_numpy(hc).cuda()
    ptrs = (ctypes.c_void_p * 12)(*[dc[k].data_ptr() for k in range(12)])
    a = torch.from_numpy(hp).cuda()
    b = a.clone()
    g = torch.zeros(max(iters, 1), dtype=torch.float64, device="cuda")
    ci = ctypes.c_int(-1)
    if form == 0:
        gb.call("appfis_gb_himeno", ptrs, a.data_ptr(), b.data_ptr(), nx, ny, nz, pitch, iters, omega, g.data_ptr(),
                ctypes.byref(ci), None)
    else:
        half = torch.empty(13 * hp.size, dtype=torch.float16, device="cuda")
        gb.call("appfis_gb_himeno_mixed_ex", ptrs, a.data_ptr(), b.data_ptr(), half.data_ptr(), nx, ny, nz, pitch, iters,
                period, omega, spp, g.data_ptr(), ctypes.byref(ci), None)
    gb.call("appfis_gb_stream_sync", None)
    out = (a if ci.value == 0 else b).cpu().numpy()[:, :, : nx + 2]
    return out, g.cpu().numpy()[:iters]


# 16-byte aligned rows select the TMA-staged kernels: ragged x tiles (the first tile starts at the
# ghost column), y not a multiple of 8, z chunks of unequal length, tiny grids
@pytest.mark.parametrize("nx,ny,nz,pitch,iters", [(1, 1, 1, 8, 3), (30, 7, 5, 32, 4), (31, 9, 33, 40, 5),
                                                  (64, 17, 70, 72, 3), (95, 8, 64, 104, 2)])
def test_tma_plain_bit_exact(gb, torch_cuda, nx, ny, nz, pitch, iters):
    coef = W.himeno_coef(nx, ny, nz, seed=3 * nx + ny)
    p = W.himeno_p(nx, ny, nz)
    p[1:-1, 1:-1, 1:-1] += W.uniform(5, nx * ny * nz).reshape(nz, ny, nx).astype(np.float32)
    out, gosa = device_run(gb, torch_cuda, coef, p, iters, pitch)
    ref, rgosa = O.himeno(coef, p, iters, 0.8)
    assert np.array_equal(out, ref)
    np.testing.assert_allclose(gosa, rgosa, rtol=1e-12)


def test_tma_and_dense_rows_agree(gb, torch_cuda):
    """The same sweep on dense rows (register-prefetch kernel) and on padded rows (TMA kernel)."""
    nx, ny, nz, iters = 45, 19, 37, 4
    coef = W.himeno_coef(nx, ny, nz, seed=11)
    p = W.himeno_p(nx, ny, nz)
    dense, gd = device_run(gb, torch_cuda, coef, p, iters, nx + 2)   # 47: not 16-byte rows
    padded, gp = device_run(gb, torch_cuda, coef, p, iters, 48)
    assert np.array_equal(dense, padded)
    np.testing.assert_allclose(gd, gp, rtol=1e-12)


@pytest.mark.parametrize("pitch", [67, 72])  # register-prefetch kernel, TMA kernel
def test_mixed_error_both_kernels(gb, torch_cuda, pitch):
    """FP16 defect correction on both inner-sweep kernels: p within 2.5e-4 of the FP64 oracle,
    gosa within 1% per sweep."""
    nx, ny, nz, iters = 65, 33, 47, 40
    p64, g64 = O.himeno(W.himeno_coef(nx, ny, nz, dtype=np.float64), W.himeno_p(nx, ny, nz, dtype=np.float64), iters, 0.8,
                        dtype=np.float64)
    mixed, gm = device_run(gb, torch_cuda, W.himeno_coef(nx, ny, nz), W.himeno_p(nx, ny, nz), iters, pitch, form=1)
    assert np.abs(mixed - p64).max() < 2.5e-4
    np.testing.assert_allclose(gm, g64, rtol=1e-2)


@pytest.mark.parametrize("nx", [64, 66, 79, 129, 143, 200, 255])
def test_mixed_tile_widths(gb, torch_cuda, nx):
    """The TMA inner sweep takes 72-wide tiles where their whole tiles overhang columns 0..nx+1
    less than 64-wide ones (nx 64, 66, 129, 143, 200) and 64-wide tiles otherwise (79, 255),
    with one or several tiles across: p within the mixed form's 2.5e-4 of the FP64 oracle and
    gosa within 1% per sweep."""
    ny, nz, iters = 21, 30, 25
    pitch = (nx + 2 + 7) // 8 * 8
    p64, g64 = O.himeno(W.himeno_coef(nx, ny, nz, dtype=np.float64), W.himeno_p(nx, ny, nz, dtype=np.float64), iters, 0.8,
                        dtype=np.float64)
    mixed, gm = device_run(gb, torch_cuda, W.himeno_coef(nx, ny, nz), W.himeno_p(nx, ny, nz), iters, pitch, form=1)
    assert np.abs(mixed - p64).max() < 2.5e-4
    np.testing.assert_allclose(gm, g64, rtol=1e-2)


@pytest.mark.parametrize("nx,ny,nz,iters,period", [(1, 1, 1, 4, 20), (30, 7, 5, 6, 20), (55, 9, 33, 7, 3), (56, 16, 70, 9, 4),
                                                   (57, 17, 64, 10, 20), (129, 23, 129, 12, 5), (257, 33, 40, 8, 20)])
def test_mixed_two_sweeps_per_pass_bit_identical(gb, torch_cuda, nx, ny, nz, iters, period):
    """Two inner sweeps per launch (56 x 8 tiles with the one-point ring recomputed, level-1
    values rounded through FP16) against one sweep per launch: p bit-identical after corrections
    and odd leftovers (periods of 3 and 5 end with a single sweep), gosa within 1e-5 (the same
    per-point squares summed in another grouping); ragged x tiles, y not a multiple of 8, z
    chunks of one plane."""
    pitch = (nx + 2 + 7) // 8 * 8
    coef, p = W.himeno_coef(nx, ny, nz, seed=nx + 5 * nz), W.himeno_p(nx, ny, nz)
    one, g1 = device_run(gb, torch_cuda, coef, p, iters, pitch, form=1, period=period, spp=1)
    two, g2 = device_run(gb, torch_cuda, coef, p, iters, pitch, form=1, period=period, spp=2)
    assert np.array_equal(one, two)
    np.testing.assert_allclose(g2, g1, rtol=1e-5, atol=0)


def test_mixed_two_sweeps_needs_aligned_rows(gb, torch_cuda):
    nx, ny, nz = 13, 5, 4
    with pytest.raises(_lib.AppfisError):
        device_run(gb, torch_cuda, W.himeno_coef(nx, ny, nz), W.himeno_p(nx, ny, nz), 2, nx + 2, form=1, spp=2)


@pytest.mark.parametrize("iters,period", [(1, 20), (2, 1), (3, 2), (5, 2), (7, 3)])
@pytest.mark.parametrize("spp", [1, 2])
def test_mixed_short_runs_and_periods(gb, torch_cuda, iters, period, spp):
    """Each correction pass also does its period's first inner sweep (from e = 0 it gives e = D);
    short runs and short periods (every sweep such a first one at period 1) against the FP64
    oracle: p within the mixed form's 2.5e-4, gosa of every sweep within 1%."""
    nx, ny, nz = 40, 13, 11
    pitch = (nx + 2 + 7) // 8 * 8
    p64, g64 = O.himeno(W.himeno_coef(nx, ny, nz, dtype=np.float64), W.himeno_p(nx, ny, nz, dtype=np.float64), iters, 0.8,
                        dtype=np.float64)
    mixed, gm = device_run(gb, torch_cuda, W.himeno_coef(nx, ny, nz), W.himeno_p(nx, ny, nz), iters, pitch, form=1, period=period,
                           spp=spp)
    assert np.abs(mixed - p64).max() < 2.5e-4
    np.testing.assert_allclose(gm, g64, rtol=1e-2)


def test_mixed_zero_sweeps_leaves_p(gb, torch_cuda):
    nx, ny, nz = 30, 9, 7
    p = W.himeno_p(nx, ny, nz)
    out, _ = device_run(gb, torch_cuda, W.himeno_coef(nx, ny, nz), p, 0, 32, form=1)
    assert np.array_equal(out, p)
