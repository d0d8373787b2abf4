"""Radius-4 star (FDTD3d) kernels vs the oracle: the reference form bit-identical (golden
fixture from the reference, odd sizes), the weighted form within FP32 rounding of the FP32
oracle, the FP16-storage form within its stated error of the FP64 oracle."""
import ctypes
import glob
import os

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def run(gb, torch, padded, iters, mode, coeff=0.1, weights=None, dtype="f32", pitch=None, ry=0, kz=0):
    nz, ny, nx = padded.shape[0] - 8, padded.shape[1] - 8, padded.shape[2] - 8
    pitch = pitch or nx + 8
    host = np.zeros(padded.shape[:2] + (pitch,), dtype=np.float32)
    host[..., : nx + 8] = padded
    tdt = torch.float32 if dtype == "f32" else torch.float16
    a = torch.from_numpy(host).cuda().to(tdt)
    b = a.clone()
    w = None if weights is None else (ctypes.c_float * 5)(*weights)
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_star_r4", a.data_ptr(), b.data_ptr(), 0 if dtype == "f32" else 3, nx, ny, nz, pitch, iters, mode,
            coeff, w, ry, kz, ctypes.byref(ci), None)
    out = (a if ci.value == 0 else b).float().cpu().numpy()
    return out[..., : nx + 8]


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "fdtd_*.npz"))), ids=os.path.basename)
def test_golden_reference_form(gb, torch_cuda, f):
    g = np.load(f)
    out = run(gb, torch_cuda, g["padded"], int(g["iters"]), 0, float(g["coeff"]))
    assert np.array_equal(out, g["out"])


@pytest.mark.parametrize("nx,ny,nz,iters,ry,kz,pitch", [(1, 1, 1, 2, 0, 0, None), (37, 29, 11, 3, 4, 0, None),
                                                        (64, 70, 33, 2, 2, 16, 80), (33, 17, 130, 2, 4, 64, None),
                                                        (100, 3, 5, 4, 2, 3, 112),
                                                        # TMA-staged tile (16-byte rows): aligned, ragged x, ragged y/z,
                                                        # short z chunks, a single plane
                                                        (64, 70, 33, 2, 0, 16, 72), (37, 29, 11, 3, 0, 0, 48),
                                                        (130, 17, 21, 2, 0, 8, 140), (4, 1, 2, 3, 0, 0, 12),
                                                        (70, 35, 19, 3, 0, 5, 80), (9, 16, 1, 2, 0, 0, 20)])
def test_reference_form_vs_oracle(gb, torch_cuda, nx, ny, nz, iters, ry, kz, pitch):
    f = W.fdtd_padded(nx, ny, nz, nx * ny + nz)
    out = run(gb, torch_cuda, f, iters, 0, 0.1, pitch=pitch, ry=ry, kz=kz)
    assert np.array_equal(out, O.star_r4(f, iters, coeff=0.1))


TMA_X4, TMA_X2, VEC, TMA_X4R4 = 8, 9, 10, 13  # APPFIS_GB_STAR_* tiles


@pytest.mark.parametrize("tile", [TMA_X4, TMA_X2, VEC, TMA_X4R4])
@pytest.mark.parametrize("nx,ny,nz,iters,kz,pitch", [(64, 70, 33, 2, 16, 72), (37, 29, 11, 3, 0, 48), (3, 17, 9, 2, 4, 12),
                                                     (95, 9, 20, 2, 0, 104)])
def test_every_tile_reference_form(gb, torch_cuda, tile, nx, ny, nz, iters, kz, pitch):
    f = W.fdtd_padded(nx, ny, nz, 3 * nx + nz)
    out = run(gb, torch_cuda, f, iters, 0, 0.1, pitch=pitch, ry=tile, kz=kz)
    assert np.array_equal(out, O.star_r4(f, iters, coeff=0.1))


@pytest.mark.parametrize("tile", [TMA_X4, TMA_X2, TMA_X4R4])
def test_tma_tiles_fp16_weighted(gb, torch_cuda, tile):
    w = W.fdtd_weights()
    f = W.fdtd_padded(70, 33, 21, 17)
    a = run(gb, torch_cuda, f, 5, 1, weights=w, dtype="f16", pitch=80, ry=tile)
    ref64 = O.star_r4(f.astype(np.float64), 5, weights=w, dtype=np.float64)
    assert np.abs(a - ref64).max() < 2e-3


def test_tile_needs_aligned_rows(gb, torch_cuda):
    f = W.fdtd_padded(9, 5, 3, 1)
    with pytest.raises(RuntimeError):
        run(gb, torch_cuda, f, 1, 0, 0.1, pitch=18, ry=TMA_X2)  # 72-byte rows


def test_weighted_form_vs_oracle(gb, torch_cuda):
    w = W.fdtd_weights()
    f = W.fdtd_padded(48, 40, 36, 5)
    out = run(gb, torch_cuda, f, 10, 1, weights=w)
    ref32 = O.star_r4(f, 10, weights=w)
    ref64 = O.star_r4(f.astype(np.float64), 10, weights=w, dtype=np.float64)
    assert np.abs(out - ref32).max() < 1e-5
    assert np.abs(out - ref64).max() < 1e-5
    assert np.all(out[:4] == 0) and np.all(out[..., :4] == 0)  # halo untouched


# scalar tile, TMA-staged tile (rows of 72 halves = 144 B), register-staged vector tile (76 halves)
@pytest.mark.parametrize("pitch,ry", [(None, 2), (72, 0), (76, 0)])
def test_fp16_tiles_agree(gb, torch_cuda, pitch, ry):
    w = W.fdtd_weights()
    f = W.fdtd_padded(64, 40, 24, 13)
    a = run(gb, torch_cuda, f, 6, 1, weights=w, dtype="f16", pitch=pitch, ry=ry)
    ref64 = O.star_r4(f.astype(np.float64), 6, weights=w, dtype=np.float64)
    assert np.abs(a - ref64).max() < 2e-3


def test_fp16_storage_error(gb, torch_cuda):
    """FP16 storage, FP32 arithmetic, 50 steps of u <- u + nu*L8(u): max error vs FP64 < 2e-3
    (inputs in [-1, 1]); the FP32 form stays within 1e-5."""
    w = W.fdtd_weights()
    f = W.fdtd_padded(64, 64, 64, 9)
    ref64 = O.star_r4(f.astype(np.float64), 50, weights=w, dtype=np.float64)
    o32 = run(gb, torch_cuda, f, 50, 1, weights=w)
    o16 = run(gb, torch_cuda, f, 50, 1, weights=w, dtype="f16")
    assert np.abs(o32 - ref64).max() < 1e-5
    assert np.abs(o16 - ref64).max() < 2e-3


def test_fp16_tma_and_vector_tiles_agree(gb, torch_cuda):
    """Same FP32 arithmetic on FP16 storage: the TMA-staged and register-staged tiles agree."""
    w = W.fdtd_weights()
    f = W.fdtd_padded(61, 23, 17, 21)
    a = run(gb, torch_cuda, f, 4, 1, weights=w, dtype="f16", pitch=72)
    b = run(gb, torch_cuda, f, 4, 1, weights=w, dtype="f16", pitch=76)
    assert np.abs(a - b).max() <= 1e-3


TB2, TB2_8 = 11, 12  # time-blocked tiles: two steps per launch (64 x 16 / 64 x 8 output tiles)


@pytest.mark.parametrize("tile", [TB2, TB2_8])
@pytest.mark.parametrize("nx,ny,nz,iters,kz,pitch", [(64, 70, 33, 2, 16, 72), (37, 29, 11, 3, 0, 48), (130, 17, 21, 4, 8, 140),
                                                     (9, 16, 1, 2, 0, 20), (64, 16, 40, 6, 0, 72), (4, 1, 2, 5, 0, 12),
                                                     (200, 45, 70, 4, 24, 208)])
def test_time_blocked_reference_form_vs_oracle(gb, torch_cuda, tile, nx, ny, nz, iters, kz, pitch):
    """Two steps per launch (an odd last step in the single-step tile): bit-identical to the
    oracle's step-by-step run of the reference form — aligned and ragged x / y / z, short z
    chunks, a single plane, odd and even step counts."""
    f = W.fdtd_padded(nx, ny, nz, 5 * nx + nz)
    out = run(gb, torch_cuda, f, iters, 0, 0.1, pitch=pitch, ry=tile, kz=kz)
    assert np.array_equal(out, O.star_r4(f, iters, coeff=0.1))


@pytest.mark.parametrize("tile", [TB2, TB2_8])
def test_time_blocked_weighted_equals_single_step(gb, torch_cuda, tile):
    """The weighted form in FP32: the time-blocked tile does the single-step tile's arithmetic in
    the same order, so 6 steps agree bit for bit."""
    w = W.fdtd_weights()
    f = W.fdtd_padded(96, 40, 30, 23)
    a = run(gb, torch_cuda, f, 6, 1, weights=w, pitch=104, ry=tile)
    b = run(gb, torch_cuda, f, 6, 1, weights=w, pitch=104, ry=TMA_X4)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("tile", [TB2, TB2_8])
def test_time_blocked_fp16_error(gb, torch_cuda, tile):
    """FP16 storage with the step-1 values kept in FP32 on chip: within the FP16 form's 2e-3 of
    the FP64 oracle after 50 steps."""
    w = W.fdtd_weights()
    f = W.fdtd_padded(64, 64, 64, 9)
    ref64 = O.star_r4(f.astype(np.float64), 50, weights=w, dtype=np.float64)
    o16 = run(gb, torch_cuda, f, 50, 1, weights=w, dtype="f16", ry=tile)
    assert np.abs(o16 - ref64).max() < 2e-3


def test_autotuner_choice_is_used_and_exact(gb, torch_cuda):
    """appfis_gb_star_r4_tune times the candidates from a into b (a and the halo untouched),
    returns a tile of the aligned-row set, and AUTO then runs that choice: the reference form
    stays bit-identical to the oracle."""
    torch = torch_cuda
    nx, ny, nz, pitch = 96, 40, 70, 104
    f = W.fdtd_padded(nx, ny, nz, 77)
    host = np.zeros(f.shape[:2] + (pitch,), dtype=np.float32)
    host[..., : nx + 8] = f
    a = torch.from_numpy(host).cuda()
    b = a.clone()
    tile, kz, ms = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_float(-1)
    gb.call("appfis_gb_star_r4_tune", a.data_ptr(), b.data_ptr(), 0, nx, ny, nz, pitch, 0, 0.1, None, ctypes.byref(tile),
            ctypes.byref(kz), ctypes.byref(ms), None)
    assert tile.value in (TMA_X4, TMA_X2, TB2, TB2_8, TMA_X4R4) and kz.value >= 0 and ms.value > 0
    assert torch.equal(a, torch.from_numpy(host).cuda())  # the input was not written
    out = run(gb, torch_cuda, f, 5, 0, 0.1, pitch=pitch, ry=0)
    assert np.array_equal(out, O.star_r4(f, 5, coeff=0.1))


def test_four_row_tile_weighted_equals_two_row_tile(gb, torch_cuda):
    """The 64 x 32 tile (4 rows per thread) does the 64 x 16 tile's per-point arithmetic: the
    weighted form agrees bit for bit, ragged y included."""
    w = W.fdtd_weights()
    f = W.fdtd_padded(96, 45, 30, 29)
    a = run(gb, torch_cuda, f, 5, 1, weights=w, pitch=104, ry=TMA_X4R4)
    b = run(gb, torch_cuda, f, 5, 1, weights=w, pitch=104, ry=TMA_X4)
    assert np.array_equal(a, b)
