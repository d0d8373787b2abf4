"""GameOfLife kernels vs the oracle: bit-exact states and populations (u8 generic, u8 SWAR,
bit-packed), both rules, pack/unpack round trip, the host-buffer job, and full-size
properties (u8 and bit-packed forms agree on the 16384^2 grid)."""
import ctypes
import glob
import os

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def run_u8(gb, torch, cells, gens, rule=0, old=None):
    ny, nx = cells.shape
    a = torch.from_numpy(np.ascontiguousarray(cells)).cuda()
    b = torch.zeros_like(a) if old is None else torch.from_numpy(np.ascontiguousarray(old)).cuda()
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_life_u8", a.data_ptr(), b.data_ptr(), nx, ny, gens, rule, ctypes.byref(ci), None)
    torch.cuda.synchronize()
    cur, prev = (a, b) if ci.value == 0 else (b, a)
    return cur.cpu().numpy(), prev.cpu().numpy()


def run_bits(gb, torch, cells, gens, rule=0):
    ny, nx = cells.shape
    c = torch.from_numpy(np.ascontiguousarray(cells)).cuda()
    wa = torch.zeros(ny * nx // 32, dtype=torch.int32, device="cuda")
    wb = torch.zeros_like(wa)
    gb.call("appfis_gb_life_pack", c.data_ptr(), wa.data_ptr(), nx, ny, None)
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_life_bits", wa.data_ptr(), wb.data_ptr(), nx, ny, gens, rule, ctypes.byref(ci), None)
    latest = wa if ci.value == 0 else wb
    out = torch.empty_like(c)
    gb.call("appfis_gb_life_unpack", latest.data_ptr(), out.data_ptr(), nx, ny, None)
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    gb.call("appfis_gb_life_population_bits", latest.data_ptr(), ny * nx // 32, cnt.data_ptr(), None)
    torch.cuda.synchronize()
    return out.cpu().numpy(), int(cnt.item())


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "gol_*.npz"))), ids=os.path.basename)
def test_golden(gb, torch_cuda, f):
    g = np.load(f)
    cur, _ = run_u8(gb, torch_cuda, g["cells"], int(g["gens"]))
    assert np.array_equal(cur, g["out"])
    if g["cells"].shape[1] % 32 == 0:
        out, pop = run_bits(gb, torch_cuda, g["cells"], int(g["gens"]))
        assert np.array_equal(out, g["out"]) and pop == int(g["live"])


# nx a multiple of 16 runs the bulk-staged sweep: one strip narrower than 4096 cells (16, 48, 512,
# 1040), exactly one strip (4096), a second strip of 16 cells (4112) and of 512 cells (8704)
@pytest.mark.parametrize("nx,ny,gens", [(37, 29, 7), (1, 5, 3), (5, 1, 4), (16, 16, 9), (512, 48, 13), (1040, 70, 6),
                                        (4096, 65, 5), (48, 131, 12), (4112, 33, 9), (8704, 40, 4)])
@pytest.mark.parametrize("rule", [0, 1])
def test_u8_vs_oracle(gb, torch_cuda, nx, ny, gens, rule):
    cells = W.gol_cells(nx, ny, 0.35, nx * 7 + ny)
    cur, prev = run_u8(gb, torch_cuda, cells, gens, rule)
    if rule == 0:
        ocur, oprev = O.gol(cells, gens)
        assert np.array_equal(cur, ocur)
        assert np.array_equal(prev, oprev)
    else:
        assert np.array_equal(cur, O.gol_b3s23(cells, gens))


# 16+ generations run the time-blocked kernel: 30-word tile columns (1056 = 33 words: a second
# column of 3 words; 960 = exactly one column; 32 = one word, fewer rows than the row halo),
# partial last row tiles, 1-7 time-blocked launches (odd counts of 3 or more go round three
# buffer pairs before ping-ponging) plus a remainder.
@pytest.mark.parametrize("nx,ny,gens", [(32, 1, 3), (32, 7, 5), (64, 40, 11), (1056, 66, 9), (2048, 130, 8), (96, 257, 21),
                                        (1056, 300, 33), (960, 70, 16), (32, 20, 16), (2048, 700, 48), (160, 1100, 17),
                                        (256, 300, 80), (320, 140, 85), (128, 64, 112), (64, 520, 64), (992, 90, 32),
                                        (1984, 40, 16), (1024, 33, 17)])
@pytest.mark.parametrize("rule", [0, 1])
def test_bits_vs_oracle(gb, torch_cuda, nx, ny, gens, rule):
    cells = W.gol_cells(nx, ny, 0.3, nx + 3 * ny)
    out, pop = run_bits(gb, torch_cuda, cells, gens, rule)
    ref = O.gol(cells, gens)[0] if rule == 0 else O.gol_b3s23(cells, gens)
    assert np.array_equal(out, ref)
    assert pop == int(ref.sum())


def test_pack_unpack_roundtrip(gb, torch_cuda):
    cells = W.gol_cells(256, 33, 0.5, 4)
    out, pop = run_bits(gb, torch_cuda, cells, 0)
    assert np.array_equal(out, cells) and pop == int(cells.sum())


def test_population_u8_ragged(gb, torch_cuda):
    for n in (1, 3, 4, 1001, 1 << 20):
        c = W.bernoulli_u8(n, n, 0.4)
        t = torch_cuda.from_numpy(c).cuda()
        cnt = torch_cuda.zeros(1, dtype=torch_cuda.int64, device="cuda")
        gb.call("appfis_gb_life_population_u8", t.data_ptr(), n, cnt.data_ptr(), None)
        assert int(cnt.item()) == int(c.sum())


@pytest.mark.parametrize("form", [0, 1])
def test_job_host_buffers(gb, torch_cuda, form):
    nx, ny, gens = 1024, 96, 25
    cells = W.gol_cells(nx, ny, 0.3, 77)
    out = np.zeros_like(cells)
    pop = ctypes.c_int64(-1)
    gb.call("appfis_gb_life_job", cells.ctypes.data, out.ctypes.data, nx, ny, gens, 0, form, ctypes.byref(pop))
    ref, _ = O.gol(cells, gens)
    assert np.array_equal(out, ref)
    assert pop.value == int(ref.sum())


@pytest.mark.parametrize("alias", [False, True])
def test_job_page_locked_buffers(gb, torch_cuda, alias):
    """Bit-packed form from page-locked host buffers (the bench's end-to-end case), also with the
    output buffer over the input."""
    torch = torch_cuda
    nx, ny, gens = 2048, 130, 37
    cells = W.gol_cells(nx, ny, 0.3, 78)
    hin = torch.from_numpy(cells).pin_memory()
    hout = hin if alias else torch.zeros_like(hin).pin_memory()
    pop = ctypes.c_int64(-1)
    gb.call("appfis_gb_life_job", hin.data_ptr(), hout.data_ptr(), nx, ny, gens, 0, 1, ctypes.byref(pop))
    ref, _ = O.gol(cells, gens)
    assert np.array_equal(hout.numpy(), ref)
    assert pop.value == int(ref.sum())


def test_full_size_forms_agree(gb, torch_cuda):
    """16384^2 (the benchmark grid), 36 generations (two time-blocked launches of 16, then 4
    single sweeps): the u8 and bit-packed forms give identical states, the population matches a
    host count, and 18+18 generations equal 36 (restart)."""
    nx = ny = 16384
    cells = W.gol_cells(nx, ny, 0.3, 42)
    a8 = np.zeros_like(cells)
    ab = np.zeros_like(cells)
    p8 = ctypes.c_int64(-1)
    pb = ctypes.c_int64(-2)
    gb.call("appfis_gb_life_job", cells.ctypes.data, a8.ctypes.data, nx, ny, 36, 0, 0, ctypes.byref(p8))
    gb.call("appfis_gb_life_job", cells.ctypes.data, ab.ctypes.data, nx, ny, 36, 0, 1, ctypes.byref(pb))
    assert np.array_equal(a8, ab)
    assert p8.value == pb.value == int(a8.sum(dtype=np.int64))
    cur, prev = run_u8(gb, torch_cuda, cells, 18)
    cur2, _ = run_u8(gb, torch_cuda, cur, 18, old=prev)
    assert np.array_equal(cur2, a8)


@pytest.mark.parametrize("rule", [0, 1])
def test_large_ragged_columns_forms_agree(gb, torch_cuda, rule):
    """15904 x 12000 (497 words: 16 full 30-word columns and one of 17 words; 47 row tiles, the
    last of 224 rows), 32 generations: bit-packed and u8 forms agree (the u8 form is pinned to
    the oracle above)."""
    nx, ny = 15904, 12000
    cells = W.gol_cells(nx, ny, 0.3, 9)
    a8 = np.zeros_like(cells)
    ab = np.zeros_like(cells)
    p8 = ctypes.c_int64(-1)
    pb = ctypes.c_int64(-2)
    gb.call("appfis_gb_life_job", cells.ctypes.data, a8.ctypes.data, nx, ny, 32, rule, 0, ctypes.byref(p8))
    gb.call("appfis_gb_life_job", cells.ctypes.data, ab.ctypes.data, nx, ny, 32, rule, 1, ctypes.byref(pb))
    assert np.array_equal(a8, ab)
    assert p8.value == pb.value
