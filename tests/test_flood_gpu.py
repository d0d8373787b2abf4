"""Batched flood model (Triton) vs the oracle.  FP64 instantiation: follows the reference's
rounding sequence except for cbrt (CUDA's and glibc's may differ in the last bit), so h/qx/qy
and every dt agree with the oracle (the reference's own CPU path, golden fixtures) to 1e-9.  FP32 form:
within its stated error of the FP64 oracle.  Batches of uneven domains: each domain equals its
own single-domain run."""
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


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "triton_*.npz"))), ids=os.path.basename)
def test_golden_fp64(gb, torch_cuda, f):
    g = np.load(f)
    dx, cn, hextra, mann, t_end, pint, ts = [float(v) for v in g["params"]]
    steps = int(g["steps"])
    r = _lib.flood_job([(g["dem"], g["h0"])], dx, cn, hextra, mann, t_end, pint, ts, max_steps=steps, dtype=_lib.F64)
    assert r["steps"][0] == steps
    np.testing.assert_allclose(r["dts"][0], g["dts"], rtol=1e-9)
    for k in ("h", "qx", "qy"):
        np.testing.assert_allclose(r[k][0], g[k], rtol=0, atol=1e-9, err_msg=k)


def test_batch_fp64_each_domain_matches_oracle(gb, torch_cuda):
    sizes = [(40, 52), (17, 90), (65, 33), (128, 70)]
    doms = [W.triton_domain(ny, nx, 500 + k) for k, (ny, nx) in enumerate(sizes)]
    r = _lib.flood_job(doms, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=80, dtype=_lib.F64)
    for k, (dem, h) in enumerate(doms):
        o = O.triton(dem, h, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=80)
        assert r["steps"][k] == o["steps"]
        np.testing.assert_allclose(r["dts"][k], o["dts"], rtol=1e-9)
        np.testing.assert_allclose(r["h"][k], o["h"], atol=1e-9)
        np.testing.assert_allclose(r["qx"][k], o["qx"], atol=1e-9)


def test_runs_to_t_end_with_print_clamp(gb, torch_cuda):
    """Small domains run to t_end = 120 s with a print interval of 50 s: dt is clamped onto 50 and
    100 s (the loop then overshoots 120 s, as the reference's does); steps, every dt, the final
    time and the mass change match the oracle."""
    doms = [W.triton_domain(ny, nx, 900 + k) for k, (ny, nx) in enumerate([(30, 40), (44, 26)])]
    r = _lib.flood_job(doms, 10.0, 0.5, 1e-3, 0.035, 120.0, 50.0, 1.0, max_steps=5000, dtype=_lib.F64)
    for k, (dem, h) in enumerate(doms):
        o = O.triton(dem, h, 10.0, 0.5, 1e-3, 0.035, 120.0, 50.0, 1.0, max_steps=5000)
        assert r["steps"][k] == o["steps"]
        np.testing.assert_allclose(r["dts"][k], o["dts"], rtol=1e-9)
        assert abs(np.sum(r["dts"][k]) - o["simtime"]) < 1e-9
        t = np.cumsum(o["dts"])
        assert np.any(np.abs(t - 50.0) < 1e-12) and np.any(np.abs(t - 100.0) < 1e-12)
        np.testing.assert_allclose(r["h"][k], o["h"], atol=1e-9)
        m0, m1 = r["mass"][k]
        assert abs(m0 - h.sum()) < 1e-9 * h.sum()
        assert abs(m1 - o["h"].sum()) < 1e-9 * h.sum()


def test_fp32_form_error(gb, torch_cuda):
    """FP32 state and arithmetic (FP64 dt min, time and mass): over 100 steps of a dam break on a
    fractal DEM the first steps agree to 1e-5 m, and after 100 steps the L1 depth error stays
    under 2% of the water volume (the differences sit at wet/dry fronts, where float rounding
    flips the hextra / dry thresholds); the mass change agrees with the FP64 oracle's to 1e-5."""
    dem, h = W.triton_domain(96, 128, 31)
    r5 = _lib.flood_job([(dem, h)], 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=3, dtype=_lib.F32)
    o5 = O.triton(dem, h, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=3)
    assert np.abs(r5["h"][0] - o5["h"]).max() < 1e-5
    r = _lib.flood_job([(dem, h)], 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=100, dtype=_lib.F32)
    o = O.triton(dem, h, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=100)
    assert r["steps"][0] == 100
    assert np.abs(r["h"][0] - o["h"]).sum() < 0.02 * o["h"].sum()
    m0, m1 = r["mass"][0]
    assert abs((m1 - m0) - (o["h"].sum() - h.sum())) <= 1e-5 * m0


@pytest.mark.parametrize("dtype", [_lib.F32, _lib.F64])
def test_skip_dry_strips_bit_identical(gb, torch_cuda, dtype):
    """Leaving out exactly dry strips changes no field, step or dt (three domains of uneven
    sizes, some strips never reached by the water, 150 steps)."""
    doms = [W.triton_domain(97, 130, 11), W.triton_domain(64, 61, 12), W.triton_domain(150, 40, 13)]
    full = _lib.flood_job(doms, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=150, dtype=dtype)
    skip = _lib.flood_job(doms, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, max_steps=150, dtype=dtype,
                          flags=_lib.FLOOD_SKIP_DRY)
    assert full["steps"] == skip["steps"]
    for k in range(len(doms)):
        assert np.array_equal(full["h"][k], skip["h"][k])
        assert np.array_equal(full["dts"][k], skip["dts"][k])


@pytest.mark.parametrize("dtype", [_lib.F32, _lib.F64])
def test_fused_step_bit_identical_to_two_phase(gb, torch_cuda, dtype):
    """The fused pass (update, wet/dry fix and next dt in one sweep over 28-column strips whose
    one-cell ring is recomputed) against the two-pass form: every field, step count and dt
    identical.  Domains narrower and shorter than one strip, widths on and off the 28- and
    30-column grids, rows not a multiple of 32, to t_end with the print clamp."""
    doms = [W.triton_domain(97, 130, 11), W.triton_domain(64, 61, 12), W.triton_domain(150, 40, 13), W.triton_domain(5, 3, 14),
            W.triton_domain(33, 56, 15), W.triton_domain(40, 29, 16)]
    args = (10.0, 0.5, 1e-3, 0.035, 300.0, 60.0, 1.0)
    fused = _lib.flood_job(doms, *args, max_steps=2000, dtype=dtype, flags=_lib.FLOOD_FUSED)
    two = _lib.flood_job(doms, *args, max_steps=2000, dtype=dtype, flags=_lib.FLOOD_TWO_PHASE)
    assert fused["steps"] == two["steps"]
    for k in range(len(doms)):
        assert np.array_equal(fused["h"][k], two["h"][k]), k
        assert np.array_equal(fused["qx"][k], two["qx"][k]), k
        assert np.array_equal(fused["qy"][k], two["qy"][k]), k
        assert np.array_equal(fused["dts"][k], two["dts"][k]), k


@pytest.mark.parametrize("dtype", [_lib.F32, _lib.F64])
def test_fused_skip_dry_bit_identical_to_two_phase_skip_dry(gb, torch_cuda, dtype):
    """Dry-strip skipping in the fused pass (28-column strips) against the two-phase form with the
    same skipping (30-column strips): fields, steps and dts identical."""
    doms = [W.triton_domain(97, 130, 11), W.triton_domain(64, 61, 12), W.triton_domain(150, 40, 13)]
    args = (10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0)
    fused = _lib.flood_job(doms, *args, max_steps=150, dtype=dtype, flags=_lib.FLOOD_SKIP_DRY | _lib.FLOOD_FUSED)
    two = _lib.flood_job(doms, *args, max_steps=150, dtype=dtype, flags=_lib.FLOOD_SKIP_DRY | _lib.FLOOD_TWO_PHASE)
    assert fused["steps"] == two["steps"]
    for k in range(len(doms)):
        assert np.array_equal(fused["h"][k], two["h"][k])
        assert np.array_equal(fused["qx"][k], two["qx"][k])
        assert np.array_equal(fused["dts"][k], two["dts"][k])


def test_fused_and_two_phase_flags_exclusive(gb, torch_cuda):
    doms = [W.triton_domain(20, 20, 3)]
    with pytest.raises(_lib.AppfisError):
        _lib.flood_job(doms, 10.0, 0.5, 1e-3, 0.035, 60.0, 60.0, 1.0, max_steps=5,
                       flags=_lib.FLOOD_FUSED | _lib.FLOOD_TWO_PHASE)


def _device_batch(torch, doms, pitch_of, offset=0):
    """FP32 device domains set up from (dem, h) pairs: one buffer of 8 fields per domain (h0 h1
    qx0 qx1 qy0 qy1 dem n2), row pitch pitch_of(nx), each field starting `offset` floats into
    its own slab (an offset that is not a multiple of 4 leaves the rows 4-byte aligned only)."""
    bufs, descs = [], (_lib.FloodDomain * len(doms))()
    for k, (dem, h) in enumerate(doms):
        ny, nx = dem.shape
        pitch = pitch_of(nx)
        slab = pitch * (ny + 2) + 8
        f = torch.zeros(8 * slab, dtype=torch.float32, device="cuda")
        bufs.append(f)
        d = descs[k]
        d.nx, d.ny, d.pitch = nx, ny, pitch
        ptr = [f[m * slab + offset:].data_ptr() for m in range(8)]
        d.h[0], d.h[1], d.qx[0], d.qx[1], d.qy[0], d.qy[1] = ptr[:6]
        d.dem, d.n2 = ptr[6], ptr[7]
        gb_dem = torch.from_numpy(dem).cuda()
        gb_h = torch.from_numpy(h).cuda()
        _lib.call("appfis_gb_flood_setup", ctypes.byref(d), _lib.F32, gb_dem.data_ptr(), gb_h.data_ptr(), None, None, 0.035,
                  None)
        torch.cuda.synchronize()
    return bufs, descs


def _device_run(torch, doms, flags, pitch_of, offset=0, steps=120):
    bufs, descs = _device_batch(torch, doms, pitch_of, offset)
    prm = _lib.FloodParams(10.0, 0.5, 1e-3, 300.0, 60.0, 1.0, 0.0, steps)
    prm.flags = flags
    st = torch.zeros(len(doms), dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    dtlog = torch.zeros(len(doms) * steps, dtype=torch.float64, device="cuda")
    _lib.call("appfis_gb_flood_run", descs, len(doms), _lib.F32, ctypes.byref(prm), dtlog.data_ptr(), st.data_ptr(), None,
              status.data_ptr(), None)
    torch.cuda.synchronize()
    assert int(status.item()) == _lib.OK
    n = st.cpu().numpy()
    out = []
    for k, (dem, _) in enumerate(doms):
        ny, nx = dem.shape
        pitch, slab = pitch_of(nx), pitch_of(nx) * (ny + 2) + 8
        b = int(n[k]) & 1
        f = bufs[k]
        fields = [f[m * slab + offset:m * slab + offset + pitch * (ny + 2)].view(ny + 2, pitch)[1:ny + 1, 1:nx + 1].cpu().numpy()
                  for m in (b, 2 + b, 4 + b)]
        out.append(fields)
    return n.tolist(), out, dtlog.cpu().numpy()


def test_staged_rows_bit_identical_to_row_loads(gb, torch_cuda):
    """The fused FP32 full sweep with its rows staged by TMA (rows 16-byte aligned: pitch a
    multiple of 4) against the same pass loading rows directly (UNSTAGED) and against the
    two-phase form: every field, step count and dt identical.  Widths on and off the 28-column
    strip grid and under one strip, rows not a multiple of 32, domains one row high and shorter
    than a stage."""
    skip = 0
    doms = [W.triton_domain(97, 130, 11), W.triton_domain(64, 61, 12), W.triton_domain(150, 40, 13), W.triton_domain(5, 3, 14),
            W.triton_domain(33, 56, 15), W.triton_domain(40, 29, 16), W.triton_domain(1, 70, 17), W.triton_domain(2, 27, 18)]
    p4 = lambda nx: (nx + 2 + 3) // 4 * 4
    staged = _device_run(torch_cuda, doms, _lib.FLOOD_FUSED | skip, p4)
    rows = _device_run(torch_cuda, doms, _lib.FLOOD_FUSED | _lib.FLOOD_UNSTAGED | skip, p4)
    two = _device_run(torch_cuda, doms, _lib.FLOOD_TWO_PHASE | skip, p4)
    assert staged[0] == rows[0] == two[0]
    assert np.array_equal(staged[2], rows[2]) and np.array_equal(staged[2], two[2])
    for k in range(len(doms)):
        for m in range(3):
            assert np.array_equal(staged[1][k][m], rows[1][k][m]), (k, m)
            assert np.array_equal(staged[1][k][m], two[1][k][m]), (k, m)


def test_unaligned_rows_take_row_loads(gb, torch_cuda):
    """Rows that are not 16-byte aligned (odd pitch, fields 4 bytes off a 16-byte boundary) cannot
    be staged: the fused pass loads them directly and gives the same fields as an aligned run."""
    doms = [W.triton_domain(45, 61, 21), W.triton_domain(30, 33, 22)]
    odd = _device_run(torch_cuda, doms, _lib.FLOOD_FUSED, lambda nx: (nx + 2) | 1, offset=1, steps=60)
    al = _device_run(torch_cuda, doms, _lib.FLOOD_FUSED, lambda nx: (nx + 2 + 3) // 4 * 4, steps=60)
    assert odd[0] == al[0]
    assert np.array_equal(odd[2], al[2])
    for k in range(len(doms)):
        for m in range(3):
            assert np.array_equal(odd[1][k][m], al[1][k][m]), (k, m)
