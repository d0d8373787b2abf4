"""Parity at the benchmark configurations' full sizes.

* GameOfLife 16384^2, 2000 generations (the headline workload): the final state of both GPU
  forms (bit-packed, u8) hashes to what the reference's own CPU path produced for the same input
  (tests/golden/gol_16384x16384_g2000.json, written by make_golden.py --full-gol), and the
  population is the reference's.
* The FP64 sweeps are pinned to the FP64 oracle at full size (bit-identical fields over a few
  sweeps; they are deterministic, so every further sweep is the same function), then stand in
  for the oracle over the whole run: Heat2D 1024^2 x 1000, Himeno 257x257x513 x 400 and FDTD
  512^3 x 200 state the error of each FP32 / FP16 / mixed form against them, within the bounds
  written in each test.
* Flood: the FP32 batch against the FP64 batch (which matches the reference to 1e-9) to
  t = 600 s on a subset of the 32 domains."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from appfis_gb300 import _lib
from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _err(x, ref):
    d = x.double() - ref
    return float(d.abs().max().item()), float((d.norm() / ref.norm()).item())


@pytest.mark.parametrize("form", [_lib.FORM_BITS, _lib.FORM_U8])
def test_gol_2000_generations_equal_reference_cpu_path(gb, torch_cuda, form):
    rec = json.load(open(os.path.join(GOLD, "gol_16384x16384_g2000.json")))
    nx, ny, gens = rec["nx"], rec["ny"], rec["gens"]
    cells = W.gol_cells(nx, ny, rec["p"], rec["seed"])
    assert hashlib.sha256(cells.tobytes()).hexdigest() == rec["input_sha256"]
    out = np.empty_like(cells)
    pop = ctypes.c_int64(-1)
    gb.call("appfis_gb_life_job", cells.ctypes.data, out.ctypes.data, nx, ny, gens, _lib.LIFE_REFERENCE, form, ctypes.byref(pop))
    assert pop.value == rec["live"]
    assert hashlib.sha256(out.tobytes()).hexdigest() == rec["sha256"]


def test_heat2d_full_size_fp64_pinned_and_fp32_error(gb, torch_cuda):
    torch = torch_cuda
    c = W.HEAT2D
    nx, ny, it = c["nx"], c["ny"], c["iters"]
    f64 = W.heat2d_padded(nx, ny, c["top"], c["seed"]).astype(np.float64)
    ref = O.heat2d(f64, it, c["r"], dtype=np.float64)
    a = torch.from_numpy(f64).cuda()
    b = a.clone()
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_heat2d_f64", a.data_ptr(), b.data_ptr(), nx, ny, nx + 2, it, float(c["r"]), float(c["r"]), ctypes.byref(ci),
            None)
    r64 = a if ci.value == 0 else b
    assert np.array_equal(r64.cpu().numpy(), ref)  # the whole 1000-iteration run, bit for bit
    f32 = torch.from_numpy(W.heat2d_padded(nx, ny, c["top"], c["seed"])).cuda()
    x, y = f32.clone(), f32.clone()
    gb.call("appfis_gb_heat2d", x.data_ptr(), y.data_ptr(), nx, ny, nx + 2, it, c["r"], c["r"], ctypes.byref(ci), None)
    mx, rel = _err(x if ci.value == 0 else y, r64)
    assert mx < 5e-6 and rel < 5e-6, (mx, rel)  # measured: 8.4e-7, 4.4e-7


def test_himeno_full_size_fp64_pinned_and_form_errors(gb, torch_cuda):
    torch = torch_cuda
    c = W.HIMENO
    nx, ny, nz, it, om = c["nx"], c["ny"], c["nz"], c["iters"], c["omega"]
    coef = W.himeno_coef(nx, ny, nz)
    p0 = W.himeno_p(nx, ny, nz)
    # FP64 sweep pinned to the FP64 oracle on the full grid (3 sweeps)
    c64 = torch.from_numpy(coef.astype(np.float64)).cuda()
    ptr64 = (ctypes.c_void_p * 12)(*[c64[k].data_ptr() for k in range(12)])
    pref, gref = O.himeno(coef.astype(np.float64), p0.astype(np.float64), 3, om, dtype=np.float64)
    qa, qb = torch.from_numpy(p0.astype(np.float64)).cuda(), torch.zeros(p0.shape, dtype=torch.float64, device="cuda")
    g64 = torch.zeros(it, dtype=torch.float64, device="cuda")
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_himeno_f64", ptr64, qa.data_ptr(), qb.data_ptr(), nx, ny, nz, nx + 2, 3, float(om), g64.data_ptr(),
            ctypes.byref(ci), None)
    assert np.array_equal((qa if ci.value == 0 else qb).cpu().numpy(), pref)
    np.testing.assert_allclose(g64[:3].cpu().numpy(), gref, rtol=1e-12, atol=0)
    # the whole 400-sweep run in FP64, then the FP32 plain and FP16 defect-correction forms
    qa.copy_(torch.from_numpy(p0.astype(np.float64)))
    gb.call("appfis_gb_himeno_f64", ptr64, qa.data_ptr(), qb.data_ptr(), nx, ny, nz, nx + 2, it, float(om), g64.data_ptr(),
            ctypes.byref(ci), None)
    p64 = qa if ci.value == 0 else qb
    del c64
    pitch = (nx + 2 + 7) // 8 * 8
    cf = torch.zeros((12, nz + 2, ny + 2, pitch), dtype=torch.float32, device="cuda")
    cf[..., : nx + 2] = torch.from_numpy(coef).cuda()
    ptrs = (ctypes.c_void_p * 12)(*[cf[k].data_ptr() for k in range(12)])
    pp = torch.zeros((nz + 2, ny + 2, pitch), dtype=torch.float32, device="cuda")
    pp[..., : nx + 2] = torch.from_numpy(p0).cuda()
    gosa = torch.zeros(it, dtype=torch.float64, device="cuda")
    half = torch.empty(13 * pp.numel(), dtype=torch.float16, device="cuda")
    bounds = {"plain": (2e-5, 2e-5, 3e-5), "mixed": (1e-4, 2e-4, 2e-3)}  # p max-abs, gosa rel (last, max)
    for form in ("plain", "mixed"):  # measured: plain 7.3e-6, 1.7e-6, 9.1e-6; mixed 2.4e-5, 3.6e-5, 7.7e-4
        a, b = pp.clone(), pp.clone()
        if form == "plain":
            gb.call("appfis_gb_himeno", ptrs, a.data_ptr(), b.data_ptr(), nx, ny, nz, pitch, it, om, gosa.data_ptr(),
                    ctypes.byref(ci), None)
        else:
            gb.call("appfis_gb_himeno_mixed", ptrs, a.data_ptr(), b.data_ptr(), half.data_ptr(), nx, ny, nz, pitch, it, 20, om,
                    gosa.data_ptr(), ctypes.byref(ci), None)
        out = (a if ci.value == 0 else b)[..., : nx + 2]
        mx, _ = _err(out, p64)
        rel = ((gosa - g64).abs() / g64.abs())
        lim = bounds[form]
        assert mx < lim[0] and rel[-1].item() < lim[1] and rel.max().item() < lim[2], (form, mx, rel[-1].item(), rel.max().item())


def test_fdtd_full_size_fp64_pinned_and_form_errors(gb, torch_cuda):
    torch = torch_cuda
    c = W.FDTD
    nx, ny, nz, it = c["nx"], c["ny"], c["nz"], c["iters"]
    wts = W.fdtd_weights()
    f = W.fdtd_padded(nx, ny, nz, c["seed"])
    w64 = (ctypes.c_double * 5)(*wts)
    ci = ctypes.c_int(-1)
    x64 = torch.from_numpy(f.astype(np.float64)).cuda()
    y64 = x64.clone()
    # FP64 sweep pinned to the FP64 oracle on the full grid (2 steps)
    ref = O.star_r4(f.astype(np.float64), 2, weights=wts, dtype=np.float64)
    gb.call("appfis_gb_star_r4_f64", x64.data_ptr(), y64.data_ptr(), nx, ny, nz, nx + 8, 2, 1, 0.0, w64, ctypes.byref(ci), None)
    assert np.array_equal((x64 if ci.value == 0 else y64).cpu().numpy(), ref)
    del ref
    x64.copy_(torch.from_numpy(f.astype(np.float64)))
    gb.call("appfis_gb_star_r4_f64", x64.data_ptr(), y64.data_ptr(), nx, ny, nz, nx + 8, it, 1, 0.0, w64, ctypes.byref(ci), None)
    r64 = x64 if ci.value == 0 else y64
    w = (ctypes.c_float * 5)(*wts)
    f32 = torch.from_numpy(f).cuda()
    for dt, tdt, lim in ((_lib.F32, torch.float32, 1e-5), (_lib.F16, torch.float16, 1e-3)):  # measured rel L2 2.8e-6, 3.6e-4
        a = f32.to(tdt, copy=True)
        b = a.clone()
        gb.call("appfis_gb_star_r4", a.data_ptr(), b.data_ptr(), dt, nx, ny, nz, nx + 8, it, 1, 0.0, w, 0, 0, ctypes.byref(ci), None)
        mx, rel = _err((a if ci.value == 0 else b).float(), r64)
        assert rel < lim, (dt, mx, rel)


def test_flood_fp32_batch_against_fp64_batch(gb, torch_cuda):
    """Four of the benchmark's 32 domains to t = 600 s: the FP32 form's depth error over the water
    volume against the FP64 form (measured on the whole batch: 0.25% mean, 0.41% max)."""
    c = W.TRITON
    doms = W.triton_batch(c["n_domains"], c["side_lo"], c["side_hi"], c["seed"])[:4]
    runs = {}
    for dt in (_lib.F32, _lib.F64):
        runs[dt] = _lib.flood_job(doms, c["dx"], c["courant"], c["hextra"], c["manning"], c["t_end"], c["t_end"], c["time_step"],
                                  dtype=dt, flags=_lib.FLOOD_SKIP_DRY if dt == _lib.F64 else 0)
    for k in range(len(doms)):
        h32, h64 = runs[_lib.F32]["h"][k], runs[_lib.F64]["h"][k]
        vol = h64.sum()
        assert np.abs(h32 - h64).sum() / vol < 0.01, k
        m0, m1 = runs[_lib.F32]["mass"][k]
        assert abs(m1 - m0) / m0 < 2e-4, k
