"""The reference's five sample applications, UNCHANGED, built against the drop-in headers and
run on the GPU, against the same sources built with the reference's own headers (APPFIS_CPU,
OpenMP, the single-rank MPI stand-in) and run on the host: the values each application prints
with -output must agree — HeatDiffusion Max/Min (FP64) and GameOfLife Live Count identical,
Himeno Sum within 2e-4 relative (the reference sums FP32 values in an FP32 accumulator, so its own
result moves by ~1e-4 with the OpenMP thread count; the engine sums in double) — and
the Triton flood application, run on a synthetic case through its own readers (key=value
configuration, ASCII DEM with its 6-line header, initial depth file, point source with a
hydrograph), must write the same h/u/v fields (6 decimals, the applications' output format).

The same applications with ONE added line, APPFIS::UseFastKernel(config, ...) after their
GridsToUpdate (appfis_gb300/Appfis/Fast.hpp), run their Execute*D loops on the hand-written
kernels (GameOfLife: the bit-packed time-blocked or the u8 sweep; Himeno: the TMA-staged sweep,
on 128-byte-pitched copies where the application's rows are not 16-byte aligned; FDTD3d: the
TMA-staged radius-4 star) and must print what the unchanged build prints: GameOfLife Live Count
and Himeno Sum identical to the unchanged build (and to the reference as above); FDTD3d's
written field identical to the reference CPU build's.

Needs oracle/_ref/apps/ (flattened from the reference tree by oracle/build_ref.py)."""
import os
import re
import subprocess

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import build_ref
from tests.dropin import build_apps

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not build_apps.available(), reason="application sources not present")]


@pytest.fixture(scope="module")
def exes(gb):
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=len(build_apps.APPS)) as ex:
        refs = ex.map(build_ref.app_ref_exe, build_apps.APPS)
        gbx = build_apps.build()
        ref = dict(zip(build_apps.APPS, refs))
    return gbx, ref


def run(exe, args, cwd):
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=600, cwd=cwd)
    assert r.returncode == 0, (exe, r.stdout[-2000:], r.stderr[-2000:])
    return r.stdout


def values(out, keys):
    got = {}
    for k in keys:
        m = re.search(r"^%s:\s*(\S+)\s*$" % re.escape(k), out, re.M)
        assert m, (k, out)
        got[k] = m.group(1)
    return got


@pytest.mark.parametrize("app,args,keys,rtol", [
    ("HeatDiffusion", ["-dimx=48", "-dimy=40", "-dimz=36", "-iteration=20"], ["Max", "Min"], 0),
    ("HeatDiffusion", ["-dimx=33", "-dimy=17", "-dimz=9", "-iteration=7"], ["Max", "Min"], 0),
    ("GameOfLife", ["-dimx=300", "-dimy=200", "-iteration=50"], ["Live Count"], 0),
    ("GameOfLife", ["-dimx=67", "-dimy=45", "-iteration=31"], ["Live Count"], 0),
    # -overlap: the overlapped executors on both sides (strips first, the ghost refresh behind the interior)
    ("GameOfLife", ["-dimx=300", "-dimy=200", "-iteration=50", "-overlap"], ["Live Count"], 0),
    ("Himeno", ["-dimx=65", "-dimy=65", "-dimz=129", "-iteration=20"], ["Sum"], 2e-4),
    ("Himeno", ["-dimx=33", "-dimy=17", "-dimz=20", "-iteration=5"], ["Sum"], 2e-4),
])
def test_application_outputs_match(exes, tmp_path, app, args, keys, rtol):
    gbx, ref = exes
    a = values(run(gbx[app], args + ["-output"], str(tmp_path)), keys)
    b = values(run(ref[app], args + ["-output", "-thread=4"], str(tmp_path)), keys)
    if rtol == 0:
        assert a == b
    else:
        for k in keys:
            assert float(a[k]) == pytest.approx(float(b[k]), rel=rtol), (k, a[k], b[k])


def test_fdtd_application_runs(exes, tmp_path):
    """FDTD3d prints no field values; it must run to completion and report its rate."""
    gbx, _ = exes
    out = run(gbx["FDTD3d"], ["-dimx=64", "-dimy=48", "-dimz=40", "-iteration=10", "-output"], str(tmp_path))
    assert re.search(r"^GFLOPS:\s*\S+", out, re.M)


@pytest.mark.parametrize("nx,ny,seed,duration", [(48, 40, 77, 120), (97, 61, 5, 90)])
def test_triton_application_case_files(exes, tmp_path, nx, ny, seed, duration):
    gbx, ref = exes
    out = {}
    for name, exe, extra in (("gb", gbx["Triton"], []), ("ref", ref["Triton"], ["-thread=4"])):
        d = tmp_path / name
        d.mkdir()
        W.write_triton_case(str(d), nx, ny, seed, duration)
        text = run(exe, ["case.cfg", "-output"] + extra, str(d))
        steps = int(re.search(r"^Number of iteration:\s*(\d+)", text, re.M).group(1))
        fields = [np.loadtxt(str(d / "output" / f)) for f in ("h.txt", "u.txt", "v.txt")]
        out[name] = (steps, fields)
    assert out["gb"][0] == out["ref"][0]
    h0 = W.triton_domain(ny, nx, seed)[1]
    assert out["ref"][1][0].sum() > h0.sum()  # the point source added water
    for a, b in zip(out["gb"][1], out["ref"][1]):
        assert a.shape == (ny, nx)
        # 6 printed decimals; cbrt/sqrt may differ in the last bit between the CUDA and host libraries
        assert np.abs(a - b).max() <= 2e-6


@pytest.fixture(scope="module")
def fast_exes(gb):
    return build_apps.build(build_apps.FAST_APPS, fast=True)


@pytest.mark.parametrize("app,args,keys,rtol", [
    ("GameOfLife", ["-dimx=320", "-dimy=200", "-iteration=50"], ["Live Count"], 0),   # bit-packed: 3 x 16 + 2 generations
    ("GameOfLife", ["-dimx=67", "-dimy=45", "-iteration=31"], ["Live Count"], 0),     # u8 cells (67 is not a multiple of 32)
    ("GameOfLife", ["-dimx=64", "-dimy=64", "-iteration=7"], ["Live Count"], 0),      # fewer generations than one time block
    ("Himeno", ["-dimx=126", "-dimy=65", "-dimz=100", "-iteration=20"], ["Sum"], 2e-4),  # 128-float rows: on the grids
    ("Himeno", ["-dimx=65", "-dimy=65", "-dimz=129", "-iteration=20"], ["Sum"], 2e-4),   # 67-float rows: padded copies
])
def test_fast_kernel_application_outputs_match(exes, fast_exes, tmp_path, app, args, keys, rtol):
    gbx, ref = exes
    f = values(run(fast_exes[app], args + ["-output"], str(tmp_path)), keys)
    u = values(run(gbx[app], args + ["-output"], str(tmp_path)), keys)
    b = values(run(ref[app], args + ["-output", "-thread=4"], str(tmp_path)), keys)
    assert f == u  # same fields as the functor path, same engine reduction
    for k in keys:
        if rtol == 0:
            assert f[k] == b[k]
        else:
            assert float(f[k]) == pytest.approx(float(b[k]), rel=rtol), (k, f[k], b[k])


@pytest.mark.parametrize("dims", [(64, 48, 40), (61, 37, 23)])
def test_fast_kernel_fdtd_field_matches_reference(exes, fast_exes, tmp_path, dims):
    """FDTD3d with its fast-kernel line writes the same field (6 decimals of every value after
    10 steps) as the reference's CPU build: the radius-4 star in the reference form is
    bit-identical (64-wide rows: TMA-staged tile; 61-wide rows: the unaligned fallback tiles)."""
    gbx, ref = exes
    args = ["-dimx=%d" % dims[0], "-dimy=%d" % dims[1], "-dimz=%d" % dims[2], "-iteration=10", "-output"]
    texts = {}
    for name, exe, extra in (("fast", fast_exes["FDTD3d"], []), ("ref", ref["FDTD3d"], ["-thread=4"])):
        d = tmp_path / name
        d.mkdir()
        run(exe, args + extra, str(d))
        texts[name] = (d / "output" / "output.txt").read_text()
    assert len(texts["ref"]) > 1000
    assert texts["fast"] == texts["ref"]


def test_triton_application_restart_from_checkpoint_files(exes, tmp_path):
    """The Triton application's restart path (Triton/src/config_utils.hpp:369-379,
    triton_appfis.hpp:158-213,311-312): a run to t = 60 s writes h/u/v; a second run starts from
    those files (h_infile, qx_infile, qy_infile, sim_start_time = 60, checkpoint_id = 1,
    it_count = the first run's steps) and continues to 120 s.  The drop-in build and the
    reference's CPU build restart from the same files and must agree like the plain runs."""
    import shutil
    gbx, ref = exes
    nx, ny, seed = 64, 48, 21
    first = tmp_path / "first"
    first.mkdir()
    W.write_triton_case(str(first), nx, ny, seed, 60)
    text = run(ref["Triton"], ["case.cfg", "-output", "-thread=4"], str(first))
    n1 = int(re.search(r"^Number of iteration:\s*(\d+)", text, re.M).group(1))
    out = {}
    for name, exe, extra in (("gb", gbx["Triton"], []), ("ref", ref["Triton"], ["-thread=4"])):
        d = tmp_path / name
        d.mkdir()
        W.write_triton_case(str(d), nx, ny, seed, 120)
        for f in ("h", "u", "v"):
            shutil.copy(str(first / "output" / ("%s.txt" % f)), str(d / ("%s0.txt" % f)))
        cfg = (d / "case.cfg").read_text().replace("h_infile=h.asc", "h_infile=h0.txt")
        cfg = cfg.replace("sim_start_time=0", "sim_start_time=60")
        cfg += "qx_infile=u0.txt\nqy_infile=v0.txt\ncheckpoint_id=1\nit_count=%d\n" % n1
        (d / "case.cfg").write_text(cfg)
        text = run(exe, ["case.cfg", "-output"] + extra, str(d))
        steps = int(re.search(r"^Number of iteration:\s*(\d+)", text, re.M).group(1))
        out[name] = (steps, [np.loadtxt(str(d / "output" / f)) for f in ("h.txt", "u.txt", "v.txt")])
    assert out["gb"][0] == out["ref"][0] > n1  # the count continues from it_count
    for a, b in zip(out["gb"][1], out["ref"][1]):
        assert a.shape == (ny, nx)
        assert np.abs(a - b).max() <= 2e-6


def test_batched_flood_point_source_matches_reference_application(exes, gb, torch_cuda, tmp_path):
    """The batched persistent flood kernel with a point source (appfis_gb_flood_run_sources, FP64)
    on the Triton application's own case files (DEM, initial depth, hydrograph converted from
    hours, source location through the reference's cell formula, triton_appfis.hpp:218-237,
    555-564) gives the reference CPU build's step count and h/u/v fields (6 printed decimals)."""
    import ctypes
    import math
    from appfis_gb300 import _lib
    torch = torch_cuda
    _, ref = exes
    nx, ny, seed, duration = 48, 40, 77, 120
    W.write_triton_case(str(tmp_path), nx, ny, seed, duration)
    text = run(ref["Triton"], ["case.cfg", "-output", "-thread=4"], str(tmp_path))
    ref_steps = int(re.search(r"^Number of iteration:\s*(\d+)", text, re.M).group(1))
    want = [np.loadtxt(str(tmp_path / "output" / f)) for f in ("h.txt", "u.txt", "v.txt")]
    dem = np.loadtxt(str(tmp_path / "dem.asc"), skiprows=6)
    h0 = np.loadtxt(str(tmp_path / "h.asc"))
    rows = [l.split("%")[0].strip() for l in open(str(tmp_path / "hydro.txt"))]
    hyd = np.array([[float(v) for v in r.split(",")] for r in rows if r])
    sx, sy = [float(v) for v in [l for l in open(str(tmp_path / "src.txt")) if not l.startswith("%")][0].split(",")]
    col, row = math.ceil(sx / 10.0) - 1, math.ceil(ny - sy / 10.0) - 1
    cells = np.array([(row + 1) * (nx + 2) + (col + 1)], dtype=np.int32)
    times = np.ascontiguousarray(hyd[:, 0] * 3600.0)
    flows = np.ascontiguousarray(hyd[:, 1:])
    srcs = (_lib.FloodSources * 1)()
    srcs[0].n, srcs[0].nt = 1, len(times)
    srcs[0].cells, srcs[0].times, srcs[0].flows = cells.ctypes.data, times.ctypes.data, flows.ctypes.data
    pitch = (nx + 2 + 15) // 16 * 16
    f = torch.zeros((8, ny + 2, pitch), dtype=torch.float64, device="cuda")
    dom = (_lib.FloodDomain * 1)()
    d = dom[0]
    d.nx, d.ny, d.pitch = nx, ny, pitch
    d.h[0], d.h[1], d.qx[0], d.qx[1], d.qy[0], d.qy[1] = [f[m].data_ptr() for m in range(6)]
    d.dem, d.n2 = f[6].data_ptr(), f[7].data_ptr()
    dd, hh = torch.from_numpy(dem).cuda(), torch.from_numpy(h0).cuda()
    gb.call("appfis_gb_flood_setup", ctypes.byref(d), _lib.F64, dd.data_ptr(), hh.data_ptr(), None, None, 0.035, None)
    prm = _lib.FloodParams(10.0, 0.5, 1e-3, float(duration), 60.0, 1.0, 0.0, 0)
    steps = torch.zeros(1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    gb.call("appfis_gb_flood_run_sources", dom, srcs, 1, _lib.F64, ctypes.byref(prm), None, steps.data_ptr(), None,
            status.data_ptr(), None)
    torch.cuda.synchronize()
    assert int(status.item()) == 0 and int(steps.item()) == ref_steps
    b = int(steps.item()) & 1
    got = [f[2 * k + b][1:ny + 1, 1:nx + 1].cpu().numpy() for k in range(3)]
    assert got[0].sum() > h0.sum()  # the source added water
    for a, w in zip(got, want):
        assert np.abs(a - w).max() <= 2e-6
