"""The drop-in C++ API (appfis_gb300/Appfis: Grid / Config / Execute*D / Execute*DReduce /
HaloExchange / Scatter / Gather) on the GPU: application-style functors driven through it give
the reference's results (golden fixtures from the reference's own CPU path, and the oracle)."""
import glob
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def runner(gb):
    from tests.dropin import build_runner
    return build_runner.build()


def run(exe, args, inputs, outputs):
    with tempfile.TemporaryDirectory() as td:
        subs = {}
        for k, a in enumerate(inputs):
            p = os.path.join(td, "in%d" % k)
            np.ascontiguousarray(a).tofile(p)
            subs["in%d" % k] = p
        for k in range(len(outputs)):
            subs["out%d" % k] = os.path.join(td, "out%d" % k)
        r = subprocess.run([exe] + [str(a).format(**subs) for a in args], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        res = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
        return res, [np.fromfile(subs["out%d" % k], dtype=dt) for k, dt in enumerate(outputs)]


# "fast": the same program with APPFIS::UseFastKernel on its Config (the hand-written kernel runs
# the Execute loop); results must be the functor path's
ROUTES = ["functor", "fast"]


@pytest.mark.parametrize("route", ROUTES)
@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "gol_*.npz"))), ids=os.path.basename)
def test_gol_golden(runner, f, route):
    g = np.load(f)
    ny, nx = g["cells"].shape
    res, (out,) = run(runner, ["gol", nx, ny, int(g["gens"]), "{in0}", "{out0}", route], [g["cells"]], [np.uint8])
    assert np.array_equal(out.reshape(ny, nx), g["out"])
    assert res["live"] == int(g["live"])


@pytest.mark.parametrize("route,nx", [("functor", 300), ("fast", 300), ("fast", 320)])
def test_gol_larger_vs_oracle(runner, route, nx):
    c = W.gol_cells(nx, 170, 0.3, 12)
    res, (out,) = run(runner, ["gol", nx, 170, 40, "{in0}", "{out0}", route], [c], [np.uint8])
    ref, _ = O.gol(c, 40)
    assert np.array_equal(out.reshape(170, nx), ref) and res["live"] == int(ref.sum())


@pytest.mark.parametrize("route", ROUTES)
@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "heat2d_*.npz"))), ids=os.path.basename)
def test_heat2d_golden(runner, f, route):
    g = np.load(f)
    ny, nx = g["padded"].shape[0] - 2, g["padded"].shape[1] - 2
    res, (out,) = run(runner, ["heat2d", nx, ny, int(g["iters"]), 0.2, 1.0, "{in0}", "{out0}", route],
                      [np.ascontiguousarray(g["padded"][1:-1, 1:-1])], [np.float32])
    assert np.array_equal(out.reshape(ny + 2, nx + 2), g["out"])
    assert np.float32(res["max"]) == np.float32(g["stats"][0])
    assert np.float32(res["min"]) == np.float32(g["stats"][1])
    assert abs(res["sum"] - g["stats"][2]) <= 1e-5 * abs(g["stats"][2])


@pytest.mark.parametrize("route", ROUTES)
@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "himeno_*.npz"))), ids=os.path.basename)
def test_himeno_golden(runner, f, route):
    g = np.load(f)
    p = g["p"]
    nz, ny, nx = p.shape[0] - 2, p.shape[1] - 2, p.shape[2] - 2
    res, (out,) = run(runner, ["himeno", nx, ny, nz, int(g["iters"]), 0.8, "{in0}", "{in1}", "{out0}", route],
                      [g["coef"], np.ascontiguousarray(p[1:-1, 1:-1, 1:-1])], [np.float32])
    assert np.array_equal(out.reshape(p.shape), g["out"])


@pytest.mark.parametrize("route", ROUTES)
@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "fdtd_*.npz"))), ids=os.path.basename)
def test_fdtd_golden(runner, f, route):
    g = np.load(f)
    pd = g["padded"]
    nz, ny, nx = pd.shape[0] - 8, pd.shape[1] - 8, pd.shape[2] - 8
    res, (out,) = run(runner, ["fdtd", nx, ny, nz, int(g["iters"]), float(g["coeff"]), "{in0}", "{out0}", route],
                      [np.ascontiguousarray(pd[4:-4, 4:-4, 4:-4])], [np.float32])
    assert np.array_equal(out.reshape(pd.shape), g["out"])


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLD, "triton_*.npz"))), ids=os.path.basename)
def test_triton_golden(runner, f):
    g = np.load(f)
    ny, nx = g["dem"].shape
    dx, cn, hextra, mann, t_end, pint, ts = [float(v) for v in g["params"]]
    res, (out, dts) = run(runner, ["triton", nx, ny, dx, cn, hextra, mann, t_end, pint, ts, int(g["steps"]), "{in0}", "{in1}",
                                   "{out0}", "{out1}"], [g["dem"], g["h0"]], [np.float64, np.float64])
    n = nx * ny
    assert res["steps"] == int(g["steps"])
    np.testing.assert_allclose(dts, g["dts"], rtol=1e-9)
    np.testing.assert_allclose(out[:n].reshape(ny, nx), g["h"], atol=1e-9)
    np.testing.assert_allclose(out[n:2 * n].reshape(ny, nx), g["qx"], atol=1e-9)
    np.testing.assert_allclose(out[2 * n:].reshape(ny, nx), g["qy"], atol=1e-9)


@pytest.mark.parametrize("lo,hi", [(-1000, 1000), (1 << 29, (1 << 31) - 1), (-(1 << 31), -(1 << 29))])
def test_int_reduce_wraps_like_int(runner, lo, hi):
    """Execute2DReduce on an int grid: MAX / MIN exact, SUM equal to the reference's int
    accumulation (wrapped modulo 2^32 when the total leaves the int range)."""
    rng = np.random.default_rng(lo & 0xffff)
    nx, ny = 301, 77
    a = rng.integers(lo, hi, size=(ny, nx), dtype=np.int64).astype(np.int32)
    res, _ = run(runner, ["ireduce", nx, ny, "{in0}"], [a], [])
    total = int(a.astype(np.int64).sum())
    wrapped = (total + (1 << 31)) % (1 << 32) - (1 << 31)
    assert res["sum"] == wrapped
    assert res["max"] == int(a.max()) and res["min"] == int(a.min())


@pytest.mark.parametrize("nx,ny,nz,iters", [(33, 17, 20, 45), (62, 9, 13, 30)])
def test_himeno_fast_routes_vs_oracle(runner, nx, ny, nz, iters):
    """Himeno through Execute3D with FAST_HIMENO (62-wide: rows of 64 floats, on the grid's own
    buffers; 33-wide: on 128-byte-pitched copies) is bit-identical to the oracle (random
    coefficient fields, so every term counts); with FAST_HIMENO_MIXED (FP16 defect correction,
    FP32 refresh every 20 sweeps) on the benchmark's coefficients it stays within the mixed
    form's 2.5e-4 of the FP64 oracle."""
    coef = W.himeno_coef(nx, ny, nz, seed=nx + nz)
    p = W.himeno_p(nx, ny, nz)
    pin = np.ascontiguousarray(p[1:-1, 1:-1, 1:-1])
    ref, _ = O.himeno(coef, p, iters, 0.8)
    _, (out,) = run(runner, ["himeno", nx, ny, nz, iters, 0.8, "{in0}", "{in1}", "{out0}", "fast"], [coef, pin], [np.float32])
    assert np.array_equal(out.reshape(p.shape), ref)
    bench = W.himeno_coef(nx, ny, nz)
    ref64, _ = O.himeno(W.himeno_coef(nx, ny, nz, dtype=np.float64), W.himeno_p(nx, ny, nz, dtype=np.float64), iters, 0.8,
                        dtype=np.float64)
    _, (mix,) = run(runner, ["himeno", nx, ny, nz, iters, 0.8, "{in0}", "{in1}", "{out0}", "mixed"], [bench, pin], [np.float32])
    assert np.abs(mix.reshape(p.shape).astype(np.float64) - ref64).max() < 2.5e-4


@pytest.mark.parametrize("route", ROUTES)
def test_device_checkpoint_restart(runner, tmp_path, route):
    """SaveDeviceState after G1 generations, LoadDeviceState into a second grid, G2 more on
    both: identical to each other and to G1 + G2 generations of the oracle (the checkpoint keeps
    both buffers, which the reference rule's stale carry reads); the gathered grid survives an
    Array::SaveBinaryFile / LoadBinaryFile round trip (Appfis/Array.hpp:421-527)."""
    nx, ny, g1, g2 = 96, 70, 19, 23
    c = W.gol_cells(nx, ny, 0.3, 31)
    res, (a, b) = run(runner, ["ckpt", nx, ny, g1, g2, "{in0}", "{out0}", "{out1}", str(tmp_path), route], [c],
                      [np.uint8, np.uint8])
    ref, _ = O.gol(c, g1 + g2)
    assert np.array_equal(a.reshape(ny, nx), ref)
    assert np.array_equal(b.reshape(ny, nx), ref)
    assert res["binary_roundtrip"] is True


@pytest.mark.parametrize("nx,ny,nz", [(40, 36, 48), (33, 45, 41)])
def test_overlap_executor_3d_periodic(runner, nx, ny, nz):
    """ExecuteOverlap3D on a periodic grid (the six boundary slabs first, the periodic ghost
    refresh on a second stream behind the interior sweep) gives Execute3D's field bit for bit,
    and the field is not trivial (the periodic ghosts matter)."""
    f = (W.uniform(nx * ny + nz, nx * ny * nz, -1.0, 1.0)).astype(np.float32)
    _, (plain, over) = run(runner, ["star_periodic", nx, ny, nz, 6, "{in0}", "{out0}", "{out1}"], [f], [np.float32, np.float32])
    assert np.array_equal(plain, over)
    assert np.abs(plain).max() > 0
