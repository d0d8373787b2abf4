"""The oracle pinned against the reference: the C++ restatement must reproduce the golden
fixtures (outputs of the reference's own CPU path, tests/golden/make_golden.py) bit for bit,
and, where the reference harnesses are built on this machine, fresh random cases too."""
import glob
import os

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def golden(prefix):
    files = sorted(glob.glob(os.path.join(GOLD, prefix + "*.npz")))
    assert files, "no golden fixtures for " + prefix
    return [(os.path.basename(f), np.load(f)) for f in files]


@pytest.mark.parametrize("name,g", golden("gol_"))
def test_gol_golden(name, g):
    cur, _ = O.gol(g["cells"], int(g["gens"]))
    assert np.array_equal(cur, g["out"])
    assert O.population(cur) == int(g["live"])


def test_gol_stale_carry_differs_from_b3s23():
    c = W.gol_cells(64, 64, 0.3, 9)
    ref, _ = O.gol(c, 12)
    conway = O.gol_b3s23(c, 12)
    assert not np.array_equal(ref, conway)


@pytest.mark.parametrize("name,g", golden("heat2d_"))
def test_heat2d_golden(name, g):
    out = O.heat2d(g["padded"], int(g["iters"]), 0.2)
    assert np.array_equal(out, g["out"])
    ny, nx = out.shape[0] - 2, out.shape[1] - 2
    box = (1, nx + 1, 1, ny + 1)
    mx, mn, sm = (O.reduce(out, box, op) for op in ("max", "min", "sum"))
    assert np.float32(mx) == np.float32(g["stats"][0])
    assert np.float32(mn) == np.float32(g["stats"][1])
    assert np.float32(sm) == np.float32(g["stats"][2])


@pytest.mark.parametrize("name,g", golden("himeno_"))
def test_himeno_golden(name, g):
    p, gosa = O.himeno(g["coef"], g["p"], int(g["iters"]), 0.8)
    assert np.array_equal(p, g["out"])
    np.testing.assert_allclose(gosa, g["gosa"], rtol=1e-12)


@pytest.mark.parametrize("name,g", golden("fdtd_"))
def test_fdtd_golden(name, g):
    out = O.star_r4(g["padded"], int(g["iters"]), coeff=float(g["coeff"]))
    assert np.array_equal(out, g["out"])


@pytest.mark.parametrize("name,g", golden("triton_"))
def test_triton_golden(name, g):
    dx, cn, hextra, mann, t_end, pint, ts = [float(v) for v in g["params"]]
    r = O.triton(g["dem"], g["h0"], dx, cn, hextra, mann, t_end, pint, ts, max_steps=int(g["steps"]))
    assert r["steps"] == int(g["steps"])
    assert np.array_equal(r["dts"], g["dts"])
    for k in ("h", "qx", "qy"):
        assert np.array_equal(r[k], g[k]), k
    assert np.abs(g["qx"]).max() > 0 and np.abs(g["qy"]).max() > 0  # the case exercises momentum


def test_reduce_max_seed_quirk():
    """MAX is seeded with numeric_limits<T>::min(): an all-negative box returns FLT_MIN."""
    a = -np.ones((4, 5), dtype=np.float32)
    assert O.reduce(a, (1, 4, 1, 3), "max") == float(np.finfo(np.float32).tiny)
    ai = -np.ones((4, 5), dtype=np.int32)
    assert O.reduce(ai, (1, 4, 1, 3), "max") == -1


@pytest.mark.skipif(not O.ref_available("gol"), reason="reference harness not built here")
def test_gol_random_vs_reference():
    for (nx, ny, gens, seed) in [(17, 13, 11, 1), (40, 3, 5, 2), (3, 3, 4, 3)]:
        c = W.gol_cells(nx, ny, 0.4, seed)
        res, (out,) = O.run_ref("gol", [nx, ny, gens, 2, "{in0}", "{out0}"], [c], [(np.uint8, None)])
        cur, _ = O.gol(c, gens)
        assert np.array_equal(cur, out.reshape(ny, nx))
        assert res["live"] == O.population(cur)


@pytest.mark.skipif(not O.ref_available("triton"), reason="reference harness not built here")
def test_triton_random_vs_reference():
    ny, nx = 21, 30
    dem, h = W.triton_domain(ny, nx, 123)
    qx = W.uniform(5, ny * nx, -0.2, 0.2).reshape(ny, nx) * h
    args = [nx, ny, 2, 10.0, 0.5, 1e-3, 0.035, 600.0, 17.0, 1.0, 40, "{in0}", "{in1}", "{out0}", "{out1}"]
    # the harness starts from qx = qy = 0; use that here too
    res, (out, dts) = O.run_ref("triton", args, [dem, h], [(np.float64, None), (np.float64, None)])
    r = O.triton(dem, h, 10.0, 0.5, 1e-3, 0.035, 600.0, 17.0, 1.0, max_steps=40)
    assert np.array_equal(r["dts"], dts)  # includes the print-interval clamp at 17 s
    assert np.array_equal(r["h"], out[: nx * ny].reshape(ny, nx))
    del qx
