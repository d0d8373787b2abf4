"""Box reductions (Execute*DReduce) vs the oracle: MAX/MIN exact with the reference's seeds,
SUM in double within 1e-12 of an exact double sum; deterministic across calls."""
import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def dev_reduce(gb, torch, arr, box, op):
    import ctypes
    t = torch.from_numpy(np.ascontiguousarray(arr)).cuda()
    shape = arr.shape if arr.ndim == 3 else (1,) + arr.shape
    b = list(box) + ([0, 1] if len(box) == 4 else [])
    code = {"max": 0, "min": 1, "sum": 2}[op]
    dt = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.int32): 2}[arr.dtype]
    res = ctypes.c_double()
    gb.call("appfis_gb_reduce_host", t.data_ptr(), dt, shape[2], shape[1], (ctypes.c_int * 6)(*b), code,
            ctypes.byref(res), None)
    return res.value


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32])
@pytest.mark.parametrize("shape,box", [((7, 9), (1, 8, 1, 6)), ((300, 1030), (1, 1029, 1, 299)),
                                       ((9, 33, 17), (2, 15, 1, 30, 3, 8)), ((66, 66, 66), (0, 66, 0, 66, 0, 66))])
def test_reduce_vs_oracle(gb, torch_cuda, dtype, shape, box):
    n = int(np.prod(shape))
    a = (W.uniform(n, n, -5, 5).reshape(shape) * (100 if dtype == np.int32 else 1)).astype(dtype)
    for op in ("max", "min"):
        assert dev_reduce(gb, torch_cuda, a, box, op) == O.reduce(a, box, op)
    s = dev_reduce(gb, torch_cuda, a, box, "sum")
    sl = tuple(slice(box[2 * k], box[2 * k + 1]) for k in range(len(box) // 2))[::-1]
    exact = a[sl].astype(np.float64).sum()
    assert abs(s - exact) <= 1e-12 * max(1.0, np.abs(a[sl]).astype(np.float64).sum())
    assert dev_reduce(gb, torch_cuda, a, box, "sum") == s


def test_max_seed_quirk(gb, torch_cuda):
    a = -np.ones((6, 6), dtype=np.float32)
    assert dev_reduce(gb, torch_cuda, a, (1, 5, 1, 5), "max") == float(np.finfo(np.float32).tiny)
