"""The allocation-free reduction entry point, for callers that cannot allocate device memory
when they reduce (under a framework allocator that holds the device memory, inside a runtime
that owns every allocation, or where a first-call cudaMalloc would stall a latency-critical
loop).

appfis_gb_reduce_noalloc is called through the C ABI and must give what appfis_gb_reduce gives
on the same field — MAX and MIN exactly, SUM within the 1e-12 relative tolerance of the other
reduction tests — on two calls in a row (the second one reuses the fixed scratch left by the
first); MAX and MIN are also checked against the oracle, SUM against a double sum of the box.  This file runs last so that a failure here
cannot hide any other test."""
import ctypes

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [((7, 9), (1, 8, 1, 6)), ((300, 1030), (1, 1029, 1, 299)), ((9, 33, 17), (2, 15, 1, 30, 3, 8))]


def _reduce(gb, name, t, dt, shape, box, op, out):
    b = list(box) + ([0, 1] if len(box) == 4 else [])
    gb.call(name, t.data_ptr(), dt, shape[2], shape[1], (ctypes.c_int * 6)(*b), op, out.data_ptr(), None)


@pytest.mark.parametrize("dtype,code", [(np.float32, 0), (np.float64, 1), (np.int32, 2)])
@pytest.mark.parametrize("shape,box", CASES)
def test_noalloc_matches_workspace_reduction(gb, torch_cuda, dtype, code, shape, box):
    torch = torch_cuda
    n = int(np.prod(shape))
    a = (W.uniform(n + 17, n, -5, 5).reshape(shape) * (100 if dtype == np.int32 else 1)).astype(dtype)
    t = torch.from_numpy(a).cuda()
    shp = shape if len(shape) == 3 else (1,) + shape
    res_dt = torch.int64 if dtype == np.int32 else torch.float64
    for op in (0, 1, 2):  # MAX, MIN, SUM
        want = torch.zeros(1, dtype=res_dt, device="cuda")
        _reduce(gb, "appfis_gb_reduce", t, code, shp, box, op, want)
        for call in range(2):  # two calls in a row share the fixed scratch
            got = torch.full((1,), -7, dtype=res_dt, device="cuda")
            _reduce(gb, "appfis_gb_reduce_noalloc", t, code, shp, box, op, got)
            torch.cuda.synchronize()
            w, g = want.item(), got.item()
            if op == 2 and dtype != np.int32:
                assert abs(g - w) <= 1e-12 * max(1.0, abs(w)), (op, call, g, w)
            else:
                assert g == w, (op, call, g, w)
        a3 = a if len(shape) == 3 else a[None]
        b6 = list(box) + ([0, 1] if len(box) == 4 else [])
        if op == 2:  # the engine sums in double (int64 for int), the oracle in the element type like the reference
            o = float(a3[b6[4]:b6[5], b6[2]:b6[3], b6[0]:b6[1]].astype(np.float64).sum())
        else:
            o = O.reduce(a3, b6, ("max", "min", "sum")[op])
        assert abs(got.item() - o) <= 1e-12 * max(1.0, abs(o)), (op, got.item(), o)
