"""FP64 sweeps (appfis_gb_heat2d_f64 / himeno_f64 / star_r4_f64) against the oracle built with
double: fields bit-identical (every multiply and add rounded separately in the reference's
order), gosa within 1e-12 relative (a different but fixed summation order).  These FP64 forms
are the precision reference that the bench states the other forms' error against."""
import ctypes

import numpy as np
import pytest

from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx,ny,iters", [(19, 23, 17), (64, 40, 40), (130, 97, 9)])
def test_heat2d_f64_bit_identical(gb, torch_cuda, nx, ny, iters):
    torch = torch_cuda
    f = W.heat2d_padded(nx, ny, 1.0, nx + ny, dtype=np.float64)
    ref = O.heat2d(f, iters, 0.2, dtype=np.float64)
    a = torch.from_numpy(f).cuda()
    b = a.clone()
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_heat2d_f64", a.data_ptr(), b.data_ptr(), nx, ny, nx + 2, iters, 0.2, 0.2, ctypes.byref(ci), None)
    out = (a if ci.value == 0 else b).cpu().numpy()
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("nx,ny,nz,iters", [(13, 11, 9, 7), (33, 17, 20, 4), (65, 9, 5, 3)])
def test_himeno_f64_bit_identical(gb, torch_cuda, nx, ny, nz, iters):
    torch = torch_cuda
    coef = W.himeno_coef(nx, ny, nz, dtype=np.float64, seed=nx + nz)
    p = W.himeno_p(nx, ny, nz, dtype=np.float64)
    pref, gref = O.himeno(coef, p, iters, 0.8, dtype=np.float64)
    cd = torch.from_numpy(coef).cuda()
    ptrs = (ctypes.c_void_p * 12)(*[cd[k].data_ptr() for k in range(12)])
    a = torch.from_numpy(p).cuda()
    b = torch.zeros_like(a)
    gosa = torch.zeros(iters, dtype=torch.float64, device="cuda")
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_himeno_f64", ptrs, a.data_ptr(), b.data_ptr(), nx, ny, nz, nx + 2, iters, 0.8, gosa.data_ptr(),
            ctypes.byref(ci), None)
    out = (a if ci.value == 0 else b).cpu().numpy()
    assert np.array_equal(out, pref)
    np.testing.assert_allclose(gosa.cpu().numpy(), gref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("nx,ny,nz,iters", [(12, 10, 9, 3), (40, 33, 17, 5)])
@pytest.mark.parametrize("mode", [0, 1])
def test_star_r4_f64_bit_identical(gb, torch_cuda, nx, ny, nz, iters, mode):
    torch = torch_cuda
    f = W.fdtd_padded(nx, ny, nz, nx + nz, dtype=np.float64)
    wts = W.fdtd_weights()
    ref = O.star_r4(f, iters, coeff=0.1 if mode == 0 else None, weights=None if mode == 0 else wts, dtype=np.float64)
    a = torch.from_numpy(f).cuda()
    b = a.clone()
    w = (ctypes.c_double * 5)(*wts)
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_star_r4_f64", a.data_ptr(), b.data_ptr(), nx, ny, nz, nx + 8, iters, mode, 0.1, w, ctypes.byref(ci),
            None)
    out = (a if ci.value == 0 else b).cpu().numpy()
    assert np.array_equal(out, ref)
