"""The bounded device-side waits, run out on purpose (appfis_gb_test_stall_next), without a GPU
fault or hang: every wait involved has a limit, the kernel gives up, the call reports
APPFIS_GB_ETIMEOUT, and the next call on the same device computes the right answer.

* The persistent flood kernels' grid barrier (fused and two-phase forms): CTA 0 does not arrive
  at the first barrier and each barrier wait gives up after 4096 polls (~64 ns sleep each).
* The TMA-staged radius-4 star: each CTA arms its first plane's mbarrier for 16 bytes more than
  the copy delivers and waits at most 1 ms; it then lets its copies land (10 ms per pending
  plane) and leaves; appfis_gb_stream_sync reads the device status word.
* The flood model's TMA-staged rows (FP32 fused pass): every warp arms its first stage of rows
  for 16 bytes more than its copies deliver and waits at most 1 ms; it lets its copies land
  (10 ms per pending stage), records the timeout and stops; the run reports APPFIS_GB_ETIMEOUT."""
import ctypes

import numpy as np
import pytest

from appfis_gb300 import _lib
from appfis_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [_lib.FLOOD_FUSED, _lib.FLOOD_TWO_PHASE])
def test_flood_grid_barrier_wait_runs_out_then_recovers(gb, torch_cuda, flags):
    doms = [W.triton_domain(70, 50, 3), W.triton_domain(40, 64, 4)]
    args = (10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0)
    gb.call("appfis_gb_test_stall_next", 1, 4096)
    with pytest.raises(_lib.AppfisError) as e:
        _lib.flood_job(doms, *args, max_steps=30, dtype=_lib.F32, flags=flags)
    assert e.value.status == _lib.ETIMEOUT, str(e.value)
    # the plan is used up: the same run now completes and matches a clean run's fields
    a = _lib.flood_job(doms, *args, max_steps=30, dtype=_lib.F32, flags=flags)
    b = _lib.flood_job(doms, *args, max_steps=30, dtype=_lib.F32, flags=flags)
    assert a["steps"] == b["steps"] == [30, 30]
    for k in range(2):
        assert np.array_equal(a["h"][k], b["h"][k])


def test_flood_staged_row_wait_runs_out_then_recovers(gb, torch_cuda):
    doms = [W.triton_domain(70, 50, 3), W.triton_domain(40, 64, 4)]
    args = (10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0)
    gb.call("appfis_gb_test_stall_next", 2, 1000000)  # 1 ms per wait
    with pytest.raises(_lib.AppfisError) as e:
        _lib.flood_job(doms, *args, max_steps=30, dtype=_lib.F32, flags=_lib.FLOOD_FUSED)
    assert e.value.status == _lib.ETIMEOUT, str(e.value)
    a = _lib.flood_job(doms, *args, max_steps=30, dtype=_lib.F32, flags=_lib.FLOOD_FUSED)
    b = _lib.flood_job(doms, *args, max_steps=30, dtype=_lib.F32, flags=_lib.FLOOD_FUSED | _lib.FLOOD_UNSTAGED)
    assert a["steps"] == b["steps"] == [30, 30]
    for k in range(2):
        assert np.array_equal(a["h"][k], b["h"][k])


def test_tma_mbarrier_wait_runs_out_then_recovers(gb, torch_cuda):
    torch = torch_cuda
    nx, ny, nz, it = 64, 48, 40, 3
    f = W.fdtd_padded(nx, ny, nz, 9)
    ref = O.star_r4(f, it, coeff=0.1)
    a = torch.from_numpy(f).cuda()
    b = a.clone()
    ci = ctypes.c_int(-1)
    gb.call("appfis_gb_test_stall_next", 2, 1000000)  # 1 ms per wait
    gb.call("appfis_gb_star_r4", a.data_ptr(), b.data_ptr(), 0, nx, ny, nz, nx + 8, it, 0, 0.1, None,
            _lib.STAR_TMA_X4, 0, ctypes.byref(ci), None)
    assert gb.lib().appfis_gb_stream_sync(None) == _lib.ETIMEOUT
    assert b"wait gave up" in gb.lib().appfis_gb_last_error()
    assert gb.lib().appfis_gb_stream_sync(None) == _lib.OK  # the status word was read and cleared
    # same device, clean run: bit-identical to the oracle
    a.copy_(torch.from_numpy(f))
    b.copy_(a)
    gb.call("appfis_gb_star_r4", a.data_ptr(), b.data_ptr(), 0, nx, ny, nz, nx + 8, it, 0, 0.1, None,
            _lib.STAR_TMA_X4, 0, ctypes.byref(ci), None)
    gb.call("appfis_gb_stream_sync", None)
    assert np.array_equal((a if ci.value == 0 else b).cpu().numpy(), ref)


def test_stall_plan_arguments_checked(gb):
    assert gb.lib().appfis_gb_test_stall_next(7, 10) == _lib.EINVAL
    assert gb.lib().appfis_gb_test_stall_next(1, 0) == _lib.EINVAL
    assert gb.lib().appfis_gb_test_stall_next(2, 10) == _lib.EINVAL
    assert gb.lib().appfis_gb_test_stall_next(0, 0) == _lib.OK
