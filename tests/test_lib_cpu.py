"""The C-ABI library builds for sm_103a, loads without a GPU, exports exactly what
include/appfis_gb.h declares, and rejects bad arguments before touching CUDA."""
import ctypes

import pytest

from appfis_gb300 import _lib, build


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    declared = _lib.declared_symbols()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(L, name), name
        assert name in _lib.SIGNATURES, "no ctypes signature for " + name


def test_version(L):
    assert L.appfis_gb_version() >= 10000


@pytest.mark.parametrize("call", [
    lambda L: L.appfis_gb_life_u8(None, None, 16, 16, 1, 0, None, None),
    lambda L: L.appfis_gb_life_u8(ctypes.c_void_p(16), ctypes.c_void_p(32), 0, 16, 1, 0, None, None),
    lambda L: L.appfis_gb_life_u8(ctypes.c_void_p(16), ctypes.c_void_p(32), 16, 16, 1, 7, None, None),
    lambda L: L.appfis_gb_life_bits(ctypes.c_void_p(16), ctypes.c_void_p(32), 48, 16, 1, 0, None, None),
    lambda L: L.appfis_gb_heat2d(ctypes.c_void_p(16), ctypes.c_void_p(16), 8, 8, 10, 1, 0.2, 0.2, None, None),
    lambda L: L.appfis_gb_heat2d(ctypes.c_void_p(16), ctypes.c_void_p(32), 8, 8, 9, 1, 0.2, 0.2, None, None),
    lambda L: L.appfis_gb_reduce(ctypes.c_void_p(16), 0, 8, 8, (ctypes.c_int * 6)(1, 9, 1, 7, 0, 1), 2,
                                 ctypes.c_void_p(64), None),
    lambda L: L.appfis_gb_reduce(ctypes.c_void_p(16), 5, 8, 8, (ctypes.c_int * 6)(1, 7, 1, 7, 0, 1), 2,
                                 ctypes.c_void_p(64), None),
])
def test_bad_arguments_are_rejected(L, call):
    assert call(L) == _lib.EINVAL
    assert len(L.appfis_gb_last_error()) > 0


def test_flood_param_struct_layout():
    """appfis_gb_flood_params: 7 doubles, max_steps, flags (64 bytes with natural alignment)."""
    from appfis_gb300 import _lib
    import ctypes
    assert ctypes.sizeof(_lib.FloodParams) == 64
    assert _lib.FloodParams.flags.offset == 60
