"""ctypes binding of libappfis_gb.so (the C ABI declared in include/appfis_gb.h).

The library must have been built (appfis_gb300.build.build() or __graft_entry__.build());
there is no fallback: loading fails loudly when it is missing.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libappfis_gb.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "appfis_gb.h")

OK, EINVAL, ECUDA, ENOMEM, ETIMEOUT = 0, 1, 2, 3, 4
F32, F64, I32, F16 = 0, 1, 2, 3
MAX, MIN, SUM = 0, 1, 2
LIFE_REFERENCE, LIFE_B3S23 = 0, 1
FORM_U8, FORM_BITS = 0, 1
STAR_AUTO, STAR_SCALAR2, STAR_SCALAR4, STAR_TMA_X4, STAR_TMA_X2, STAR_VEC, STAR_TB2, STAR_TB2_8, STAR_TMA_X4R4 = 0, 2, 4, 8, 9, 10, 11, 12, 13

_P = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64
_f = ctypes.c_float
_d = ctypes.c_double

# name -> argtypes (restype is int unless listed in _RESTYPES)
SIGNATURES = {
    "appfis_gb_last_error": [],
    "appfis_gb_version": [],
    "appfis_gb_stream_sync": [_P],
    "appfis_gb_test_stall_next": [_i, ctypes.c_ulonglong],
    "appfis_gb_reduce": [_P, _i, _i, _i, _P, _i, _P, _P],
    "appfis_gb_reduce_host": [_P, _i, _i, _i, _P, _i, _P, _P],
    "appfis_gb_reduce_noalloc": [_P, _i, _i, _i, _P, _i, _P, _P],
    "appfis_gb_ghost_periodic": [_P, _i, _i, _P, _i, _P],
    "appfis_gb_life_u8": [_P, _P, _i, _i, _i, _i, _P, _P],
    "appfis_gb_life_pack": [_P, _P, _i, _i, _P],
    "appfis_gb_life_unpack": [_P, _P, _i, _i, _P],
    "appfis_gb_life_bits": [_P, _P, _i, _i, _i, _i, _P, _P],
    "appfis_gb_life_from_i32": [_P, _i, _i, _P, _i, _i, _P],
    "appfis_gb_life_to_i32": [_P, _i, _i, _P, _i, _i, _P],
    "appfis_gb_life_population_u8": [_P, _i64, _P, _P],
    "appfis_gb_life_population_bits": [_P, _i64, _P, _P],
    "appfis_gb_life_job": [_P, _P, _i, _i, _i, _i, _i, _P],
    "appfis_gb_heat2d": [_P, _P, _i, _i, _i, _i, _f, _f, _P, _P],
    "appfis_gb_heat2d_sweep": [_P, _P, _i, _i, _i, _f, _f, _P],
    "appfis_gb_heat2d_job": [_P, _i, _i, _i, _f, _f, _P],
    "appfis_gb_himeno": [_P, _P, _P, _i, _i, _i, _i, _i, _f, _P, _P, _P],
    "appfis_gb_himeno_mixed": [_P, _P, _P, _P, _i, _i, _i, _i, _i, _i, _f, _P, _P, _P],
    "appfis_gb_himeno_mixed_ex": [_P, _P, _P, _P, _i, _i, _i, _i, _i, _i, _f, _i, _P, _P, _P],
    "appfis_gb_himeno_job": [_P, _P, _i, _i, _i, _i, _f, _i, _i, _P],
    "appfis_gb_star_r4": [_P, _P, _i, _i, _i, _i, _i, _i, _i, _f, _P, _i, _i, _P, _P],
    "appfis_gb_star_r4_tune": [_P, _P, _i, _i, _i, _i, _i, _i, _f, _P, _P, _P, _P, _P],
    "appfis_gb_heat2d_f64": [_P, _P, _i, _i, _i, _i, _d, _d, _P, _P],
    "appfis_gb_himeno_f64": [_P, _P, _P, _i, _i, _i, _i, _i, _d, _P, _P, _P],
    "appfis_gb_star_r4_f64": [_P, _P, _i, _i, _i, _i, _i, _i, _d, _P, _P, _P],
    "appfis_gb_flood_run": [_P, _i, _i, _P, _P, _P, _P, _P, _P],
    "appfis_gb_flood_setup": [_P, _i, _P, _P, _P, _P, _d, _P],
    "appfis_gb_flood_run_sources": [_P, _P, _i, _i, _P, _P, _P, _P, _P, _P],
    "appfis_gb_flood_job": [_i, _P, _P, _P, _P, _P, _P, _d, _P, _i, _P, _P, _P],
}


class FloodDomain(ctypes.Structure):
    """appfis_gb_flood_domain"""
    _fields_ = [("nx", _i), ("ny", _i), ("pitch", _i), ("h", _P * 2), ("qx", _P * 2), ("qy", _P * 2),
                ("dem", _P), ("n2", _P)]


class FloodSources(ctypes.Structure):
    """appfis_gb_flood_sources"""
    _fields_ = [("n", _i), ("nt", _i), ("cells", _P), ("times", _P), ("flows", _P)]


class FloodParams(ctypes.Structure):
    """appfis_gb_flood_params"""
    _fields_ = [("dx", _d), ("courant", _d), ("hextra", _d), ("t_end", _d), ("print_interval", _d),
                ("time_step", _d), ("t_start", _d), ("max_steps", _i), ("flags", _i)]


FLOOD_SKIP_DRY = 1
FLOOD_TWO_PHASE = 2
FLOOD_FUSED = 4
FLOOD_UNSTAGED = 8


def flood_job(domains, dx, courant, hextra, manning, t_end, print_interval=None, time_step=1.0, max_steps=0,
              dtype=F32, qx=None, qy=None, flags=0):
    """Run a batch of flood domains from host arrays.  domains: list of (dem, h) FP64 (ny, nx)
    arrays.  Returns dict(h=[...], qx=[...], qy=[...], steps=[...], mass=[(m0, m1)], dts=[...])."""
    import numpy as np
    nd = len(domains)
    nx = (_i * nd)(*[d[0].shape[1] for d in domains])
    ny = (_i * nd)(*[d[0].shape[0] for d in domains])
    dems = [np.ascontiguousarray(d[0], dtype=np.float64) for d in domains]
    hs = [np.ascontiguousarray(d[1], dtype=np.float64).copy() for d in domains]
    qxs = [np.zeros_like(a) if qx is None else np.ascontiguousarray(qx[k], dtype=np.float64).copy() for k, a in enumerate(hs)]
    qys = [np.zeros_like(a) if qy is None else np.ascontiguousarray(qy[k], dtype=np.float64).copy() for k, a in enumerate(hs)]
    P = lambda arrs: (_P * nd)(*[a.ctypes.data for a in arrs])
    prm = FloodParams(dx, courant, hextra, t_end, t_end if print_interval is None else print_interval, time_step, 0.0,
                      max_steps, flags)
    steps = (_i * nd)()
    mass = (_d * (2 * nd))()
    dtlog = np.zeros(nd * max(max_steps, 1), dtype=np.float64)
    call("appfis_gb_flood_job", nd, nx, ny, P(dems), P(hs), P(qxs), P(qys), manning, ctypes.byref(prm), dtype, steps,
         mass, dtlog.ctypes.data if max_steps > 0 else None)
    st = list(steps)
    return dict(h=hs, qx=qxs, qy=qys, steps=st, mass=[(mass[2 * k], mass[2 * k + 1]) for k in range(nd)],
                dts=[dtlog[k * max_steps:k * max_steps + st[k]] for k in range(nd)] if max_steps > 0 else None)
_RESTYPES = {"appfis_gb_last_error": ctypes.c_char_p}


class AppfisError(RuntimeError):
    def __init__(self, name, status, message):
        super().__init__("%s failed with status %d: %s" % (name, status, message))
        self.status = status


_lib = None


def declared_symbols():
    """Every function name declared in include/appfis_gb.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"APPFIS_GB_API\s+(?:const\s+char\s*\*|int)\s+(appfis_gb_\w+)\s*\(", text)))


def lib():
    """The loaded library with argtypes set; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libappfis_gb.so is not built (run appfis_gb300.build.build() or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = L
    return _lib


def call(name, *args):
    """Call an entry point; raise AppfisError with the library's message on a non-zero status."""
    st = getattr(lib(), name)(*args)
    if st != OK:
        raise AppfisError(name, st, lib().appfis_gb_last_error().decode(errors="replace"))
    return st


def ptr(x):
    """Device/host address of a torch tensor or numpy array (or an int / None)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data
