"""ctypes bindings of the oracle library and runners for the reference harnesses.

TEST INFRASTRUCTURE ONLY: used as the checker by tests/, __graft_entry__.smoke() and as the
timed CPU baseline by bench.py.  See appfis_oracle.cpp for the reference file:line each
restated routine follows.
"""
import ctypes
import json
import os
import subprocess
import tempfile

import numpy as np

from . import build_oracle, build_ref

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i, d, f = ctypes.c_int, ctypes.c_double, ctypes.c_float
        L.oracle_gol.argtypes = [i, i, i, P, P, i]
        L.oracle_gol_b3s23.argtypes = [i, i, i, P, i]
        L.oracle_population.argtypes = [P, ctypes.c_int64]
        L.oracle_population.restype = ctypes.c_int64
        L.oracle_heat2d_f32.argtypes = [i, i, i, f, f, P, P, i]
        L.oracle_heat2d_f64.argtypes = [i, i, i, d, d, P, P, i]
        for n, rt in (("oracle_reduce_f32", d), ("oracle_reduce_f64", d), ("oracle_reduce_i32", ctypes.c_int64)):
            getattr(L, n).argtypes = [P, i, i, P, i]
            getattr(L, n).restype = rt
        L.oracle_himeno_f32.argtypes = [i, i, i, i, f, P, P, P, P, i]
        L.oracle_himeno_f64.argtypes = [i, i, i, i, d, P, P, P, P, i]
        L.oracle_star_r4_f32.argtypes = [i, i, i, i, i, f, P, P, P, i]
        L.oracle_star_r4_f64.argtypes = [i, i, i, i, i, d, P, P, P, i]
        L.oracle_triton.argtypes = [i, i, i, d, d, d, d, d, d, d, i, P, P, P, P, P, P, i]
        L.oracle_triton.restype = i
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _threads(threads):
    return int(threads) if threads else (os.cpu_count() or 1)


# ---------------------------------------------------------------- GameOfLife
def gol(cells, gens, threads=None, old=None):
    """Reference rule (S234 + stale carry).  Returns (cur, old) after `gens` sweeps."""
    cur = np.ascontiguousarray(cells, dtype=np.uint8).copy()
    ny, nx = cur.shape
    o = np.zeros_like(cur) if old is None else np.ascontiguousarray(old, dtype=np.uint8).copy()
    lib().oracle_gol(nx, ny, int(gens), _p(cur), _p(o), _threads(threads))
    return cur, o


def gol_b3s23(cells, gens, threads=None):
    cur = np.ascontiguousarray(cells, dtype=np.uint8).copy()
    ny, nx = cur.shape
    lib().oracle_gol_b3s23(nx, ny, int(gens), _p(cur), _threads(threads))
    return cur


def population(cells):
    c = np.ascontiguousarray(cells, dtype=np.uint8)
    return int(lib().oracle_population(_p(c), c.size))


# ---------------------------------------------------------------- Heat2D
def heat2d(padded, iters, r, threads=None, dtype=np.float32):
    """padded: (ny+2, nx+2) field with the Dirichlet ghost ring; returns the field after iters."""
    a = np.ascontiguousarray(padded, dtype=dtype).copy()
    b = a.copy()
    ny, nx = a.shape[0] - 2, a.shape[1] - 2
    fn = lib().oracle_heat2d_f32 if dtype == np.float32 else lib().oracle_heat2d_f64
    fn(nx, ny, int(iters), r, r, _p(a), _p(b), _threads(threads))
    return a


# ---------------------------------------------------------------- reductions
def reduce(field, box, op):
    """op: 'max' | 'min' | 'sum' with the reference's seeds; box = (x0,x1,y0,y1[,z0,z1])."""
    a = np.ascontiguousarray(field)
    shape = a.shape if a.ndim == 3 else (1,) + a.shape
    b = list(box) + ([0, 1] if len(box) == 4 else [])
    bx = np.array(b, dtype=np.int32)
    code = {"max": 0, "min": 1, "sum": 2}[op]
    fn = {np.dtype(np.float32): lib().oracle_reduce_f32, np.dtype(np.float64): lib().oracle_reduce_f64,
          np.dtype(np.int32): lib().oracle_reduce_i32}[a.dtype]
    return fn(_p(a), shape[2], shape[1], _p(bx), code)


# ---------------------------------------------------------------- Himeno
def himeno(coef, p, iters, omega, threads=None, dtype=np.float32):
    """coef: (12, nz+2, ny+2, nx+2); p: padded (nz+2, ny+2, nx+2).  Returns (p, gosa[iters])."""
    c = np.ascontiguousarray(coef, dtype=dtype)
    a = np.ascontiguousarray(p, dtype=dtype).copy()
    w = np.zeros_like(a)
    gosa = np.zeros(int(iters), dtype=np.float64)
    nz, ny, nx = a.shape[0] - 2, a.shape[1] - 2, a.shape[2] - 2
    fn = lib().oracle_himeno_f32 if dtype == np.float32 else lib().oracle_himeno_f64
    fn(nx, ny, nz, int(iters), omega, _p(c), _p(a), _p(w), _p(gosa), _threads(threads))
    return a, gosa


# ---------------------------------------------------------------- radius-4 star (FDTD3d)
def star_r4(padded, iters, coeff=None, weights=None, threads=None, dtype=np.float32):
    """padded: (nz+8, ny+8, nx+8).  Reference form when `weights` is None (uniform `coeff`),
    else the weighted form with weights = (w_center, w1, w2, w3, w4)."""
    a = np.ascontiguousarray(padded, dtype=dtype).copy()
    b = a.copy()
    nz, ny, nx = a.shape[0] - 8, a.shape[1] - 8, a.shape[2] - 8
    w = np.zeros(5, dtype=dtype) if weights is None else np.asarray(weights, dtype=dtype)
    fn = lib().oracle_star_r4_f32 if dtype == np.float32 else lib().oracle_star_r4_f64
    fn(nx, ny, nz, int(iters), 0 if weights is None else 1, 0.0 if coeff is None else coeff, _p(w), _p(a), _p(b),
       _threads(threads))
    return a


# ---------------------------------------------------------------- Triton
def triton(dem, h, dx, courant, hextra, mann, t_end, print_interval=None, time_step=1.0, max_steps=0, qx=None, qy=None,
           prec=64, threads=None):
    """Returns dict(h, qx, qy, dts, steps, simtime) for one domain (interiors, FP64 arrays)."""
    dem = np.ascontiguousarray(dem, dtype=np.float64)
    ny, nx = dem.shape
    hh = np.ascontiguousarray(h, dtype=np.float64).copy()
    qxa = np.zeros_like(hh) if qx is None else np.ascontiguousarray(qx, dtype=np.float64).copy()
    qya = np.zeros_like(hh) if qy is None else np.ascontiguousarray(qy, dtype=np.float64).copy()
    cap = max_steps if max_steps > 0 else 1_000_000
    dts = np.zeros(cap, dtype=np.float64)
    st = ctypes.c_double(0.0)
    pi = t_end if print_interval is None else print_interval
    steps = lib().oracle_triton(int(prec), nx, ny, dx, courant, hextra, mann, t_end, pi, time_step, int(max_steps),
                                _p(dem), _p(hh), _p(qxa), _p(qya), _p(dts), ctypes.byref(st), _threads(threads))
    return dict(h=hh, qx=qxa, qy=qya, dts=dts[:steps].copy(), steps=steps, simtime=st.value)


# ---------------------------------------------------------------- the reference itself
def ref_available(name):
    return build_ref.exe_path(name) is not None


def run_ref(name, args, inputs, outputs):
    """Run oracle/_ref/ref_<name> with raw-file inputs.  inputs: list of np arrays written to
    temp files (paths substituted for '{in0}', '{in1}', ...); outputs: list of (dtype, count)
    read back from '{out0}', ... (count None: the whole file, 0: not read).  Returns
    (json_dict, [arrays])."""
    exe = build_ref.exe_path(name)
    if exe is None:
        raise RuntimeError("reference harness %s is not built on this machine" % name)
    with tempfile.TemporaryDirectory() as td:
        subs = {}
        for k, arr in enumerate(inputs):
            p = os.path.join(td, "in%d" % k)
            np.ascontiguousarray(arr).tofile(p)
            subs["in%d" % k] = p
        for k in range(len(outputs)):
            subs["out%d" % k] = os.path.join(td, "out%d" % k)
        argv = [exe] + [str(a).format(**subs) for a in args]
        r = subprocess.run(argv, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("%s failed (%d): %s" % (name, r.returncode, r.stderr[-2000:]))
        line = [l for l in r.stdout.splitlines() if l.startswith("{")][-1]
        res = json.loads(line)
        outs = []
        for k, (dt, cnt) in enumerate(outputs):
            if cnt == 0:  # not wanted
                outs.append(None)
                continue
            a = np.fromfile(subs["out%d" % k], dtype=dt)
            if cnt is not None:
                a = a[:cnt]
            outs.append(a)
        return res, outs
