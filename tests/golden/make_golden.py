"""Generates the golden fixtures in this directory by running the REFERENCE's own CPU path
(oracle/_ref: the reference's headers built with APPFIS_CPU and a single-rank MPI stand-in)
on small seeded inputs.  Needs the reference tree (builds oracle/_ref first).

    python tests/golden/make_golden.py            # the small fixtures (seconds)
    python tests/golden/make_golden.py --full-gol # the full GameOfLife workload (minutes)

Each fixture holds the inputs, the reference's outputs and its printed scalars; tests check the
oracle restatement and the GPU kernels against them.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from appfis_gb300 import workloads as W  # noqa: E402
from oracle import build_ref, oracle as O  # noqa: E402


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, {k: v.shape for k, v in arrays.items()})


def gol(nx, ny, gens, seed):
    cells = W.gol_cells(nx, ny, 0.3, seed)
    res, (out,) = O.run_ref("gol", [nx, ny, gens, 1, "{in0}", "{out0}"], [cells], [(np.uint8, None)])
    save("gol_%dx%d_g%d" % (nx, ny, gens), cells=cells, out=out.reshape(ny, nx), live=np.int64(res["live"]),
         gens=np.int64(gens))


def heat2d(nx, ny, iters, seed):
    f = W.heat2d_padded(nx, ny, 1.0, seed)
    res, (out,) = O.run_ref("heat2d", [nx, ny, iters, 1, 0.2, 1.0, "{in0}", "{out0}"],
                            [np.ascontiguousarray(f[1:-1, 1:-1])], [(np.float32, None)])
    save("heat2d_%dx%d_i%d" % (nx, ny, iters), padded=f, out=out.reshape(ny + 2, nx + 2), iters=np.int64(iters),
         stats=np.array([res["max"], res["min"], res["sum"]], dtype=np.float64))


def himeno(nx, ny, nz, iters, seed):
    coef = W.himeno_coef(nx, ny, nz, seed=seed)
    p = W.himeno_p(nx, ny, nz)
    p[1:-1, 1:-1, 1:-1] += W.uniform(seed + 1, nx * ny * nz).reshape(nz, ny, nx).astype(np.float32) * np.float32(0.1)
    res, (out, gosa) = O.run_ref("himeno", [nx, ny, nz, iters, 1, 0.8, "{in0}", "{in1}", "{out0}", "{out1}"],
                                 [coef, np.ascontiguousarray(p[1:-1, 1:-1, 1:-1])],
                                 [(np.float32, None), (np.float64, None)])
    save("himeno_%dx%dx%d_i%d" % (nx, ny, nz, iters), coef=coef, p=p, out=out.reshape(p.shape), gosa=gosa,
         iters=np.int64(iters), sum=np.float64(res["sum"]))


def fdtd(nx, ny, nz, iters, seed):
    f = W.fdtd_padded(nx, ny, nz, seed)
    res, (out,) = O.run_ref("fdtd", [nx, ny, nz, iters, 1, 0.1, "{in0}", "{out0}"],
                            [np.ascontiguousarray(f[4:-4, 4:-4, 4:-4])], [(np.float32, None)])
    save("fdtd_%dx%dx%d_i%d" % (nx, ny, nz, iters), padded=f, out=out.reshape(f.shape), iters=np.int64(iters),
         coeff=np.float32(0.1))


def triton(nx, ny, steps, seed):
    dem, h = W.triton_domain(ny, nx, seed)
    args = [nx, ny, 1, 10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0, steps, "{in0}", "{in1}", "{out0}", "{out1}"]
    res, (out, dts) = O.run_ref("triton", args, [dem, h], [(np.float64, None), (np.float64, None)])
    n = nx * ny
    save("triton_%dx%d_s%d" % (nx, ny, steps), dem=dem, h0=h, h=out[:n].reshape(ny, nx), qx=out[n:2 * n].reshape(ny, nx),
         qy=out[2 * n:].reshape(ny, nx), dts=dts, params=np.array([10.0, 0.5, 1e-3, 0.035, 600.0, 600.0, 1.0]),
         steps=np.int64(res["steps"]))


def gol_full(nx=16384, ny=16384, gens=2000, seed=42, p=0.3):
    """The benchmark's GameOfLife workload through the reference's own CPU path, all host
    threads: the final population and a SHA-256 of the final interior (u8, x fastest) go to a
    small JSON fixture, so a GPU run of the same 5.4e11 cell updates can be checked bit for bit
    without the 268 MB state."""
    cells = W.gol_cells(nx, ny, p, seed)
    res, (out,) = O.run_ref("gol", [nx, ny, gens, os.cpu_count(), "{in0}", "{out0}"], [cells], [(np.uint8, None)])
    rec = {"nx": nx, "ny": ny, "gens": gens, "seed": seed, "p": p, "rule": "reference (S234, stale carry)",
           "live": int(res["live"]), "live_recount": int(out.sum(dtype=np.int64)),
           "sha256": hashlib.sha256(np.ascontiguousarray(out).tobytes()).hexdigest(),
           "input_sha256": hashlib.sha256(np.ascontiguousarray(cells).tobytes()).hexdigest(),
           "reference_seconds": res["seconds"], "threads": os.cpu_count()}
    name = "gol_%dx%d_g%d.json" % (nx, ny, gens)
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(rec, f, indent=1)
    print(name, rec)


if __name__ == "__main__":
    build_ref.build()
    if "--full-gol" in sys.argv:
        gol_full()
        sys.exit(0)
    gol(37, 29, 9, 5)
    gol(64, 48, 17, 6)
    heat2d(19, 23, 17, 3)
    heat2d(64, 40, 40, 4)
    himeno(13, 11, 9, 7, 11)
    fdtd(12, 10, 9, 3, 5)
    triton(52, 40, 60, 77)
    triton(33, 47, 150, 78)
