"""Builds libappfis_gb.so (the C-ABI library) from appfis_gb300/csrc/*.cu for sm_103a.

One nvcc process per translation unit, in parallel, objects in appfis_gb300/_build/, the shared
library next to this file.  An object is rebuilt when its source, any csrc header or
include/appfis_gb.h is newer, or when it was built for another host architecture.

    python -m appfis_gb300.build [--verbose]
"""
import glob
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libappfis_gb.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# per-file extra flags: the FP64 flood model keeps the reference's separate multiply/add rounding;
# the FP32 flood form (tolerance-checked against the FP64 oracle) uses the fast single-precision
# division / square root / cube root (~1-2 ulp), which its ~40 divisions per face make worthwhile
PER_FILE_FLAGS = {"flood_f64.cu": ["-fmad=false"], "flood_f32.cu": ["--use_fast_math"]}
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stamp():
    return os.path.join(BUILD, "arch.txt")


def _deps_mtime():
    files = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max([os.path.getmtime(f) for f in files] + [0.0])


def _compile(src, force, verbose):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps_mtime()):
        return obj
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + PER_FILE_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-6000:]))
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(verbose=False, extra=None):
    """Compile every csrc/*.cu and link libappfis_gb.so; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    arch = platform.machine()
    force = not (os.path.exists(_stamp()) and open(_stamp()).read() == arch)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    with open(_stamp(), "w") as f:
        f.write(arch)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv))
