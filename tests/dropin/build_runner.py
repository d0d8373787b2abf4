"""Builds tests/dropin/_build/dropin_runner (the drop-in test program) against the engine's
drop-in headers and libappfis_gb.so.  -fmad=false keeps every multiply and add separately
rounded so that results can be compared bit for bit with the CPU oracle."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
EXE = os.path.join(OUT, "dropin_runner")
SRC = os.path.join(HERE, "dropin_runner.cu")
LIBDIR = os.path.join(ROOT, "appfis_gb300")


def _newest_input():
    files = [SRC, os.path.join(LIBDIR, "libappfis_gb.so")]
    for d in (os.path.join(LIBDIR, "Appfis"), os.path.join(LIBDIR, "csrc")):
        files += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".hpp", ".cuh"))]
    return max(os.path.getmtime(f) for f in files)


def build():
    os.makedirs(OUT, exist_ok=True)
    stamp = EXE + ".arch"
    import platform
    fresh = (os.path.exists(EXE) and os.path.exists(stamp) and open(stamp).read() == platform.machine()
             and os.path.getmtime(EXE) >= _newest_input())
    if fresh:
        return EXE
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
           "-I", os.path.join(ROOT, "include"), "-o", EXE, SRC, "-L", LIBDIR, "-lappfis_gb",
           "-Xlinker", "-rpath=" + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the drop-in runner failed:\n" + r.stderr[-4000:])
    with open(stamp, "w") as f:
        f.write(platform.machine())
    return EXE
