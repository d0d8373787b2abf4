"""Builds the reference's five sample applications, unchanged, against the drop-in headers
(appfis_gb300/Appfis) and libappfis_gb.so, the way their makefiles build the APPFIS_CUDA
configuration (nvcc -x cu -DAPPFIS_CUDA=1), by default plus -fmad=false so that the functors' multiplies
and adds round separately like the reference's CPU build.

The application sources come from oracle/_ref/apps/<app>.gb.cpp (flattened by
oracle/build_ref.py from the reference tree; git-ignored, never committed).  Executables go to
the same folder as <app>.gb (<app>.gbfma without -fmad=false); they are rebuilt when the library, the drop-in headers or the
source change, or when they were built for another host architecture."""
import os
import platform
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
APPS_DIR = os.path.join(ROOT, "oracle", "_ref", "apps")
LIBDIR = os.path.join(ROOT, "appfis_gb300")
APPS = ["HeatDiffusion", "GameOfLife", "Himeno", "FDTD3d", "Triton"]


def source(app):
    return os.path.join(APPS_DIR, "%s.gb.cpp" % app)


def _newest_input(src):
    files = [src, os.path.join(LIBDIR, "libappfis_gb.so")]
    d = os.path.join(LIBDIR, "Appfis")
    files += [os.path.join(d, f) for f in os.listdir(d) if f.endswith(".hpp")]
    return max(os.path.getmtime(f) for f in files)


# The one line an application adds to route its Execute*D loop to a hand-written kernel
# (appfis_gb300/Appfis/Fast.hpp), inserted right after its `config.GridsToUpdate(...);`.
FAST_LINE = {"GameOfLife": "APPFIS::UseFastKernel(config, APPFIS::FAST_LIFE);",
             "Himeno": "APPFIS::UseFastKernel(config, APPFIS::FAST_HIMENO);",
             "FDTD3d": "APPFIS::UseFastKernel(config, APPFIS::FAST_STAR_R4);"}
FAST_APPS = sorted(FAST_LINE)


def fast_source(app):
    """<app>.fast.cpp: the flattened application with its one opt-in line added."""
    src = source(app)
    dst = os.path.join(APPS_DIR, "%s.fast.cpp" % app)
    text = open(src).read()
    lines = text.split("\n")
    hits = [n for n, l in enumerate(lines) if l.strip().startswith("config.GridsToUpdate(")]
    if len(hits) != 1:
        raise RuntimeError("%s: expected one config.GridsToUpdate line, found %d" % (app, len(hits)))
    indent = lines[hits[0]][: len(lines[hits[0]]) - len(lines[hits[0]].lstrip())]
    lines.insert(hits[0] + 1, indent + FAST_LINE[app])
    out = "\n".join(lines)
    if not (os.path.exists(dst) and open(dst).read() == out):
        with open(dst, "w") as f:
            f.write(out)
    return dst


def build_one(app, exact=True, fast=False):
    """exact: -fmad=false (the functors' multiplies and adds rounded separately, as on the
    reference's CPU build); otherwise nvcc's default contraction, as the reference's own GPU
    build uses (for timing against it).  fast: the application with its UseFastKernel line."""
    src = fast_source(app) if fast else source(app)
    exe = os.path.join(APPS_DIR, "%s.%s" % (app, "fast" if fast else ("gb" if exact else "gbfma")))
    stamp = exe + ".arch"
    if (os.path.exists(exe) and os.path.exists(stamp) and open(stamp).read() == platform.machine()
            and os.path.getmtime(exe) >= _newest_input(src)):
        return exe
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-x", "cu", "-DAPPFIS_CUDA=1", "-O3", "-std=c++11",
           "-w", "-I", os.path.join(LIBDIR, "Appfis"), "-I", os.path.join(ROOT, "include"), "-o", exe, src,
           "-L", LIBDIR, "-lappfis_gb", "-Xlinker", "-rpath=" + LIBDIR] + (["-fmad=false"] if exact else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building %s against the drop-in failed:\n%s" % (app, r.stderr[-4000:]))
    with open(stamp, "w") as f:
        f.write(platform.machine())
    return exe


def available():
    return all(os.path.exists(source(a)) for a in APPS)


def build(apps=APPS, exact=True, fast=False):
    with ThreadPoolExecutor(max_workers=len(apps)) as ex:
        return dict(zip(apps, ex.map(lambda a: build_one(a, exact, fast), apps)))
