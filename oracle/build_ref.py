"""Build recipe for oracle/_ref — ORACLE TEST INFRASTRUCTURE ONLY.

Builds the reference framework's own CPU path (header-only C++, APPFIS_CPU, OpenMP) into
small harness programs, one per workload (ref_harness/ref_*.cpp), against the single-rank
MPI stand-in in mpi_stub/.  Outputs go to oracle/_ref/ only (git-ignored).

Two stages, so that the same reference code can also run on a machine that has no copy of
the reference sources:

1. Where the reference tree is present (REF_ROOT: $APPFIS_REF_ROOT, else a checkout named
   `reference` beside this repository), each harness
   TU is flattened into oracle/_ref/ref_<name>.flat.cpp: every quoted #include that
   resolves (the harness helper, the reference's app header, Appfis/*.hpp, the MPI
   stand-in) is inlined in place, system <...> includes are kept.  Nothing of it is
   committed.
2. Each flattened TU is compiled with g++ -O3 -fopenmp -ffp-contract=off into
   oracle/_ref/ref_<name>.  -ffp-contract=off keeps the FP operation sequence identical on
   x86-64 (no FMA in the baseline ISA) and aarch64 (FMA contraction would otherwise be on).

Run:  python oracle/build_ref.py [--jobs N]
"""
import argparse
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("APPFIS_REF_ROOT") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
HARNESSES = ["gol", "heat2d", "himeno", "fdtd", "triton"]
INC_RE = re.compile(r'^\s*#\s*include\s+"([^"]+)"')


def _resolve(name, cur_dir, search):
    for d in [cur_dir] + search:
        p = os.path.normpath(os.path.join(d, name))
        if os.path.isfile(p):
            return p
    return None


def flatten(path, search, seen_once, out_lines):
    """Inline quoted includes recursively, each file once (all of them carry include guards
    or #pragma once, and the reference headers include each other in cycles)."""
    if path in seen_once:
        return
    seen_once.add(path)
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        lines = f.read().splitlines()
    out_lines.append('#line 1 "%s"' % os.path.basename(path))
    for n, line in enumerate(lines, 1):
        m = INC_RE.match(line)
        if m:
            target = _resolve(m.group(1), os.path.dirname(path), search)
            if target is not None:
                flatten(target, search, seen_once, out_lines)
                out_lines.append('#line %d "%s"' % (n + 1, os.path.basename(path)))
                continue
        if line.strip() == "#pragma once":
            continue
        out_lines.append(line)


# ------------------------------------------------------------------ the reference's applications
# The five sample applications, unchanged, as test inputs for the drop-in headers: each
# <app>/src/main.cpp is flattened twice into oracle/_ref/apps/ (git-ignored, never committed):
#   <app>.ref.cpp   — with the reference's own Appfis headers and the MPI stand-in inlined (built
#                     here with g++ and APPFIS_CPU: the reference's CPU path);
#   <app>.gb.cpp    — with the application's own files inlined and every Appfis include replaced
#                     by the drop-in's "Appfis.hpp" (built with nvcc by tests/dropin/build_apps.py).
APPS = ["HeatDiffusion", "GameOfLife", "Himeno", "FDTD3d", "Triton"]
APPS_DIR = os.path.join(OUT, "apps")


def _flatten_app(path, search, seen, out_lines, appfis_dir, dropin):
    if path in seen:
        return
    seen.add(path)
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        lines = f.read().splitlines()
    for line in lines:
        m = INC_RE.match(line)
        if m:
            target = _resolve(m.group(1), os.path.dirname(path), search)
            if target is not None:
                if dropin and os.path.dirname(target) == appfis_dir:
                    if "<appfis>" not in seen:
                        seen.add("<appfis>")
                        out_lines.append('#include "Appfis.hpp"')
                    continue
                _flatten_app(target, search, seen, out_lines, appfis_dir, dropin)
                continue
        if line.strip() == "#pragma once":
            continue
        out_lines.append(line)


def app_source(app, variant):
    return os.path.join(APPS_DIR, "%s.%s.cpp" % (app, variant))


def make_app_flats():
    """Writes the flattened application sources (needs the reference tree)."""
    os.makedirs(APPS_DIR, exist_ok=True)
    appfis_dir = os.path.normpath(os.path.join(REF_ROOT, "Appfis"))
    for app in APPS:
        main = os.path.join(REF_ROOT, app, "src", "main.cpp")
        for variant, dropin in (("ref", False), ("gb", True)):
            lines = []
            search = [os.path.join(HERE, "mpi_stub")] if not dropin else []
            _flatten_app(main, search, set(), lines, appfis_dir, dropin)
            text = "\n".join(lines) + "\n"
            path = app_source(app, variant)
            if not (os.path.exists(path) and open(path).read() == text):
                with open(path, "w") as f:
                    f.write(text)


def app_ref_exe(app):
    """The reference CPU build of an application (built on first use), or None."""
    src = app_source(app, "ref")
    if not os.path.exists(src):
        return None
    exe = os.path.join(APPS_DIR, "%s.ref" % app)
    if not (_runs_here(exe) and os.path.getmtime(exe) >= os.path.getmtime(src)):
        cmd = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-std=c++11", "-DAPPFIS_CPU=1", "-w", src, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building %s failed:\n%s" % (exe, r.stderr[-4000:]))
    return exe


def app_refgpu_exe(app):
    """The reference's own GPU build of an application (APPFIS_CUDA for sm_103a, the MPI
    stand-in; built on first use with nvcc), or None."""
    src = app_source(app, "ref")
    if not os.path.exists(src):
        return None
    exe = os.path.join(APPS_DIR, "%s.refgpu" % app)
    if not (_runs_here(exe) and os.path.getmtime(exe) >= os.path.getmtime(src)):
        cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-x", "cu", "-DAPPFIS_CUDA=1", "-O3", "-std=c++11", "-w",
               "-Xcompiler", "-fopenmp", src, "-o", exe, "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building %s failed:\n%s" % (exe, r.stderr[-4000:]))
    return exe


def flat_path(name):
    return os.path.join(OUT, "ref_%s.flat.cpp" % name)


def make_flat(name):
    search = [os.path.join(HERE, "ref_harness"), os.path.join(HERE, "mpi_stub"), REF_ROOT]
    lines = []
    flatten(os.path.join(HERE, "ref_harness", "ref_%s.cpp" % name), search, set(), lines)
    text = "\n".join(lines) + "\n"
    path = flat_path(name)
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


_ELF_MACHINE = {"x86_64": 0x3E, "aarch64": 0xB7, "arm64": 0xB7}


def _runs_here(exe):
    """True when exe is an ELF binary for this machine's architecture."""
    import platform
    try:
        with open(exe, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    want = _ELF_MACHINE.get(platform.machine())
    return len(head) == 20 and head[:4] == b"\x7fELF" and (want is None or head[18] == want)


def compile_one(name):
    src = flat_path(name)
    exe = os.path.join(OUT, "ref_%s" % name)
    if _runs_here(exe) and os.path.getmtime(exe) >= os.path.getmtime(src):
        return exe
    cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-std=c++11", "-DAPPFIS_CPU=1", "-w", src, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building %s failed:\n%s" % (exe, r.stderr[-4000:]))
    return exe


def build(jobs=8, quiet=True):
    """Build every harness that can be built here; return the list of executables."""
    os.makedirs(OUT, exist_ok=True)
    have_ref = os.path.isdir(os.path.join(REF_ROOT, "Appfis"))
    if have_ref:
        make_app_flats()
    names = []
    for name in HARNESSES:
        if have_ref:
            make_flat(name)
        if os.path.exists(flat_path(name)):
            names.append(name)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        exes = list(ex.map(compile_one, names))
    if not quiet:
        print("\n".join(exes))
    return exes


def exe_path(name):
    p = os.path.join(OUT, "ref_%s" % name)
    return p if _runs_here(p) else None


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=8)
    a = ap.parse_args()
    try:
        build(a.jobs, quiet=False)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
