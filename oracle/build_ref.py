"""Build recipe for oracle/_ref — ORACLE TEST INFRASTRUCTURE ONLY.

Builds the reference framework's own CPU path (header-only C++, APPFIS_CPU, OpenMP) into
small harness programs, one per workload (ref_harness/ref_*.cpp), against the single-rank
MPI stand-in in mpi_stub/.  Outputs go to oracle/_ref/ only (git-ignored).

Two stages, so that the same reference code can also run on a machine that has no copy of
the reference sources:

1. Where the reference tree is present (REF_ROOT, default /root/reference), each harness
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
REF_ROOT = os.environ.get("APPFIS_REF_ROOT", "/root/reference")
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
