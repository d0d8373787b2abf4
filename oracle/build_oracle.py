"""Build recipe for the oracle library oracle/_build/liboracle.so — TEST INFRASTRUCTURE ONLY.

Compiles oracle/appfis_oracle.cpp (the CPU restatement of the reference's algorithms) with
-ffp-contract=off so that x86-64 and aarch64 builds give bit-identical results.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "appfis_oracle.cpp")
LIB = os.path.join(OUT_DIR, "liboracle.so")
_STAMP = os.path.join(OUT_DIR, "liboracle.arch")


def build():
    os.makedirs(OUT_DIR, exist_ok=True)
    arch = platform.machine()
    fresh = (os.path.exists(LIB) and os.path.exists(_STAMP) and open(_STAMP).read() == arch
             and os.path.getmtime(LIB) >= os.path.getmtime(SRC))
    if fresh:
        return LIB
    cmd = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-std=c++14", "-shared", "-fPIC", SRC, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the oracle failed:\n" + r.stderr[-4000:])
    with open(_STAMP, "w") as f:
        f.write(arch)
    return LIB


if __name__ == "__main__":
    print(build())
