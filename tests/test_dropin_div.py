"""The drop-in executors number the points of ragged-width planes consecutively and recover the
row and column with a multiply-shift division (Appfis/Runtime.hpp MakeDiv / DivQ).  This host
program, compiled against the headers, checks the quotients against exact division for 40 000
divisors, including the extremes of the 31-bit range the launches use.  No GPU needed."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_multiply_shift_division_is_exact():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "div_check")
        cmd = ["nvcc", "-std=c++11", "-x", "cu", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "appfis_gb300"),
               os.path.join(ROOT, "tests", "dropin", "div_check.cu"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
