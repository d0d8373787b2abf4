"""bench.py helpers that need no GPU: the DRAM traffic figures parsed from the ncu summaries
under profiles/ (the bench line's roofline.traffic and the per-workload traffic), the peak
table, and the reference arm's JSON line on a small sample."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


@pytest.mark.parametrize("kernel", ["life_bits_tb", "life_u8_bulk", "heat2d_regs", "himeno_tma<plain>", "himeno_mixed2",
                                    "star_r4_tma<float>", "star_r4_tma<half>"])
def test_profiled_traffic_present(kernel):
    t = bench.profiled_traffic(kernel)
    assert t is not None and t > 1e6


def test_profiled_traffic_absent():
    assert bench.profiled_traffic("no_such_kernel") is None


def test_peaks_measured_or_fallback():
    v, kind = bench.peaks()
    assert v > 1000 and kind in ("measured", "fallback")


@pytest.mark.slow
def test_reference_arm_json_line():
    """`bench.py --impl reference` prints one JSON line with the reference arm's keys."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3",
                        "--ref-gens", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["unit"] == "GLUP/s" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
