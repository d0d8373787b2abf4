"""The reference's five sample applications build UNCHANGED against the drop-in headers
(appfis_gb300/Appfis) with nvcc for sm_103a, the way their makefiles build the APPFIS_CUDA
configuration (nvcc -x cu -DAPPFIS_CUDA=1 -std=c++11).  The sources are copied to a temporary
tree whose Appfis/ is the drop-in; they are compiled and linked, not run (that needs the GPU
and the application input files).  Skipped where the reference tree is absent."""
import os
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference checkout: $APPFIS_REF_ROOT, else a directory named `reference` beside this repository
REF = os.environ.get("APPFIS_REF_ROOT") or os.path.normpath(os.path.join(ROOT, "..", "reference"))
APPS = ["HeatDiffusion", "GameOfLife", "Himeno", "FDTD3d", "Triton"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "Appfis")), reason="reference sources not present")
def test_reference_apps_build_unchanged():
    from appfis_gb300 import build
    build.build()
    with tempfile.TemporaryDirectory() as td:
        os.symlink(os.path.join(ROOT, "appfis_gb300", "Appfis"), os.path.join(td, "Appfis"))
        for a in APPS:
            shutil.copytree(os.path.join(REF, a, "src"), os.path.join(td, a, "src"))

        def compile_app(a):
            cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-x", "cu", "-DAPPFIS_CUDA=1", "-O1", "-std=c++11",
                   "-I", os.path.join(ROOT, "include"), "-o", os.path.join(td, a + ".bin"), os.path.join(td, a, "src", "main.cpp"),
                   "-L", os.path.join(ROOT, "appfis_gb300"), "-lappfis_gb"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            return a, r.returncode, r.stderr[-3000:]

        with ThreadPoolExecutor(max_workers=5) as ex:
            results = list(ex.map(compile_app, APPS))
        failed = [(a, err) for a, rc, err in results if rc != 0]
        assert not failed, failed
