"""The job protocol driven from C (tests/finter_driver.c): the call sequence
of elwave.f90:141-190 through the C ABI alone, on the grid pattern and on a
node-permuted one, compiled with gcc against include/wtomo3d_gpu.h and
libwtomo3d_gpu.so."""
import os
import shutil
import subprocess

import pytest

import wtomo3d_gb300 as wt

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_driver_job_protocol(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    libdir = os.path.dirname(wt.LIB_PATH)
    exe = str(tmp_path / "finter_driver")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "finter_driver.c"), "-L", libdir, "-lwtomo3d_gpu",
                    "-Wl,-rpath," + libdir, "-lm", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
    assert r.stdout.count("relres") == 4
