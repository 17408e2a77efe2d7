"""The C-ABI from a C program: tests/c_driver/kat_driver.c is compiled
with gcc against include/rimp2_gpu.h and linked with the library, as a C
host program would be.  Without a GPU it must report RIMP2_ERR_NODEV (exit
2); on a GB300 it must reproduce the reference's closed-form fixtures
through rimp2_steps5to8 and the closed-form energy through rimp2_energy."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT, has_gpu

SRC = os.path.join(ROOT, "tests", "c_driver", "kat_driver.c")


def _build(tmp_path):
    from rimp2_gpu_gb300 import _lib
    _lib.lib()  # fails loudly if the library is not built
    lib = _lib.LIB_PATH
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "kat_driver")
    libdir = os.path.dirname(lib)
    cmd = [gcc, "-O2", "-std=c99", SRC, "-I", os.path.join(ROOT, "include"), "-L", libdir,
           "-lrimp2_gpu_gb300", "-Wl,-rpath," + libdir, "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_builds_and_reports_no_gpu(tmp_path):
    exe = _build(tmp_path)
    if has_gpu():
        pytest.skip("GPU present: covered by the GPU test")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2, r.stdout + r.stderr


@pytest.mark.gpu
def test_c_driver_reference_fixtures(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
