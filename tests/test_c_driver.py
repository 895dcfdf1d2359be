"""A plain C11 program (tests/c_driver.c) against include/ogl_beamformer_lib.h and
libogl_beamformer_lib.so: the call sequence of the reference's own C drivers. It
compiles and links everywhere; it runs on the GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(ROOT, "ogl_beamforming_cuda_gb300", "lib")


def _build(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    if not os.path.exists(os.path.join(LIBDIR, "libogl_beamformer_lib.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "c_driver")
    r = subprocess.run(["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", f"{HERE}/c_driver.c",
                        f"-I{ROOT}/include", f"-L{LIBDIR}", "-logl_beamformer_lib", f"-Wl,-rpath,{LIBDIR}", "-lm",
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_compiles_and_links(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
def test_c_driver_runs(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok:"), r.stdout + r.stderr
