"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer: the library's
planning and filter/matrix code (csrc/bf_host.cpp) and the CPU oracle
(oracle/bf_oracle.c), driven by tests/sanitize_host.cpp, which also cross-checks
the two over seeded random parameters and pipelines. No GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
SAN = ["-g", "-O1", "-fno-omit-frame-pointer", "-fsanitize=address,undefined", "-fno-sanitize-recover=all"]


def test_host_code_under_sanitizers(tmp_path):
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("no host compiler")
    inc = [f"-I{ROOT}/include", f"-I{ROOT}/ogl_beamforming_cuda_gb300/csrc", f"-I{ROOT}/oracle", f"-I{CUDA}/include"]
    jobs = [
        ["g++", "-std=c++17"] + SAN + inc + ["-c", f"{HERE}/sanitize_host.cpp", "-o", f"{tmp_path}/drv.o"],
        ["g++", "-std=c++17", "-ffp-contract=off"] + SAN + inc +
        ["-c", f"{ROOT}/ogl_beamforming_cuda_gb300/csrc/bf_host.cpp", "-o", f"{tmp_path}/host.o"],
        ["gcc", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"] + SAN +
        ["-c", f"{ROOT}/oracle/bf_oracle.c", "-o", f"{tmp_path}/oracle.o"],
        ["g++", "-fsanitize=address,undefined", "-fopenmp", f"{tmp_path}/drv.o", f"{tmp_path}/host.o",
         f"{tmp_path}/oracle.o", "-o", f"{tmp_path}/san", "-lm"],
    ]
    for cmd in jobs:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode and ("asan" in r.stderr or "ubsan" in r.stderr):
            pytest.skip("sanitizer runtime unavailable: " + r.stderr.strip().splitlines()[-1])
        assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1",
               OMP_NUM_THREADS="2")
    r = subprocess.run([f"{tmp_path}/san"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert " 0 mismatches" in r.stdout and "runtime error" not in r.stderr, r.stdout + r.stderr
