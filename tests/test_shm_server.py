"""The shared-memory server (beamformer_gb300_serve): clients of the reference's
protocol push parameters, pipeline, channel mapping and filters, upload RF and
read back the beamformed frame and the timing table through the region. On the
CPU the reference's own client library (when oracle/_ref holds it) and the
restated client (oracle/shm_client.c) check the protocol: every call returns,
no lock is left held, filters created through the queue land in the library.
On the GPU the restated client's frame is checked against the oracle."""
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_CLIENT = os.path.join(ROOT, "oracle", "_ref", "libref_client.so")


def serve_session(lib, kind, tmp_path, timeout=60):
    t = threading.Thread(target=lib.beamformer_gb300_serve, args=(30000,), daemon=True)
    t.start()
    for _ in range(200):
        if os.path.exists("/dev/shm/ogl_beamformer_shared_memory"):
            break
        time.sleep(0.02)
    out = str(tmp_path / "frame.npy")
    try:
        r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "shm_session.py"), kind, out],
                           capture_output=True, text=True, timeout=timeout)
    finally:
        lib.beamformer_gb300_serve_stop()
        t.join(timeout=10)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1]), np.load(out)


def check_protocol(lib, res):
    for k in ("params", "pipeline", "chmap", "filter", "filter0"):
        assert res[k] == 1, (k, res)
    assert res["locks"] == [0] * 10, res["locks"]
    taps = np.zeros(64, np.float32)
    n = abi.ctypes.c_int32()
    assert lib.beamformer_gb300_get_filter(2, taps.ctypes.data_as(abi.ctypes.POINTER(abi.ctypes.c_float)), 64,
                                           abi.ctypes.byref(n))
    from oracle.bf_oracle import kaiser
    assert n.value == 36 and np.array_equal(taps[:36], kaiser(5e6, 25e6, 5.65, 36))


@pytest.mark.skipif(not os.path.exists(REF_CLIENT), reason="the reference's client library is built from its checkout")
def test_reference_client_protocol(lib, tmp_path):
    res, _ = serve_session(lib, "reference", tmp_path)
    check_protocol(lib, res)


def test_restated_client_protocol(lib, tmp_path):
    res, _ = serve_session(lib, "restated", tmp_path)
    assert res["open"] == 1
    check_protocol(lib, res)


@pytest.mark.gpu
def test_server_beamforms_through_shared_memory(lib, tmp_path):
    res, frame = serve_session(lib, "restated", tmp_path)
    assert res["beamform"] == 1 and res["timings"] == 1, res
    check_protocol(lib, res)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from bf_cases import small_params, small_raw, check_volume
    from oracle.bf_oracle import OraclePipeline
    SH = abi.SHADER
    bp = small_params(S=512, C=16, T=16, points=(24, 1, 20))
    raw = small_raw(bp)
    orc = OraclePipeline()
    orc.bp = bp
    orc.shaders = [SH["Decode"], SH["Demodulate"], SH["DAS"]]
    orc.data_kind = abi.DATA_KIND["Int16"]
    orc.create_kaiser(5.65, 5e6, 25e6, 32, 0)
    orc.create_kaiser(5.65, 5e6, 25e6, 36, 2)
    chmap = np.arange(256, dtype=np.int16)
    chmap[:16] = np.random.default_rng(5).permutation(16)
    orc.chmap = chmap
    orc.focal = np.zeros((256, 2), np.float32)
    orc.sparse = np.arange(256, dtype=np.int16)
    ref = orc.compute(raw)
    check_volume(frame, ref["frame"], "frame through the shared-memory server")


def test_server_executable_starts_and_exits():
    exe = os.path.join(ROOT, "ogl_beamforming_cuda_gb300", "lib", "ogl_beamformer_server")
    r = subprocess.run([exe, "--idle-exit-ms", "200"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert "serving /ogl_beamformer_shared_memory" in r.stderr
    assert not os.path.exists("/dev/shm/ogl_beamformer_shared_memory")
