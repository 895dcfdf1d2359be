"""Client session for tests/test_shm_server.py, run in its own process: drives a
running beamformer_gb300_serve through a client library of the shared-memory
protocol (the reference's own, or the restated oracle/shm_client.c) and prints
one JSON line with the results."""
import ctypes
import json
import mmap
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from ogl_beamforming_cuda_gb300 import abi  # noqa: E402  (struct layouts only; the library is not loaded)
from bf_cases import small_params, small_raw  # noqa: E402


def lock_states():
    with open("/dev/shm/ogl_beamformer_shared_memory", "r+b") as f:
        m = mmap.mmap(f.fileno(), 4096)
        v = np.frombuffer(m[8:48], np.int32).tolist()
        m.close()
    return v


def main():
    kind, out_path = sys.argv[1], sys.argv[2]
    SH = abi.SHADER
    bp = small_params(S=512, C=16, T=16, points=(24, 1, 20))
    raw = small_raw(bp)
    pipeline = (ctypes.c_int32 * 3)(SH["Decode"], SH["Demodulate"], SH["DAS"])
    chmap = np.arange(256, dtype=np.int16)
    chmap[:16] = np.random.default_rng(5).permutation(16)
    pts = (ctypes.c_int32 * 3)(24, 1, 20)
    out = np.zeros(2 * 24 * 20, np.float32)
    table = (ctypes.c_uint8 * 2048)()
    res = {}
    if kind == "reference":
        L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_client.so"))
        L.beamformer_set_global_timeout(5000)
        res["params"] = L.beamformer_push_parameters(ctypes.byref(bp))
        res["pipeline"] = L.beamformer_push_pipeline(pipeline, 3, abi.DATA_KIND["Int16"])
        res["chmap"] = L.beamformer_push_channel_mapping(chmap.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), 256)
        f = ctypes.c_float
        L.beamformer_create_kaiser_low_pass_filter.argtypes = [f, f, f, ctypes.c_int16, ctypes.c_uint8]
        res["filter"] = L.beamformer_create_kaiser_low_pass_filter(5.65, 5e6, 25e6, 36, 2)
        res["filter0"] = L.beamformer_create_kaiser_low_pass_filter(5.65, 5e6, 25e6, 32, 0)
        res["beamform"] = L.beamform_data_synchronized(raw.ctypes.data_as(ctypes.c_void_p), raw.nbytes, pts,
                                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 5000)
        res["timings"] = L.beamformer_compute_timings(ctypes.byref(table), 5000)
        res["error"] = L.beamformer_get_last_error()
    else:
        from oracle.bf_oracle import build_shm_client
        L = ctypes.CDLL(build_shm_client())
        f = ctypes.c_float
        L.shmc_create_kaiser.argtypes = [f, f, f, ctypes.c_int16, ctypes.c_uint8]
        res["open"] = L.shmc_open()
        res["params"] = L.shmc_push_parameters(ctypes.byref(bp), 5000)
        res["pipeline"] = L.shmc_push_pipeline(pipeline, 3, abi.DATA_KIND["Int16"], 5000)
        res["chmap"] = L.shmc_push_channel_mapping(chmap.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), 256, 5000)
        res["filter"] = L.shmc_create_kaiser(5.65, 5e6, 25e6, 36, 2)
        res["filter0"] = L.shmc_create_kaiser(5.65, 5e6, 25e6, 32, 0)
        res["beamform"] = L.shmc_beamform_data_synchronized(raw.ctypes.data_as(ctypes.c_void_p), raw.nbytes, pts,
                                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 5000)
        res["timings"] = L.shmc_compute_timings(ctypes.byref(table), 2048, 5000)
    res["locks"] = lock_states()
    np.save(out_path, out)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
