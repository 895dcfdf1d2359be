"""Generate tests/golden/reference_outputs.npz from the reference itself.

Runs the reference's own code, built by oracle/build_ref.py from the reference
checkout (math.c host functions, and the decode/filter/das/sum/min_max compute
shaders compiled as C++), on small seeded inputs and stores inputs and outputs.
tests/test_golden.py checks the CPU oracle against these on any machine,
including ones without the reference checkout.

Stage dispatch parameters come from the oracle's restatement of the pipeline
planning (beamformer.c:303-481); everything else is the reference's output.
Usage: python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import bf_oracle as O  # noqa: E402
from ogl_beamforming_cuda_gb300 import synth  # noqa: E402
from ogl_beamforming_cuda_gb300.abi import BeamformerParameters, SHADER, DATA_KIND  # noqa: E402

vp = ctypes.c_void_p


def params_blob(bp):
    return np.frombuffer(bytes(bp), np.uint8).copy()


def main():
    libs = O.ref_libs()
    if libs is None:
        raise SystemExit("oracle/_ref is not built (python oracle/build_ref.py)")
    sh, mt, _ = libs
    sh.ref_decode.argtypes = [ctypes.POINTER(O.DecodeUBO), ctypes.c_int, ctypes.c_int, vp, ctypes.c_uint64, vp,
                              ctypes.c_uint64, vp, ctypes.c_uint64, vp, ctypes.c_int, vp, vp]
    sh.ref_filter.argtypes = [ctypes.POINTER(O.FilterUBO), ctypes.c_int, vp, ctypes.c_uint64, vp, ctypes.c_uint64,
                              vp, ctypes.c_int, vp, vp]
    sh.ref_das.argtypes = [ctypes.POINTER(BeamformerParameters), ctypes.c_int, vp, ctypes.c_uint64, vp, vp, vp, vp, vp]
    sh.ref_sum.argtypes = [vp, vp, ctypes.c_int, ctypes.c_float, vp]
    sh.ref_min_max.argtypes = [vp, vp, ctypes.c_int, vp, ctypes.c_uint64]
    mt.ref_kaiser.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int, vp]
    mt.ref_matched.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int, vp]
    mt.ref_i0.restype, mt.ref_i0.argtypes = ctypes.c_double, [ctypes.c_double]
    mt.ref_voxel_transform.argtypes = [ctypes.POINTER(BeamformerParameters), vp]
    mt.ref_hadamard.argtypes = [ctypes.c_int, vp, ctypes.c_int]

    g = {}
    rng = np.random.default_rng(20261203)

    # host math
    for n in (2, 4, 8, 16, 32, 64, 128, 12, 20):
        extra = 64 if n in (12, 20) else 0
        out = np.zeros(n * n + extra, np.int32)
        mt.ref_hadamard(n, out.ctypes.data, out.size)
        g[f"hadamard_{n}"] = out
    for L in (16, 36, 64, 128):
        out = np.zeros(L, np.float32)
        mt.ref_kaiser(5e6, 25e6, 5.65, L, out.ctypes.data)
        g[f"kaiser_{L}"] = out
    out = np.zeros(20, np.float32)
    mt.ref_matched(12.5e6, 12.5e6, 50e6, 20, out.ctypes.data)
    g["matched_20"] = out
    xs = np.array([0.0, 0.5, 3.0, 5.65, 8.0, 9.5, 30.0])
    g["i0_x"] = xs
    g["i0_y"] = np.array([mt.ref_i0(float(x)) for x in xs])
    for name, das, pts in (("hercules_plane", "HERCULES", (128, 1, 128)), ("hercules_vol", "HERCULES", (64, 32, 16)),
                           ("forces", "FORCES", (40, 1, 30))):
        bp = synth.make_parameters(points=pts, das_id=das)
        m = np.zeros(16, np.float32)
        mt.ref_voxel_transform(ctypes.byref(bp), m.ctypes.data)
        g[f"voxel_{name}_params"] = params_blob(bp)
        g[f"voxel_{name}"] = m

    # decode (first stage int16 and the demodulating variant)
    S, C, T = 32, 4, 16
    raw = rng.integers(-32768, 32767, size=(C, T, S), dtype=np.int16)
    chmap = np.concatenate([np.array([2, 0, 3, 1]), np.arange(4, 256)]).astype(np.int16)
    g["decode_raw"], g["decode_chmap"] = raw, chmap
    for label, shaders in (("plain", [SHADER["Decode"]]), ("tofloat", [SHADER["Decode"], SHADER["Demodulate"]])):
        bp = synth.make_parameters(samples=S, channels=C, transmits=T)
        p = O.plan(bp, shaders, [0] * len(shaders), DATA_KIND["Int16"], [(0, 8, 25e6, 5.65, 5e6), None, None, None])
        H = O.hadamard(T).astype(np.int8).ravel()
        out = np.zeros(2 * S * C * T, np.float32)
        scratch = np.zeros(4 * S * C * T, np.float32)
        sh.ref_decode(ctypes.byref(p.decode), p.shaders[0], 1, raw.ctypes.data, raw.nbytes, scratch.ctypes.data,
                      scratch.nbytes, out.ctypes.data, out.nbytes, H.ctypes.data, T, chmap.ctypes.data,
                      p.decode_dispatch)
        g[f"decode_{label}_params"] = params_blob(bp)
        g[f"decode_{label}_out"] = out
        if label == "tofloat":
            taps = np.zeros(8, np.float32)
            mt.ref_kaiser(5e6, 25e6, 5.65, 8, taps.ctypes.data)
            dem = np.zeros_like(out)
            sh.ref_filter(ctypes.byref(p.demod), p.shaders[1], out.ctypes.data, out.nbytes, dem.ctypes.data,
                          dem.nbytes, taps.ctypes.data, 8, chmap.ctypes.data, p.demod_dispatch)
            g["demod_taps"], g["demod_out"] = taps, dem

    # DAS (fast path, nearest and cubic; FORCES) on random channel data
    for label, das, interp, pts in (("herc_nearest", "HERCULES", 0, (12, 1, 10)), ("herc_cubic", "HERCULES", 1, (8, 2, 6)),
                                    ("forces_cubic", "FORCES", 1, (12, 1, 10))):
        bp = synth.make_parameters(samples=64, channels=8, transmits=8, points=pts, interpolate=interp, das_id=das,
                                   extent=((-4e-4, -4e-4, 1e-3), (4e-4, 4e-4, 2e-3)))
        bp.sampling_frequency, bp.time_offset = 12.5e6, 1e-7
        rf = rng.standard_normal(2 * 64 * 8 * 8).astype(np.float32)
        focal = np.zeros(512, np.float32)
        focal[1::2] = np.inf
        sparse = np.arange(256, dtype=np.int16)
        M = O.voxel_transform(bp)
        frame = np.zeros(2 * int(np.prod(pts)), np.float32)
        d = np.array(pts, np.int32)
        sh.ref_das(ctypes.byref(bp), 1, rf.ctypes.data, rf.nbytes, sparse.ctypes.data, focal.ctypes.data,
                   M.ctypes.data, frame.ctypes.data, d.ctypes.data)
        g[f"das_{label}_params"], g[f"das_{label}_rf"], g[f"das_{label}_out"] = params_blob(bp), rf, frame

    # sum and min/max
    dims = np.array((64, 2, 32), np.int32)
    frames = [rng.standard_normal(2 * int(np.prod(dims))).astype(np.float32) for _ in range(3)]
    ptrs = (ctypes.c_void_p * 3)(*[f.ctypes.data for f in frames])
    s = np.zeros_like(frames[0])
    sh.ref_sum(s.ctypes.data, ptrs, 3, np.float32(1 / 3), dims.ctypes.data)
    nf = O.lib().bfo_min_max_levels_floats(O._arr(dims, ctypes.c_int32))
    mm = np.zeros(nf, np.float32)
    sh.ref_min_max(frames[0].ctypes.data, dims.ctypes.data, O.frame_mips(dims), mm.ctypes.data, nf)
    g["sum_in"], g["sum_out"], g["minmax_out"] = np.stack(frames), s, mm

    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **g)
    print("wrote", os.path.join(HERE, "reference_outputs.npz"))


if __name__ == "__main__":
    main()
