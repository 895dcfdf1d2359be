"""Python binding and pipeline glue for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
as the checker. The glue in `OraclePipeline` follows the reference's compute
orchestration (beamformer.c:842-1111 `complete_queue`, :521-709
`do_compute_shader`): plan, run each planned stage on ping-pong channel buffers,
keep a ring of MAX_BEAMFORMED_SAVED_FRAMES frames for the Sum stage.
"""
import ctypes
import os
import subprocess

import numpy as np

from ogl_beamforming_cuda_gb300.abi import BeamformerParameters, SHADER, DATA_KIND

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbf_oracle.so")
REF = os.path.join(HERE, "_ref")

u32, i32, f32 = ctypes.c_uint32, ctypes.c_int32, ctypes.c_float


class DecodeUBO(ctypes.Structure):
    _fields_ = [(n, u32) for n in ("input_channel_stride", "input_sample_stride", "input_transmit_stride",
                                   "output_channel_stride", "output_sample_stride", "output_transmit_stride",
                                   "transmit_count", "decode_mode")]


class FilterUBO(ctypes.Structure):
    _fields_ = [(n, u32) for n in ("input_channel_stride", "input_sample_stride", "input_transmit_stride",
                                   "output_channel_stride", "output_sample_stride", "output_transmit_stride",
                                   "decimation_rate", "map_channels")] + \
               [("demodulation_frequency", f32), ("sampling_frequency", f32)]


class FilterSpec(ctypes.Structure):
    _fields_ = [("kind", i32), ("length", i32), ("sampling_frequency", f32), ("param0", f32), ("param1", f32)]


class Plan(ctypes.Structure):
    _fields_ = [("shaders", i32 * 16), ("filter_slots", ctypes.c_uint8 * 16), ("shader_count", i32),
                ("decode_dispatch", u32 * 3), ("demod_dispatch", u32 * 3), ("rf_size", u32),
                ("decode", DecodeUBO), ("demod", FilterUBO), ("filter", FilterUBO), ("das", BeamformerParameters)]


SHM_CLIENT = os.path.join(BUILD, "libshm_client.so")


def build_shm_client(force=False):
    """oracle/shm_client.c: the restated client side of the shared-memory protocol."""
    src = os.path.join(HERE, "shm_client.c")
    if not force and os.path.exists(SHM_CLIENT) and os.path.getmtime(SHM_CLIENT) >= os.path.getmtime(src):
        return SHM_CLIENT
    os.makedirs(BUILD, exist_ok=True)
    subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-Wall", src, "-o", SHM_CLIENT + ".tmp", "-lrt"])
    os.replace(SHM_CLIENT + ".tmp", SHM_CLIENT)
    return SHM_CLIENT


def build(force=False):
    build_shm_client(force)
    src = [os.path.join(HERE, "bf_oracle.c")]
    deps = src + [os.path.join(HERE, "bf_oracle_das.inc"), os.path.join(HERE, "bf_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unknown-pragmas"] + src + ["-o", LIB + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, P = ctypes.c_void_p, ctypes.POINTER
        sig = {
            "bfo_i0": (ctypes.c_double, [ctypes.c_double]),
            "bfo_hadamard_transpose": (i32, [i32, P(i32)]),
            "bfo_kaiser_low_pass": (None, [f32, f32, f32, i32, P(f32)]),
            "bfo_kaiser_low_pass_f64": (None, [ctypes.c_double] * 3 + [i32, P(ctypes.c_double)]),
            "bfo_matched_filter": (None, [f32, f32, f32, i32, P(f32)]),
            "bfo_voxel_transform": (None, [P(BeamformerParameters), P(f32)]),
            "bfo_frame_mips": (i32, [P(i32)]),
            "bfo_plan": (None, [P(BeamformerParameters), P(i32), P(ctypes.c_uint8), i32, i32, P(FilterSpec), P(Plan)]),
            "bfo_decode": (None, [P(DecodeUBO), i32, i32, i32, vp, ctypes.c_uint64, vp, ctypes.c_uint64, P(i32), i32,
                                  P(ctypes.c_int16), P(u32), i32]),
            "bfo_filter": (None, [P(FilterUBO), i32, vp, ctypes.c_uint64, vp, ctypes.c_uint64, P(f32), i32,
                                  P(ctypes.c_int16), P(u32), i32]),
            "bfo_filter_f64": (None, [P(FilterUBO), i32, vp, ctypes.c_uint64, vp, ctypes.c_uint64,
                                      P(ctypes.c_double), i32, P(u32), i32]),
            "bfo_das": (None, [P(BeamformerParameters), i32, vp, ctypes.c_uint64, P(ctypes.c_int16), P(f32), P(f32),
                               vp, P(i32), ctypes.c_int64, ctypes.c_int64, i32, i32]),
            "bfo_das_f64": (None, [P(BeamformerParameters), i32, vp, ctypes.c_uint64, P(ctypes.c_int16), P(f32),
                                   P(ctypes.c_double), vp, P(i32), ctypes.c_int64, ctypes.c_int64, i32, i32]),
            "bfo_sum": (None, [vp, P(vp), i32, f32, P(i32), i32]),
            "bfo_min_max": (None, [vp, P(i32), vp, i32]),
            "bfo_min_max_levels_floats": (ctypes.c_uint64, [P(i32)]),
            "bfo_das_active_terms": (ctypes.c_uint64, [P(BeamformerParameters), P(ctypes.c_int16), P(f32), P(f32),
                                                       P(i32), ctypes.c_int64, ctypes.c_int64, i32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def threads():
    return int(os.environ.get("BF_ORACLE_THREADS", str(os.cpu_count() or 1)))


def _ptr(a, t=ctypes.c_void_p):
    return ctypes.cast(a.ctypes.data, t) if t is not ctypes.c_void_p else ctypes.c_void_p(a.ctypes.data)


def _arr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def hadamard(n):
    out = np.zeros(n * n, np.int32)
    ok = lib().bfo_hadamard_transpose(n, _arr(out, i32))
    return out.reshape(n, n) if ok else None


def kaiser(cutoff, fs, beta, length):
    out = np.zeros(length, np.float32)
    lib().bfo_kaiser_low_pass(cutoff, fs, beta, length, _arr(out, f32))
    return out


def kaiser_f64(cutoff, fs, beta, length):
    out = np.zeros(length, np.float64)
    lib().bfo_kaiser_low_pass_f64(cutoff, fs, beta, length, _arr(out, ctypes.c_double))
    return out


def matched(fxdc, ftx, fs, length):
    out = np.zeros(length, np.float32)
    lib().bfo_matched_filter(fxdc, ftx, fs, length, _arr(out, f32))
    return out


def voxel_transform(bp):
    out = np.zeros(16, np.float32)
    lib().bfo_voxel_transform(ctypes.byref(bp), _arr(out, f32))
    return out


def frame_mips(dims):
    d = np.asarray(dims, np.int32)
    return lib().bfo_frame_mips(_arr(d, i32))


def das_active_terms(bp, dims, sparse, focal, voxel_begin=0, voxel_end=None):
    M = voxel_transform(bp)
    d = np.asarray(dims, np.int32)
    ve = int(np.prod(dims)) if voxel_end is None else voxel_end
    return lib().bfo_das_active_terms(ctypes.byref(bp), _arr(sparse, ctypes.c_int16), _arr(focal, f32),
                                      _arr(M, f32), _arr(d, i32), voxel_begin, ve, threads())


def das(bp, rf, dims, sparse, focal, fast=True, voxel_begin=0, voxel_end=None, interpolation=-1, out=None, f64=False):
    """Delay-and-sum of float2 channel data rf (float32 or float64) into a frame."""
    d = np.asarray(dims, np.int32)
    n = int(np.prod(dims))
    ve = n if voxel_end is None else voxel_end
    if f64:
        M = voxel_transform(bp).astype(np.float64)
        frame = np.zeros(2 * n, np.float64) if out is None else out
        rf = np.ascontiguousarray(rf, np.float64)
        lib().bfo_das_f64(ctypes.byref(bp), int(fast), _ptr(rf), rf.size, _arr(sparse, ctypes.c_int16),
                          _arr(focal, f32), _arr(M, ctypes.c_double), _ptr(frame), _arr(d, i32), voxel_begin, ve,
                          interpolation, threads())
    else:
        M = voxel_transform(bp)
        frame = np.zeros(2 * n, np.float32) if out is None else out
        rf = np.ascontiguousarray(rf, np.float32)
        lib().bfo_das(ctypes.byref(bp), int(fast), _ptr(rf), rf.size, _arr(sparse, ctypes.c_int16), _arr(focal, f32),
                      _arr(M, f32), _ptr(frame), _arr(d, i32), voxel_begin, ve, interpolation, threads())
    return frame


def sum_frames(frames, prescale, dims):
    d = np.asarray(dims, np.int32)
    out = np.zeros(2 * int(np.prod(dims)), np.float32)
    ptrs = (ctypes.c_void_p * len(frames))(*[f.ctypes.data for f in frames])
    lib().bfo_sum(_ptr(out), ptrs, len(frames), prescale, _arr(d, i32), threads())
    return out


def min_max(frame, dims):
    d = np.asarray(dims, np.int32)
    n = lib().bfo_min_max_levels_floats(_arr(d, i32))
    out = np.zeros(n, np.float32)
    lib().bfo_min_max(_ptr(frame), _arr(d, i32), _ptr(out), threads())
    return out


def analytic_signal(x):
    """Discrete analytic signal of real rows x[..., N] (float64 result): the
    CudaHilbert stage (BeamformerShaderKind_CudaHilbert, beamformer.c:567-570;
    the reference runs it in its external cuda_toolkit plugin, whose source it
    does not ship, so this restates the published definition -- Marple, IEEE
    Trans. Signal Processing 47(9), 1999: one-sided FFT spectrum, Z[0] and Z[N/2]
    kept, Z[1 .. N/2-1] doubled, the rest zeroed, inverse FFT). Parity for this
    stage is unpinned by the reference."""
    x = np.asarray(x, np.float64)
    n = x.shape[-1]
    h = np.zeros(n)
    h[0] = 1.0
    if n % 2 == 0:
        h[n // 2] = 1.0
        h[1:n // 2] = 2.0
    else:
        h[1:(n + 1) // 2] = 2.0
    return np.fft.ifft(np.fft.fft(x, axis=-1) * h, axis=-1)


def plan(bp, shaders, slots, data_kind, filter_specs):
    sh = np.zeros(16, np.int32)
    sh[:len(shaders)] = shaders
    sl = np.zeros(16, np.uint8)
    sl[:len(slots)] = slots
    specs = (FilterSpec * 4)()
    for i, s in enumerate(filter_specs):
        if s is not None:
            specs[i] = FilterSpec(*s)
    p = Plan()
    lib().bfo_plan(ctypes.byref(bp), _arr(sh, i32), _arr(sl, ctypes.c_uint8), len(shaders), data_kind, specs,
                   ctypes.byref(p))
    return p


class OraclePipeline:
    """State machine mirroring the library context: parameters, pipeline, filters,
    channel mapping / sparse elements / focal vectors, and the frame ring."""

    def __init__(self):
        self.bp = BeamformerParameters()
        self.shaders = []
        self.slots = [0] * 16
        self.data_kind = DATA_KIND["Int16"]
        self.filters = [None] * 4          # (kind, length, fs, p0, p1)
        self.taps = [None] * 4
        self.chmap = np.arange(256, dtype=np.int16)
        self.sparse = np.arange(256, dtype=np.int16)
        self.focal = np.zeros(512, np.float32)
        self.frames = [None] * 16
        self.frame_index = 0
        self.interpolation = -1

    def create_kaiser(self, beta, cutoff, fs, length, slot):
        s = slot % 4
        self.filters[s] = (0, length, fs, beta, cutoff)
        self.taps[s] = kaiser(cutoff, fs, beta, length)

    def create_matched(self, fxdc, ftx, fs, length, slot):
        s = slot % 4
        self.filters[s] = (1, length, fs, fxdc, ftx)
        self.taps[s] = matched(fxdc, ftx, fs, length)

    def compute(self, raw, want_stages=False):
        """Run the planned pipeline on raw RF (numpy array of the data kind)."""
        L = lib()
        p = plan(self.bp, self.shaders, self.slots[:len(self.shaders)], self.data_kind, self.filters)
        dims = [max(1, int(x)) for x in self.bp.output_points[:3]]
        dd = p.das.dec_data_dim
        chan_bytes = 8 * int(self.bp.dec_data_dim[0]) * int(self.bp.dec_data_dim[1]) * int(self.bp.dec_data_dim[2])
        bufs = [np.zeros(chan_bytes // 4, np.float32), np.zeros(chan_bytes // 4, np.float32)]
        last = 0
        raw = np.ascontiguousarray(raw)
        stages = {}
        frame = np.zeros(2 * int(np.prod(dims)), np.float32)
        averaged = None
        mips = None
        nt = threads()
        for i in range(p.shader_count):
            kind = p.shaders[i]
            out_idx, in_idx = 1 - last, last
            if kind in (SHADER["Decode"], SHADER["DecodeInt16Complex"], SHADER["DecodeFloat"],
                        SHADER["DecodeFloatComplex"], SHADER["DecodeInt16ToFloat"], SHADER["CudaDecode"]):
                first = i == 0
                src = raw if first else bufs[in_idx]
                H = hadamard(int(p.decode.transmit_count))
                Hp = _arr(H.ravel().astype(np.int32), i32) if H is not None else None
                Harr = H.ravel().astype(np.int32) if H is not None else np.zeros(1, np.int32)
                bufs[out_idx][:] = 0
                L.bfo_decode(ctypes.byref(p.decode), kind, int(first), self.data_kind, _ptr(src), src.nbytes,
                             _ptr(bufs[out_idx]), bufs[out_idx].nbytes, _arr(Harr, i32), int(p.decode.transmit_count),
                             _arr(self.chmap, ctypes.c_int16), p.decode_dispatch, nt)
                last = out_idx
            elif kind in (SHADER["Demodulate"], SHADER["DemodulateFloat"], SHADER["Filter"]):
                ubo = p.filter if kind == SHADER["Filter"] else p.demod
                src = raw if (kind != SHADER["Filter"] and ubo.map_channels) else bufs[in_idx]
                taps = self.taps[p.filter_slots[i] % 4]
                bufs[out_idx][:] = 0
                L.bfo_filter(ctypes.byref(ubo), kind, _ptr(src), src.nbytes, _ptr(bufs[out_idx]), bufs[out_idx].nbytes,
                             _arr(taps, f32), len(taps), _arr(self.chmap, ctypes.c_int16), p.demod_dispatch, nt)
                last = out_idx
            elif kind == SHADER["CudaHilbert"]:
                # rows of S complex samples in the DAS layout [channel][transmit][sample]
                S, rows = int(dd[0]), int(dd[1]) * int(dd[2])
                src = bufs[in_idx][: 2 * S * rows].reshape(rows, S, 2)
                z = analytic_signal(src[:, :, 0])
                bufs[out_idx][:] = 0
                out = bufs[out_idx][: 2 * S * rows].reshape(rows, S, 2)
                out[:, :, 0] = z.real
                out[:, :, 1] = z.imag
                last = out_idx
            elif kind in (SHADER["DAS"], SHADER["DASFast"]):
                rf = bufs[in_idx][: p.rf_size // 4]
                das(p.das, rf, dims, self.sparse, self.focal, fast=(kind == SHADER["DASFast"]),
                    interpolation=self.interpolation, out=frame)
            elif kind == SHADER["Sum"]:
                n = int(p.das.output_points[3])
                ring = []
                base = self.frame_index % 16
                for k in range(n):
                    idx = (base + 1 - n + k) % 16
                    f = frame if idx == base else self.frames[idx]
                    if f is None or f.size != frame.size:
                        f = np.zeros_like(frame)
                    ring.append(f)
                averaged = sum_frames(ring, np.float32(1.0) / np.float32(n), dims)
            elif kind == SHADER["MinMax"]:
                mips = min_max(frame, dims)
            if want_stages:
                stages[i] = (kind, bufs[last].copy())
        self.frames[self.frame_index % 16] = frame
        self.frame_index += 1
        return dict(plan=p, frame=frame, averaged=averaged, mips=mips, channel_data=bufs[last], dims=dims,
                    stages=stages)


def ref_available():
    return all(os.path.exists(os.path.join(REF, f)) for f in ("libref_shaders.so", "libref_math.so"))


def ref_libs():
    """(shaders, math, client) ctypes handles of oracle/_ref, or None."""
    if not ref_available():
        return None
    return (ctypes.CDLL(os.path.join(REF, "libref_shaders.so")), ctypes.CDLL(os.path.join(REF, "libref_math.so")),
            ctypes.CDLL(os.path.join(REF, "libref_client.so")))
