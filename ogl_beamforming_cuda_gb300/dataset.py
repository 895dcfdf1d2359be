"""Captured-dataset format of the reference (tests/throughput.c:31-51, 171-213):
a study directory `<base>/<study>/` holding

  <study>.bp      one zemp_bp_v1 parameter block (3728 bytes, magic 0x5042504D455AFECA,
                  version 1)
  <study>_NN.zst  raw RF frames, int16 [channel][transmit][sample], each a zstd frame

plus the reference's mapping of the parameter block onto BeamformerParameters
(fill_beamformer_parameters_from_zemp_bp_v1, tests/throughput.c:196-211) and
its throughput driver (execute_study, tests/throughput.c:301-404: one frame
pushed repeatedly through the library, frame time and RF GB/s reported).
Command line: python -m ogl_beamforming_cuda_gb300.dataset <base> <study>.

zstd is the system library (libzstd.so.1), loaded at first use; reading or
writing a frame fails with RuntimeError where it is absent.
"""
import argparse
import ctypes
import ctypes.util
import json
import os
import time

import numpy as np

from . import abi

ZEMP_BP_MAGIC = 0x5042504D455AFECA


class ZempBpV1(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_uint64), ("version", ctypes.c_uint32), ("decode_mode", ctypes.c_uint16),
                ("beamform_mode", ctypes.c_uint16), ("raw_data_dim", ctypes.c_uint32 * 4),
                ("decoded_data_dim", ctypes.c_uint32 * 4), ("xdc_element_pitch", ctypes.c_float * 2),
                ("xdc_transform", ctypes.c_float * 16), ("channel_mapping", ctypes.c_int16 * 256),
                ("transmit_angles", ctypes.c_float * 256), ("focal_depths", ctypes.c_float * 256),
                ("sparse_elements", ctypes.c_int16 * 256), ("hadamard_rows", ctypes.c_int16 * 256),
                ("speed_of_sound", ctypes.c_float), ("center_frequency", ctypes.c_float),
                ("sampling_frequency", ctypes.c_float), ("time_offset", ctypes.c_float),
                ("transmit_mode", ctypes.c_int32)]


assert ctypes.sizeof(ZempBpV1) == 3728

_zstd = None


def _zstd_lib():
    global _zstd
    if _zstd is None:
        name = ctypes.util.find_library("zstd") or "libzstd.so.1"
        try:
            z = ctypes.CDLL(name)
        except OSError as e:
            raise RuntimeError(f"zstd library not available: {e}") from e
        sz = ctypes.c_size_t
        z.ZSTD_getFrameContentSize.argtypes = [ctypes.c_void_p, sz]
        z.ZSTD_getFrameContentSize.restype = ctypes.c_ulonglong
        z.ZSTD_decompress.argtypes = [ctypes.c_void_p, sz, ctypes.c_void_p, sz]
        z.ZSTD_decompress.restype = sz
        z.ZSTD_compress.argtypes = [ctypes.c_void_p, sz, ctypes.c_void_p, sz, ctypes.c_int]
        z.ZSTD_compress.restype = sz
        z.ZSTD_compressBound.argtypes = [sz]
        z.ZSTD_compressBound.restype = sz
        z.ZSTD_isError.argtypes = [sz]
        z.ZSTD_isError.restype = ctypes.c_uint
        _zstd = z
    return _zstd


def decompress(data):
    """bytes of one zstd frame (its content size must be recorded, as the
    reference's reader requires) -> bytes"""
    z = _zstd_lib()
    src = ctypes.create_string_buffer(bytes(data), len(data))
    n = z.ZSTD_getFrameContentSize(src, len(data))
    if n >= (1 << 63):                          # ZSTD_CONTENTSIZE_UNKNOWN / _ERROR
        raise RuntimeError("zstd frame without a content size")
    dst = ctypes.create_string_buffer(int(n))
    got = z.ZSTD_decompress(dst, n, src, len(data))
    if z.ZSTD_isError(got) or got != n:
        raise RuntimeError("zstd decompression failed")
    return dst.raw


def compress(data, level=3):
    z = _zstd_lib()
    src = bytes(data)
    cap = z.ZSTD_compressBound(len(src))
    dst = ctypes.create_string_buffer(cap)
    n = z.ZSTD_compress(dst, cap, src, len(src), level)
    if z.ZSTD_isError(n):
        raise RuntimeError("zstd compression failed")
    return dst.raw[:n]


def read_parameters(path):
    """The zemp_bp_v1 block of a .bp file (read_zemp_bp_v1: exact size, magic,
    version 1), or ValueError."""
    raw = open(path, "rb").read()
    if len(raw) != ctypes.sizeof(ZempBpV1):
        raise ValueError(f"{path}: {len(raw)} bytes, expected {ctypes.sizeof(ZempBpV1)}")
    zbp = ZempBpV1.from_buffer_copy(raw)
    if zbp.magic != ZEMP_BP_MAGIC or zbp.version != 1:
        raise ValueError(f"{path}: not a zemp_bp_v1 parameter block")
    return zbp


def to_beamformer_parameters(zbp, bp=None):
    """fill_beamformer_parameters_from_zemp_bp_v1: the acquisition fields; the
    output grid, interpolation and filter settings stay as given in bp."""
    bp = bp if bp is not None else abi.BeamformerParameters()
    bp.xdc_transform[:] = zbp.xdc_transform[:]
    bp.dec_data_dim[:] = zbp.decoded_data_dim[:]
    bp.xdc_element_pitch[:] = zbp.xdc_element_pitch[:]
    bp.rf_raw_dim[:] = zbp.raw_data_dim[:2]
    bp.transmit_mode = zbp.transmit_mode
    bp.decode = zbp.decode_mode
    bp.das_shader_id = zbp.beamform_mode
    bp.time_offset = zbp.time_offset
    bp.sampling_frequency = zbp.sampling_frequency
    bp.center_frequency = zbp.center_frequency
    bp.speed_of_sound = zbp.speed_of_sound
    return bp


def focal_vectors(zbp):
    """(angle, depth) pairs as pushed by the throughput driver (tests/throughput.c:360-368)."""
    v = np.zeros(512, np.float32)
    v[0::2] = np.asarray(zbp.transmit_angles[:], np.float32)
    v[1::2] = np.asarray(zbp.focal_depths[:], np.float32)
    return v


class Study:
    """One study directory: parameters and frames."""

    def __init__(self, base, study):
        self.dir = os.path.join(base, study)
        self.name = study
        self.zbp = read_parameters(os.path.join(self.dir, study + ".bp"))

    def frame_path(self, index):
        return os.path.join(self.dir, f"{self.name}_{index:02d}.zst")

    def frame_count(self):
        n = 0
        while os.path.exists(self.frame_path(n)):
            n += 1
        return n

    def frame(self, index):
        """int16 raw RF of frame `index` (rf_raw_dim[0] x rf_raw_dim[1] samples)"""
        data = decompress(open(self.frame_path(index), "rb").read())
        return np.frombuffer(data, np.int16).copy()


def write_study(base, study, bp, frames, channel_mapping=None, focal=None, sparse=None, level=3):
    """Write a study in the reference's layout (parameters from bp, frames as
    int16 arrays): the writer behind the tests and for converting other data."""
    d = os.path.join(base, study)
    os.makedirs(d, exist_ok=True)
    z = ZempBpV1()
    z.magic = ZEMP_BP_MAGIC
    z.version = 1
    z.decode_mode = bp.decode
    z.beamform_mode = bp.das_shader_id
    z.raw_data_dim[:] = [bp.rf_raw_dim[0], bp.rf_raw_dim[1], 0, 0]
    z.decoded_data_dim[:] = bp.dec_data_dim[:]
    z.xdc_element_pitch[:] = bp.xdc_element_pitch[:]
    z.xdc_transform[:] = bp.xdc_transform[:]
    z.channel_mapping[:] = (np.arange(256, dtype=np.int16) if channel_mapping is None
                            else np.asarray(channel_mapping, np.int16)).tolist()
    fv = np.zeros(512, np.float32) if focal is None else np.asarray(focal, np.float32)
    z.transmit_angles[:] = fv[0::2].tolist()
    z.focal_depths[:] = fv[1::2].tolist()
    z.sparse_elements[:] = (np.zeros(256, np.int16) if sparse is None else np.asarray(sparse, np.int16)).tolist()
    z.speed_of_sound = bp.speed_of_sound
    z.center_frequency = bp.center_frequency
    z.sampling_frequency = bp.sampling_frequency
    z.time_offset = bp.time_offset
    z.transmit_mode = bp.transmit_mode
    with open(os.path.join(d, study + ".bp"), "wb") as f:
        f.write(bytes(z))
    for i, fr in enumerate(frames):
        with open(os.path.join(d, f"{study}_{i:02d}.zst"), "wb") as f:
            f.write(compress(np.ascontiguousarray(fr, np.int16).tobytes(), level))
    return d


def driver_setup(zbp, output_points=(512, 1, 1024), lateral=(-60e-3, 60e-3), axial=(10e-3, 165e-3), f_number=0.5):
    """The library configuration of the reference's throughput driver for a
    study (execute_study, tests/throughput.c:301-378): acquisition parameters
    from the block, an output plane of output_points over the lateral x axial
    extent, the pipeline Demodulate -> Decode -> Filter -> DAS on int16 data with
    a Kaiser low-pass (beta 5.65, 1.2 MHz, 36 taps) on the Demodulate stage and a
    matched filter on the Filter stage, demodulation at fs / 4 without
    decimation, sparse elements 0..255 where the block's first entry is -1.
    Returns keyword arguments for client.Beamformer.configure plus "bp" and
    "pipeline"."""
    bp = to_beamformer_parameters(zbp)
    bp.output_points[:] = [output_points[0], output_points[1], output_points[2], 1]
    bp.output_min_coordinate[:] = [lateral[0], 0, axial[0], 0]
    bp.output_max_coordinate[:] = [lateral[1], 0, axial[1], 0]
    bp.f_number = f_number
    bp.beamform_plane = 0
    bp.interpolate = 0
    f32 = np.float32
    xdc_frequency = f32(bp.center_frequency)
    fs = f32(bp.sampling_frequency)
    bp.decimation_rate = 1
    bp.center_frequency = float(fs / f32(4))
    fc = f32(bp.center_frequency)
    matched_fs = f32(4) * fs / f32(2) / f32(bp.decimation_rate)
    matched_len = int(np.ceil(f32(4) * f32(2) * fs / f32(2) / fc))
    sparse = np.asarray(zbp.sparse_elements[:], np.int16)
    if sparse[0] == -1:
        sparse = np.arange(256, dtype=np.int16)
    SH = abi.SHADER
    return {"bp": bp, "pipeline": [SH["Demodulate"], SH["Decode"], SH["Filter"], SH["DAS"]],
            "kaiser": (5.65, 1.2e6, float(fs / f32(2)), 36),
            "matched": (float(xdc_frequency), float(fc), float(matched_fs), matched_len, 1),
            "stage_slots": {0: 0, 2: 1},
            "channel_mapping": np.asarray(zbp.channel_mapping[:], np.int16),
            "focal_vectors": focal_vectors(zbp), "sparse_elements": sparse}


def throughput(base, study, frame=0, loops=16, das_precision=0, **extent):
    """Frame time and RF throughput of one study frame pushed `loops` times
    through the library with the reference driver's configuration (its looping
    mode, tests/throughput.c:384-404); das_precision 1 beamforms HERCULES
    studies from the FP16 interpolation table."""
    from .client import Beamformer
    st = Study(base, study)
    cfg = driver_setup(st.zbp, **extent)
    bp, pipeline = cfg.pop("bp"), cfg.pop("pipeline")
    bf = Beamformer().configure(bp, pipeline, **cfg).set_precision(das=das_precision)
    data = st.frame(frame)
    size = int(bp.rf_raw_dim[0]) * int(bp.rf_raw_dim[1]) * 2
    if data.nbytes < size:
        raise ValueError(f"frame {frame} holds {data.nbytes} bytes, parameters need {size}")
    data = data[:size // 2]
    bf.push(data)
    bf.synchronize()
    t0 = time.perf_counter()
    for _ in range(loops):
        bf.push(data)
    bf.synchronize()
    dt = (time.perf_counter() - t0) / loops
    bf.set_precision(das=0)
    return {"study": study, "frame": frame, "frames": loops, "ms_per_frame": dt * 1e3,
            "rf_gb_per_s": size / dt / 1e9, "output_points": [int(v) for v in bp.output_points[:3]],
            "das_precision": das_precision}


def main():
    ap = argparse.ArgumentParser(description="beamform a captured study (reference dataset layout)")
    ap.add_argument("base")
    ap.add_argument("study")
    ap.add_argument("--frame", type=int, default=0)
    ap.add_argument("--loops", type=int, default=16)
    ap.add_argument("--das-precision", type=int, default=0, choices=[0, 1],
                    help="1: HERCULES DAS from the FP16 interpolation table")
    a = ap.parse_args()
    print(json.dumps(throughput(a.base, a.study, frame=a.frame, loops=a.loops, das_precision=a.das_precision)))


if __name__ == "__main__":
    main()
