"""Python client of the C-ABI library, shaped like the reference's callers.

The call sequence follows the reference's own drivers (tests/throughput.c:319-378,
tests/decode.c:226-261): push parameters, filters, channel mapping, focal
vectors and pipeline, then push RF and beamform. Every call goes through
lib/libogl_beamformer_lib.so; failures raise with the library's error string.
"""
import ctypes

import numpy as np

from . import abi


class BeamformerError(RuntimeError):
    pass


class Beamformer:
    def __init__(self):
        self.lib = abi.load()

    def _check(self, ok, what):
        if not ok:
            err = self.lib.beamformer_get_last_error()
            msg = self.lib.beamformer_get_last_error_string().decode()
            raise BeamformerError(f"{what}: {msg} (error {err})")
        return ok

    # ---- configuration ----
    def configure(self, bp, pipeline, data_kind=abi.DATA_KIND["Int16"], kaiser=None, matched=None,
                  channel_mapping=None, focal_vectors=None, sparse_elements=None, stage_slots=None,
                  interpolation=-1):
        L = self.lib
        self.bp = bp
        if kaiser is not None:
            beta, cutoff, fs, length = kaiser
            self._check(L.beamformer_create_kaiser_low_pass_filter(beta, cutoff, fs, length, 0), "kaiser filter")
        if matched is not None:
            fxdc, ftx, fs, length, slot = matched
            self._check(L.beamformer_create_matched_filter(fxdc, ftx, fs, length, slot), "matched filter")
        cm = np.arange(256, dtype=np.int16) if channel_mapping is None else np.asarray(channel_mapping, np.int16)
        self._check(L.beamformer_push_channel_mapping(cm.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), len(cm)),
                    "channel mapping")
        fv = np.zeros(512, np.float32) if focal_vectors is None else np.asarray(focal_vectors, np.float32)
        if focal_vectors is None:
            fv[1::2] = np.inf
        self._check(L.beamformer_push_focal_vectors(fv.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(fv) // 2),
                    "focal vectors")
        se = np.arange(256, dtype=np.int16) if sparse_elements is None else np.asarray(sparse_elements, np.int16)
        self._check(L.beamformer_push_sparse_elements(se.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), len(se)),
                    "sparse elements")
        self.focal = fv
        self.sparse = se
        self.chmap = cm
        self._check(L.beamformer_push_parameters(ctypes.byref(bp)), "parameters")
        sh = (ctypes.c_int32 * len(pipeline))(*pipeline)
        self._check(L.beamformer_push_pipeline(sh, len(pipeline), data_kind), "pipeline")
        # every pipeline position gets its filter slot (0 unless given), so no
        # slot of an earlier configuration carries over
        slots = stage_slots or {}
        for stage in range(16):
            L.beamformer_set_pipeline_stage_parameters(stage, slots.get(stage, 0))
        self._check(L.beamformer_gb300_set_interpolation(interpolation), "interpolation")
        return self

    def set_precision(self, filter=None, das=None):
        """Arithmetic of the front end (0 FP32, 1 FP16, 2 BF16 Decode output with the
        tensor-core FIR) and of HERCULES DAS (0 FP32, 1 FP16 interpolation table);
        None leaves that one as it is. Both persist in the library until changed."""
        if filter is not None:
            self._check(self.lib.beamformer_gb300_set_filter_precision(int(filter)), "filter precision")
        if das is not None:
            self._check(self.lib.beamformer_gb300_set_das_precision(int(das)), "DAS precision")
        return self

    # ---- compute ----
    def beamform(self, raw, timeout_ms=-1):
        """beamform_data_synchronized: push host RF, compute, return the output volume."""
        pts = (ctypes.c_int32 * 3)(*[int(v) for v in self.bp.output_points[:3]])
        n = max(1, pts[0]) * max(1, pts[1]) * max(1, pts[2])
        out = np.empty(2 * n, np.float32)
        raw = np.ascontiguousarray(raw)
        self._check(self.lib.beamform_data_synchronized(raw.ctypes.data_as(ctypes.c_void_p), raw.nbytes, pts,
                                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                        timeout_ms), "beamform_data_synchronized")
        return out

    def push(self, raw, compute=True):
        raw = np.ascontiguousarray(raw)
        if compute:
            return self._check(self.lib.beamformer_push_data_with_compute(raw.ctypes.data_as(ctypes.c_void_p),
                                                                          raw.nbytes, 0), "push_data_with_compute")
        return self._check(self.lib.beamformer_push_data(raw.ctypes.data_as(ctypes.c_void_p), raw.nbytes), "push_data")

    def push_device(self, ptr, nbytes, compute=True):
        self._check(self.lib.beamformer_gb300_push_data_device(ctypes.c_void_p(ptr), nbytes), "push_data_device")
        if compute:
            self._check(self.lib.beamformer_start_compute(), "start_compute")

    def synchronize(self, timeout_ms=-1):
        return self._check(self.lib.beamformer_gb300_synchronize(timeout_ms), "synchronize")

    def frame(self, which=0, level=0):
        dims = (ctypes.c_int32 * 3)()
        self._check(self.lib.beamformer_gb300_export_frame(which, level, None, 0, dims), "export_frame dims")
        out = np.empty(2 * dims[0] * dims[1] * dims[2], np.float32)
        self._check(self.lib.beamformer_gb300_export_frame(which, level, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                           out.nbytes, dims), "export_frame")
        return out, tuple(dims)

    def channel_data(self):
        n = ctypes.c_uint64()
        self._check(self.lib.beamformer_gb300_export_channel_data(None, 0, ctypes.byref(n)), "channel data size")
        out = np.empty(n.value // 4, np.float32)
        self._check(self.lib.beamformer_gb300_export_channel_data(out.ctypes.data_as(ctypes.c_void_p), n.value, None),
                    "channel data")
        return out

    def timings(self):
        t = abi.BeamformerComputeStatsTable()
        self._check(self.lib.beamformer_compute_timings(ctypes.byref(t), -1), "compute_timings")
        return np.ctypeslib.as_array(t.times).copy(), np.ctypeslib.as_array(t.rf_time_deltas).copy()

    def launches(self):
        return int(self.lib.beamformer_gb300_kernel_launch_count())

    def beamform_batch(self, params, rf_ptrs, rf_sizes, out_ptrs, timeout_ms=-1):
        """beamformer_gb300_beamform_batch over device buffers (integer addresses)."""
        n = len(params)
        arr = (abi.BeamformerParameters * n)(*params)
        rf = (ctypes.c_void_p * n)(*rf_ptrs)
        sz = (ctypes.c_uint64 * n)(*rf_sizes)
        out = (ctypes.c_void_p * n)(*out_ptrs)
        self._check(self.lib.beamformer_gb300_beamform_batch(arr, n, rf, sz, out, timeout_ms), "beamform_batch")

    def batch_tuning(self):
        """(volume tiles, persistent CTAs, candidate milliseconds) of the current batch."""
        vt, ctas, cnt = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.beamformer_gb300_batch_tuning(ctypes.byref(vt), ctypes.byref(ctas), None, 0,
                                                           ctypes.byref(cnt)), "batch_tuning")
        ms = np.zeros(max(cnt.value, 1), np.float32)
        self._check(self.lib.beamformer_gb300_batch_tuning(None, None, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                           len(ms), ctypes.byref(cnt)), "batch_tuning")
        return bool(vt.value), int(ctas.value), ms[:cnt.value]
