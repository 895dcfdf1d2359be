"""ctypes mirror of include/ogl_beamformer_lib.h.

The product is the C-ABI shared library; this module is the Python-side binding a
caller (tests, bench, a Python client) uses to reach it, the way the reference's
MATLAB and C clients bind helpers/ogl_beamformer_lib_base.h. It loads the
in-tree library and fails loudly if it has not been built.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libogl_beamformer_lib.so")

# BeamformerShaderKind (beamformer_parameters.h:14-41)
SHADER = dict(CudaDecode=0, CudaHilbert=1, DAS=2, Decode=3, Filter=4, Demodulate=5, MinMax=6, Sum=7,
              DecodeInt16Complex=8, DecodeFloat=9, DecodeFloatComplex=10, DecodeInt16ToFloat=11,
              DemodulateFloat=12, DASFast=13, Render3D=14, Count=15)
DATA_KIND = dict(Int16=0, Int16Complex=1, Float32=2, Float32Complex=3)
DAS_KIND = dict(FORCES=0, UFORCES=1, HERCULES=2, RCA_VLS=3, RCA_TPW=4, UHERCULES=5, RACES=6,
                EPIC_FORCES=7, EPIC_UFORCES=8, EPIC_UHERCULES=9, FLASH=10)
ERR = dict(NONE=0, VERSION_MISMATCH=1, INVALID_ACCESS=2, COMPUTE_STAGE_OVERFLOW=3, INVALID_COMPUTE_STAGE=4,
           INVALID_START_SHADER=5, INVALID_DEMOD_DATA_KIND=6, INVALID_IMAGE_PLANE=7, BUFFER_OVERFLOW=8,
           WORK_QUEUE_FULL=9, EXPORT_SPACE_OVERFLOW=10, SHARED_MEMORY=11, SYNC_VARIABLE=12, INVALID_TIMEOUT=13,
           CUDA_DEVICE=14, CUDA_RUNTIME=15, UNSUPPORTED=16)
MAX_COMPUTE_SHADER_STAGES = 16
BEAMFORMER_FILTER_SLOTS = 4

f32, u32, i32 = ctypes.c_float, ctypes.c_uint32, ctypes.c_int32

_HEAD = [("xdc_transform", f32 * 16), ("dec_data_dim", u32 * 4), ("xdc_element_pitch", f32 * 2),
         ("rf_raw_dim", u32 * 2), ("transmit_mode", i32), ("decode", u32), ("das_shader_id", u32),
         ("time_offset", f32)]
_UI = [("output_min_coordinate", f32 * 4), ("output_max_coordinate", f32 * 4), ("output_points", i32 * 4),
       ("sampling_frequency", f32), ("center_frequency", f32), ("speed_of_sound", f32), ("off_axis_pos", f32),
       ("beamform_plane", i32), ("f_number", f32), ("interpolate", u32), ("coherency_weighting", u32)]
_TAIL = [("decimation_rate", u32), ("readi_group_id", u32), ("readi_group_size", u32)]


class BeamformerParameters(ctypes.Structure):
    _fields_ = _HEAD + _UI + _TAIL + [("_pad", f32 * 1)]


class BeamformerUIParameters(ctypes.Structure):
    _fields_ = _UI


class BeamformerParametersHead(ctypes.Structure):
    _fields_ = _HEAD


class BeamformerComputeStatsTable(ctypes.Structure):
    _fields_ = [("times", (f32 * 15) * 32), ("rf_time_deltas", f32 * 32)]


class BeamformerLiveImagingParameters(ctypes.Structure):
    _fields_ = [("active", u32), ("save_enabled", u32), ("save_active", u32), ("transmit_power", f32),
                ("image_plane_offsets", f32 * 4), ("tgc_control_points", f32 * 8)]


assert ctypes.sizeof(BeamformerParameters) == 208
assert BeamformerParameters.output_min_coordinate.offset == 112
assert BeamformerParameters.decimation_rate.offset == 192
assert ctypes.sizeof(BeamformerComputeStatsTable) == 2048

vp = ctypes.c_void_p
P = ctypes.POINTER
# (name, restype, argtypes) for every symbol of include/ogl_beamformer_lib.h
SIGNATURES = [
    ("beamformer_get_api_version", u32, []),
    ("beamformer_get_last_error", i32, []),
    ("beamformer_get_last_error_string", ctypes.c_char_p, []),
    ("beamformer_error_string", ctypes.c_char_p, [i32]),
    ("beamformer_set_global_timeout", u32, [i32]),
    ("beamform_data_synchronized", u32, [vp, u32, P(i32), P(f32), i32]),
    ("beamformer_compute_timings", u32, [P(BeamformerComputeStatsTable), i32]),
    ("beamformer_start_compute", u32, []),
    ("beamformer_wait_for_compute_dispatch", u32, [i32]),
    ("beamformer_push_data_with_compute", u32, [vp, u32, u32]),
    ("beamformer_push_data", u32, [vp, u32]),
    ("beamformer_push_channel_mapping", u32, [P(ctypes.c_int16), u32]),
    ("beamformer_push_sparse_elements", u32, [P(ctypes.c_int16), u32]),
    ("beamformer_push_focal_vectors", u32, [P(f32), u32]),
    ("beamformer_set_pipeline_stage_parameters", u32, [i32, i32]),
    ("beamformer_push_pipeline", u32, [P(i32), i32, i32]),
    ("beamformer_push_parameters", u32, [P(BeamformerParameters)]),
    ("beamformer_push_parameters_ui", u32, [P(BeamformerUIParameters)]),
    ("beamformer_push_parameters_head", u32, [P(BeamformerParametersHead)]),
    ("beamformer_create_kaiser_low_pass_filter", u32, [f32, f32, f32, ctypes.c_int16, ctypes.c_uint8]),
    ("beamformer_create_matched_filter", u32, [f32, f32, f32, ctypes.c_int16, ctypes.c_uint8]),
    ("beamformer_live_parameters_get_dirty_flag", i32, []),
    ("beamformer_set_live_parameters", u32, [P(BeamformerLiveImagingParameters)]),
    ("beamformer_get_live_parameters", P(BeamformerLiveImagingParameters), []),
    # extensions
    ("beamformer_gb300_push_data_device", u32, [vp, ctypes.c_uint64]),
    ("beamformer_gb300_set_stream", u32, [vp]),
    ("beamformer_gb300_get_stream", vp, []),
    ("beamformer_gb300_synchronize", u32, [i32]),
    ("beamformer_gb300_export_frame", u32, [u32, u32, P(f32), ctypes.c_uint64, P(i32)]),
    ("beamformer_gb300_export_channel_data", u32, [vp, ctypes.c_uint64, P(ctypes.c_uint64)]),
    ("beamformer_gb300_get_filter", u32, [ctypes.c_uint8, P(f32), i32, P(i32)]),
    ("beamformer_gb300_set_interpolation", u32, [i32]),
    ("beamformer_gb300_set_filter_precision", u32, [i32]),
    ("beamformer_gb300_set_das_precision", u32, [i32]),
    ("beamformer_gb300_set_receive_subsampling", u32, [i32]),
    ("beamformer_gb300_serve", i32, [i32]),
    ("beamformer_gb300_serve_stop", None, []),
    ("beamformer_gb300_beamform_batch", u32, [P(BeamformerParameters), u32, P(vp), P(ctypes.c_uint64), P(vp), i32]),
    ("beamformer_gb300_batch_tuning", u32, [P(i32), P(i32), P(f32), i32, P(i32)]),
    ("beamformer_gb300_das_no_alloc", u32, [P(BeamformerParameters), P(f32), P(ctypes.c_int16), vp, ctypes.c_uint64,
                                       vp, vp]),
    ("beamformer_gb300_measure_shared_bandwidth", u32, [P(ctypes.c_double)]),
    ("beamformer_gb300_kernel_launch_count", ctypes.c_uint64, []),
    ("beamformer_gb300_shutdown", None, []),
]
REFERENCE_SYMBOLS = [s[0] for s in SIGNATURES if not s[0].startswith("beamformer_gb300_")]

_lib = None


def load(path=None):
    """Load the C-ABI library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
