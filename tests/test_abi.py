"""C-ABI tests that need no GPU: exports, struct layout, validation and error
behaviour, compared with the reference client library (oracle/_ref) where built."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "ogl_beamformer_lib.h")
REF_CLIENT = os.path.join(ROOT, "oracle", "_ref", "libref_client.so")
REF_LAYOUT = os.path.join(ROOT, "oracle", "_ref", "parameters_layout.txt")


def header_symbols():
    text = "\n".join(ln for ln in open(HEADER).read().splitlines() if not ln.lstrip().startswith("#"))
    return sorted(set(re.findall(r"LIB_FN[^;(]*?\**\s*(\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = header_symbols()
    assert len(names) >= 24 + 10
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(names) <= exported
    assert set(abi.REFERENCE_SYMBOLS) <= exported and len(abi.REFERENCE_SYMBOLS) == 24


def test_library_exports_every_unet_symbol(lib):
    """include/bf_unet.h (the learned variant's kernels): every declared function is exported."""
    text = open(os.path.join(ROOT, "include", "bf_unet.h")).read()
    names = sorted(set(re.findall(r"^uint32_t\s+(\w+)\s*\(", text, re.M)))
    assert {"bf_unet_conv3d", "bf_unet_conv3d_grad_input", "bf_unet_ema", "bf_unet_tc_errors"} <= set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(names) <= exported, sorted(set(names) - exported)


@pytest.mark.skipif(not os.path.exists(REF_CLIENT), reason="reference client library not built")
def test_reference_exports_are_a_subset():
    out = subprocess.run(["nm", "-D", "--defined-only", REF_CLIENT], capture_output=True, text=True).stdout
    ref = {line.split()[-1] for line in out.splitlines() if " T " in line and "beamform" in line}
    assert ref == set(abi.REFERENCE_SYMBOLS)


LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include <stdint.h>
#include HDR
#define O(f) printf(#f " %zu\n", offsetof(BeamformerParameters, f));
int main(void) {
  O(xdc_transform) O(dec_data_dim) O(xdc_element_pitch) O(rf_raw_dim) O(transmit_mode) O(decode) O(das_shader_id)
  O(time_offset) O(output_min_coordinate) O(output_max_coordinate) O(output_points) O(sampling_frequency)
  O(center_frequency) O(speed_of_sound) O(off_axis_pos) O(beamform_plane) O(f_number) O(interpolate)
  O(coherency_weighting) O(decimation_rate) O(readi_group_id) O(readi_group_size)
  printf("size %zu %zu %zu %zu %zu\n", sizeof(BeamformerParameters), sizeof(BeamformerUIParameters),
         sizeof(BeamformerParametersHead), sizeof(BeamformerComputeStatsTable), sizeof(BeamformerLiveImagingParameters));
  return 0;
}
"""


def layout_of(header, tmp_path, name):
    src = tmp_path / f"{name}.c"
    src.write_text(LAYOUT_C.replace("HDR", f'"{header}"'))
    exe = tmp_path / name
    subprocess.check_call(["gcc", "-std=c11", str(src), "-o", str(exe)])
    return subprocess.check_output([str(exe)], text=True)


def test_parameter_layout(tmp_path):
    ours = layout_of(HEADER, tmp_path, "ours")
    expect = dict(xdc_transform=0, dec_data_dim=64, xdc_element_pitch=80, rf_raw_dim=88, transmit_mode=96, decode=100,
                  das_shader_id=104, time_offset=108, output_min_coordinate=112, output_max_coordinate=128,
                  output_points=144, sampling_frequency=160, center_frequency=164, speed_of_sound=168,
                  off_axis_pos=172, beamform_plane=176, f_number=180, interpolate=184, coherency_weighting=188,
                  decimation_rate=192, readi_group_id=196, readi_group_size=200)
    got = dict(line.split() for line in ours.splitlines() if not line.startswith("size"))
    assert {k: int(v) for k, v in got.items()} == expect
    assert "size 208 80 112 2048 64" in ours
    for name, off in expect.items():
        assert getattr(abi.BeamformerParameters, name).offset == off


@pytest.mark.skipif(not os.path.exists(REF_LAYOUT), reason="reference-side checkers not built (oracle/build_ref.py)")
def test_parameter_layout_equals_reference(tmp_path):
    """Our header's layout against the one oracle/build_ref.py printed from the
    reference's own beamformer_parameters.h."""
    ref = open(REF_LAYOUT).read()
    ours = layout_of(HEADER, tmp_path, "ours2")
    strip = lambda s: [ln for ln in s.splitlines() if not ln.startswith("size")]  # noqa: E731
    assert strip(ref) == strip(ours)
    assert ref.splitlines()[-1].split()[1:3] == ours.splitlines()[-1].split()[1:3]


def test_version_and_error_strings(lib):
    assert lib.beamformer_get_api_version() == 11
    assert lib.beamformer_error_string(99) == b"invalid error kind"
    assert lib.beamformer_error_string(-1) == b"invalid error kind"
    assert lib.beamformer_error_string(abi.ERR["CUDA_RUNTIME"]) == b"CUDA runtime error"


@pytest.mark.skipif(not os.path.exists(REF_CLIENT), reason="reference client library not built")
def test_error_strings_match_reference(lib):
    ref = ctypes.CDLL(REF_CLIENT)
    ref.beamformer_error_string.restype = ctypes.c_char_p
    ref.beamformer_error_string.argtypes = [ctypes.c_int32]
    for k in range(14):
        assert lib.beamformer_error_string(k) == ref.beamformer_error_string(k), k
    assert lib.beamformer_error_string(14 + 10) == ref.beamformer_error_string(14 + 10)


PIPELINE_CASES = [
    ([abi.SHADER["Decode"]] * 17, 0, "COMPUTE_STAGE_OVERFLOW"),
    ([abi.SHADER["Decode"], 15], 0, "INVALID_COMPUTE_STAGE"),
    ([abi.SHADER["Decode"], -1], 0, "INVALID_COMPUTE_STAGE"),
    ([abi.SHADER["DAS"]], 0, "INVALID_START_SHADER"),
    ([abi.SHADER["CudaDecode"], abi.SHADER["DAS"]], 0, "INVALID_START_SHADER"),
    ([abi.SHADER["Demodulate"], abi.SHADER["Decode"]], abi.DATA_KIND["Int16Complex"], "INVALID_DEMOD_DATA_KIND"),
    ([abi.SHADER["Demodulate"], abi.SHADER["Decode"]], abi.DATA_KIND["Float32Complex"], "INVALID_DEMOD_DATA_KIND"),
]


def push_pipeline(L, shaders, kind):
    arr = (ctypes.c_int32 * len(shaders))(*shaders)
    return L.beamformer_push_pipeline(arr, len(shaders), kind)


@pytest.mark.parametrize("shaders,kind,err", PIPELINE_CASES)
def test_pipeline_validation(lib, shaders, kind, err):
    assert push_pipeline(lib, shaders, kind) == 0
    assert lib.beamformer_get_last_error() == abi.ERR[err]
    if os.path.exists(REF_CLIENT):
        ref = ctypes.CDLL(REF_CLIENT)
        ref.beamformer_push_pipeline.argtypes = [ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_int32]
        ref.beamformer_push_pipeline.restype = ctypes.c_uint32
        ref.beamformer_get_last_error.restype = ctypes.c_int32
        arr = (ctypes.c_int32 * len(shaders))(*shaders)
        assert ref.beamformer_push_pipeline(arr, len(shaders), kind) == 0
        assert ref.beamformer_get_last_error() == abi.ERR[err]


def test_valid_pipeline_and_render_kind_pass_validation(lib):
    assert push_pipeline(lib, [abi.SHADER["Decode"], abi.SHADER["Demodulate"], abi.SHADER["DAS"]], 0) == 1
    # the reference accepts kind 14 (its range check is inclusive of ComputeCount)
    assert push_pipeline(lib, [abi.SHADER["Decode"], 14], 0) == 1
    assert push_pipeline(lib, [abi.SHADER["Demodulate"], abi.SHADER["Decode"]], abi.DATA_KIND["Float32"]) == 1


def test_timeouts_and_sizes(lib):
    assert lib.beamformer_set_global_timeout(-2) == 0
    assert lib.beamformer_get_last_error() == abi.ERR["INVALID_TIMEOUT"]
    for t in (-1, 0, 1000):
        assert lib.beamformer_set_global_timeout(t) == 1
    lib.beamformer_set_global_timeout(0)
    m = (ctypes.c_int16 * 257)()
    assert lib.beamformer_push_channel_mapping(m, 257) == 0
    assert lib.beamformer_get_last_error() == abi.ERR["BUFFER_OVERFLOW"]
    assert lib.beamformer_push_sparse_elements(m, 257) == 0
    f = (ctypes.c_float * 514)()
    assert lib.beamformer_push_focal_vectors(f, 257) == 0
    assert lib.beamformer_push_channel_mapping(m, 256) == 1
    assert lib.beamformer_push_focal_vectors(f, 256) == 1
    assert lib.beamformer_create_kaiser_low_pass_filter(5.65, 1e6, 25e6, 0, 0) == 0
    assert lib.beamformer_create_kaiser_low_pass_filter(5.65, 1e6, 25e6, 16, 5) == 1   # slot taken modulo 4
    taps = (ctypes.c_float * 16)()
    n = ctypes.c_int32()
    assert lib.beamformer_gb300_get_filter(1, taps, 16, ctypes.byref(n)) == 1 and n.value == 16
    from oracle import bf_oracle as O
    assert np.allclose(np.ctypeslib.as_array(taps), O.kaiser(1e6, 25e6, 5.65, 16), rtol=0, atol=1e-7)


def test_live_parameters_roundtrip(lib):
    lp = abi.BeamformerLiveImagingParameters(active=1, transmit_power=0.5)
    assert lib.beamformer_set_live_parameters(ctypes.byref(lp)) == 1
    got = lib.beamformer_get_live_parameters().contents
    assert got.active == 1 and abs(got.transmit_power - 0.5) < 1e-7
    assert lib.beamformer_live_parameters_get_dirty_flag() == -1


def test_parameters_sub_blocks(lib):
    bp = abi.BeamformerParameters()
    bp.f_number = 2.0
    assert lib.beamformer_push_parameters(ctypes.byref(bp)) == 1
    ui = abi.BeamformerUIParameters(f_number=1.5)
    assert lib.beamformer_push_parameters_ui(ctypes.byref(ui)) == 1
    head = abi.BeamformerParametersHead(das_shader_id=2)
    assert lib.beamformer_push_parameters_head(ctypes.byref(head)) == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_no_device_fails_loudly(lib):
    raw = np.zeros(64, np.int16)
    assert lib.beamformer_push_data(raw.ctypes.data_as(ctypes.c_void_p), raw.nbytes) == 0
    assert lib.beamformer_get_last_error() == abi.ERR["CUDA_DEVICE"]
    assert lib.beamformer_start_compute() == 0


def test_filter_precision_argument_checks(lib):
    assert lib.beamformer_gb300_set_filter_precision(3) == 0
    assert lib.beamformer_get_last_error() == abi.ERR["UNSUPPORTED"]
    assert lib.beamformer_gb300_set_filter_precision(-1) == 0
    for p in (1, 2, 0):
        assert lib.beamformer_gb300_set_filter_precision(p) == 1
    assert lib.beamformer_gb300_set_das_precision(2) == 0
    assert lib.beamformer_get_last_error() == abi.ERR["UNSUPPORTED"]
    assert lib.beamformer_gb300_set_das_precision(-1) == 0
    for p in (1, 0):
        assert lib.beamformer_gb300_set_das_precision(p) == 1
    from ogl_beamforming_cuda_gb300.client import Beamformer, BeamformerError
    with pytest.raises(BeamformerError):
        Beamformer().set_precision(das=2)
    with pytest.raises(BeamformerError):
        Beamformer().set_precision(filter=5)
    assert Beamformer().set_precision(filter=0, das=0) is not None


def test_server_rejects_bad_arguments():
    """ogl_beamformer_server refuses an unknown option and a DAS precision out of
    range before it creates the shared-memory region (no GPU needed)."""
    exe = os.path.join(ROOT, "ogl_beamforming_cuda_gb300", "lib", "ogl_beamformer_server")
    if not os.path.exists(exe):
        pytest.skip("server not built")
    r = subprocess.run([exe, "--bogus"], capture_output=True, text=True, timeout=30)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, "--das-precision", "7"], capture_output=True, text=True, timeout=30)
    assert r.returncode == 2 and "unsupported" in r.stderr.lower()
