"""GPU parity: every stage of the CUDA pipeline against the CPU oracle, through the
C ABI (decode bit-exact; float stages NRMSE <= -80 dB and max-abs <= 1e-4 of peak).
"""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi, synth
from bf_cases import small_params, small_raw, run_both, check_volume, oracle_for

pytestmark = pytest.mark.gpu
SH = abi.SHADER
DK = abi.DATA_KIND

def perm_map(n, seed=5):
    return np.concatenate([np.random.default_rng(seed).permutation(n), np.arange(n, 256)]).astype(np.int16)


TEST_MAP = perm_map(16)


@pytest.mark.parametrize("T", [2, 4, 8, 16, 32, 64, 128])
@pytest.mark.parametrize("to_float", [False, True])
def test_decode_sylvester_bit_exact(T, to_float):
    bp = small_params(S=256, C=16, T=T)
    raw = np.random.default_rng(T).integers(-32768, 32767, size=(16, T, 256), dtype=np.int16)
    pipe = [SH["Decode"], SH["Demodulate"]] if to_float else [SH["Decode"]]
    bf, ref = run_both(bp, pipe, raw, chmap=TEST_MAP)
    got = bf.channel_data()
    exp = ref["channel_data"]
    if to_float:
        check_volume(got, exp, "decode->demod")
    else:
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


@pytest.mark.parametrize("T", [12, 20, 24, 40, 256])
def test_decode_kronecker_and_large_orders_bit_exact(T):
    bp = small_params(S=128, C=8, T=T)
    raw = np.random.default_rng(T).integers(-32768, 32767, size=(8, T, 128), dtype=np.int16)
    bf, ref = run_both(bp, [SH["Decode"]], raw)
    assert np.array_equal(bf.channel_data().view(np.uint32), ref["channel_data"].view(np.uint32))


@pytest.mark.parametrize("kind,shape,dtype", [
    ("Int16Complex", (8, 16, 64, 2), np.int16), ("Float32", (8, 16, 64), np.float32),
    ("Float32Complex", (8, 16, 64, 2), np.float32)])
def test_decode_other_data_kinds(kind, shape, dtype):
    bp = small_params(S=64, C=8, T=16)
    rng = np.random.default_rng(11)
    raw = (rng.integers(-30000, 30000, size=shape).astype(dtype) if dtype == np.int16
           else rng.standard_normal(shape).astype(dtype))
    bf, ref = run_both(bp, [SH["Decode"]], raw, data_kind=DK[kind])
    assert np.array_equal(bf.channel_data().view(np.uint32), ref["channel_data"].view(np.uint32))


def test_decode_mode_none_reshapes():
    bp = small_params(S=64, C=8, T=16)
    bp.decode = 0
    raw = np.random.default_rng(2).integers(-32768, 32767, size=(8, 16, 64), dtype=np.int16)
    bf, ref = run_both(bp, [SH["Decode"]], raw, chmap=perm_map(8))
    assert np.array_equal(bf.channel_data().view(np.uint32), ref["channel_data"].view(np.uint32))


@pytest.mark.parametrize("D,L", [(1, 16), (2, 32), (2, 64), (4, 64), (3, 37)])
def test_demodulate_fir(D, L):
    bp = small_params(S=512, C=16, T=16, D=D)
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"]], raw, kaiser=(5.65, 5e6, 25e6, L))
    check_volume(bf.channel_data(), ref["channel_data"], f"demod D={D} L={L}")


def test_matched_filter_stage():
    bp = small_params(S=512, C=16, T=16, D=2)
    raw = small_raw(bp)
    pipe = [SH["Decode"], SH["Demodulate"], SH["Filter"]]
    bf, ref = run_both(bp, pipe, raw, matched=(12.5e6, 12.5e6, 12.5e6 * 4, 20, 1), slots={2: 1})
    # The Filter stage writes [channel][transmit][sample] with channel stride
    # output_channel_stride; past that region its output buffer still holds the
    # Decode stage's output (the reference's release build clears nothing between
    # stages, the oracle zeroes each stage's output), so only the written region
    # is compared.
    n = 2 * int(ref["plan"].filter.output_channel_stride) * int(bp.dec_data_dim[1])
    check_volume(bf.channel_data()[:n], ref["channel_data"][:n], "decode->demod->matched filter")


def test_demodulate_first_int16_snorm_then_decode():
    bp = small_params(S=512, C=16, T=16, D=2)
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Demodulate"], SH["Decode"]], raw, chmap=perm_map(16))
    check_volume(bf.channel_data(), ref["channel_data"], "demod(i16)->decode")


def test_demodulate_first_float_then_decode():
    bp = small_params(S=512, C=16, T=16, D=2)
    raw = small_raw(bp).astype(np.float32) / 16384.0
    bf, ref = run_both(bp, [SH["Demodulate"], SH["Decode"]], raw, data_kind=DK["Float32"])
    check_volume(bf.channel_data(), ref["channel_data"], "demod(f32)->decode")


DAS_CASES = [(das, interp, coh) for das in ("HERCULES", "UHERCULES", "FORCES", "UFORCES", "RCA_TPW", "RCA_VLS", "FLASH")
             for interp in (0, 1, 2) for coh in (0, 1)]


@pytest.mark.parametrize("das,interp,coh", DAS_CASES)
def test_das_modes(das, interp, coh):
    bp = small_params(S=512, C=16, T=16, points=(16, 3, 20), das=das, coherency=coh)
    raw = small_raw(bp)
    rng = np.random.default_rng(9)
    focal = np.zeros(512, np.float32)
    focal[0::2] = rng.uniform(-8, 8, 256)
    focal[1::2] = np.where(rng.random(256) < 0.5, np.inf, rng.uniform(5e-3, 3e-2, 256))
    focal[0], focal[1] = 0.0, np.inf
    sparse = rng.permutation(16).astype(np.int16)
    sparse = np.concatenate([sparse, np.arange(16, 256, dtype=np.int16)])
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], raw, focal=focal, sparse=sparse,
                       interpolation=interp)
    vol, dims = bf.frame(0)
    check_volume(vol, ref["frame"], f"DAS {das} interp={interp} coherency={coh}")


@pytest.mark.parametrize("interp", (0, 1, 2))
@pytest.mark.parametrize("points", ((16, 3, 20), (40, 1, 48)))
def test_das_hercules_generic_kernel(monkeypatch, interp, points):
    """HERCULES volumes normally take the dedicated kernel; the general kernel
    (OGL_BF_DAS_GENERIC=1) must agree with the oracle too."""
    monkeypatch.setenv("OGL_BF_DAS_GENERIC", "1")
    bp = small_params(S=512, C=16, T=16, points=points)
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], raw, interpolation=interp)
    check_volume(bf.frame(0)[0], ref["frame"], f"HERCULES general kernel interp={interp}")


@pytest.mark.parametrize("interp", (0, 1, 2))
def test_das_hercules_plane_32_channels(interp):
    bp = small_params(S=1024, C=32, T=32, points=(48, 1, 64), D=2)
    raw = small_raw(bp, n_points=12, n_speckle=200)
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DASFast"]], raw, interpolation=interp)
    check_volume(bf.frame(0)[0], ref["frame"], f"HERCULES DASFast 32x32 interp={interp}")


@pytest.mark.parametrize("interp", (0, 1, 2))
@pytest.mark.parametrize("fc_scale", (0.5, 0.77, 1.0, 1.3, 2.0))
def test_das_hercules_phase_paths(interp, fc_scale):
    """Demodulation phase of the table path: the phase of the integer sample (cubic
    and linear: of the segment's middle) sits in the per-frame table and the term
    rotates by the rest (the bench has theta = 2 pi fc / fs = 2 pi exactly; above
    2 pi that angle is reduced first). Nearest uses rotated samples for voxels
    whose indices are proven in range and the reference's angle elsewhere."""
    bp = small_params(S=2048, C=16, T=16, points=(24, 2, 48), D=2)
    bp.center_frequency *= fc_scale
    raw = small_raw(bp, n_points=12, n_speckle=300)
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DASFast"]], raw, interpolation=interp)
    check_volume(bf.frame(0)[0], ref["frame"], f"HERCULES phase fc x {fc_scale} interp={interp}")


def test_das_unknown_kind_is_zero():
    bp = small_params(S=512, C=16, T=16, das="RACES")
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], raw)
    vol, _ = bf.frame(0)
    assert not np.any(vol) and not np.any(ref["frame"])


def test_das_without_demodulation_uses_no_phase():
    bp = small_params(S=256, C=16, T=16, D=1)
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["DAS"]], raw, kaiser=None)
    check_volume(bf.frame(0)[0], ref["frame"], "decode->DAS (fc = 0)")


def test_sum_and_min_max_bit_exact():
    bp = small_params(S=512, C=16, T=16, points=(64, 2, 64), frames=4)
    pipe = [SH["Decode"], SH["Demodulate"], SH["DAS"], SH["Sum"], SH["MinMax"]]
    from ogl_beamforming_cuda_gb300.client import Beamformer
    from oracle.bf_oracle import OraclePipeline
    bf = Beamformer().configure(bp, pipe, kaiser=(5.65, 5e6, 25e6, 32))
    orc = oracle_for(bf, bp, pipe, kaiser=(5.65, 5e6, 25e6, 32))
    gpu_frames = []
    for seed in range(6):       # more frames than averaged: the ring wraps
        raw = small_raw(bp, seed=seed)
        bf.push(raw)
        ref = orc.compute(raw)
        bf.synchronize()
        gpu_frames.append(bf.frame(0)[0].copy())
    das, _ = bf.frame(0)
    check_volume(das, ref["frame"], "DAS frame")
    avg, _ = bf.frame(1)
    check_volume(avg, ref["averaged"], "averaged frame")
    # sum and min/max themselves are bit exact: feed the GPU frames to the oracle
    from oracle import bf_oracle as O
    expect = O.sum_frames(gpu_frames[-4:], np.float32(1.0) / np.float32(4), (64, 2, 64))
    assert np.array_equal(avg.view(np.uint32), expect.view(np.uint32)), "Sum not bit-exact"
    levels = O.min_max(das, (64, 2, 64))
    off = 0
    mips = O.frame_mips((64, 2, 64))
    for lvl in range(1, mips):
        got, d = bf.frame(0, lvl)
        n = got.size
        assert np.array_equal(got, levels[off:off + n], equal_nan=True), f"mip {lvl}"
        off += n


def test_beamform_data_synchronized_matches_oracle():
    bp = small_params(S=512, C=32, T=32, points=(32, 1, 32))
    raw = small_raw(bp)
    from ogl_beamforming_cuda_gb300.client import Beamformer
    bf = Beamformer().configure(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], kaiser=(5.65, 5e6, 25e6, 32))
    vol = bf.beamform(raw)
    orc = oracle_for(bf, bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], kaiser=(5.65, 5e6, 25e6, 32))
    check_volume(vol, orc.compute(raw)["frame"], "beamform_data_synchronized")


def test_device_input_waits_for_default_stream_writes():
    """push_data_device: RF written on the legacy default stream (PyTorch's default)
    behind a bounded delay is complete before the library's compute reads it."""
    import torch
    from ogl_beamforming_cuda_gb300.client import Beamformer
    bp = small_params(S=512, C=16, T=16)
    raw = small_raw(bp)
    bf = Beamformer().configure(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], kaiser=(5.65, 5e6, 25e6, 32))
    orc = oracle_for(bf, bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], kaiser=(5.65, 5e6, 25e6, 32))
    ref = orc.compute(raw)
    host = torch.from_numpy(raw).pin_memory()
    dev = torch.zeros(raw.shape, dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    torch.cuda._sleep(200_000_000)              # ~0.1 s of GPU time on the default stream
    dev.copy_(host, non_blocking=True)          # queued behind it
    bf.push_device(dev.data_ptr(), dev.numel() * 2)
    bf.synchronize()
    check_volume(bf.frame(0)[0], ref["frame"], "device input behind default-stream work")


@pytest.mark.parametrize("dims", [(64, 2, 64), (17, 1, 40), (100, 3, 70), (128, 1, 128), (33, 65, 7), (1, 1, 1),
                                  (256, 4, 96)])
def test_min_max_pyramid_shapes(dims):
    """Every mip level bit-exact against the oracle for sizes that are not powers
    of two, planes, single texels and frames whose dispatch leaves NaN regions."""
    from ogl_beamforming_cuda_gb300.client import Beamformer
    from oracle import bf_oracle as O
    bp = small_params(S=256, C=8, T=8, points=dims)
    pipe = [SH["Decode"], SH["Demodulate"], SH["DAS"], SH["MinMax"]]
    bf = Beamformer().configure(bp, pipe, kaiser=(5.65, 5e6, 25e6, 16))
    bf.push(small_raw(bp))
    bf.synchronize()
    das, _ = bf.frame(0)
    levels = O.min_max(das, dims)
    off = 0
    for lvl in range(1, O.frame_mips(dims)):
        got, d = bf.frame(0, lvl)
        assert np.array_equal(got, levels[off:off + got.size], equal_nan=True), f"mip {lvl} of {dims}"
        off += got.size


def transformed_xdc(bp, z_degrees, scale, x_degrees=0.0):
    """xdc_transform with a rotation about z (then about x), scaled, translation
    kept: the transducer frame the reference applies per voxel (das.glsl:182,
    220, 263). The stored matrix is column-major: X[column][row]."""
    X = np.asarray(bp.xdc_transform[:], np.float64).reshape(4, 4)
    a, b = np.radians(z_degrees), np.radians(x_degrees)
    rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    rx = np.array([[1, 0, 0], [0, np.cos(b), -np.sin(b)], [0, np.sin(b), np.cos(b)]])
    M = scale * (rx @ rz)                       # row-major M[row][column]
    X[:3, :3] = M.T
    bp.xdc_transform[:] = X.astype(np.float32).ravel().tolist()
    return bp


XDC_CASES = [(25.0, 1.1, 0.0), (-40.0, 0.8, 0.0), (15.0, 1.0, 8.0)]


@pytest.mark.parametrize("z_deg,scale,x_deg", XDC_CASES)
@pytest.mark.parametrize("interp", (0, 1, 2))
@pytest.mark.parametrize("kernel", ("hercules", "generic", "forces"))
def test_das_rotated_scaled_transducer_transform(monkeypatch, z_deg, scale, x_deg, interp, kernel):
    """A rotated and scaled (and, in the last case, tilted) xdc_transform through
    the HERCULES fast path (its per-voxel range proof works in transducer
    coordinates), the general kernel and FORCES, against the oracle."""
    if kernel == "generic":
        monkeypatch.setenv("OGL_BF_DAS_GENERIC", "1")
    das = "FORCES" if kernel == "forces" else "HERCULES"
    bp = transformed_xdc(small_params(S=1024, C=16, T=16, points=(20, 4, 24), das=das), z_deg, scale, x_deg)
    raw = small_raw(bp, n_points=10, n_speckle=200)
    shader = SH["DASFast"] if kernel == "hercules" else SH["DAS"]
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], shader], raw, interpolation=interp)
    assert np.any(ref["frame"] != 0)
    check_volume(bf.frame(0)[0], ref["frame"], f"{kernel} xdc rot z {z_deg} x {x_deg} scale {scale} interp={interp}")


@pytest.mark.parametrize("interp", (1, 2))
@pytest.mark.parametrize("points", ((48, 1, 64), (16, 6, 32)))
@pytest.mark.parametrize("fc_scale", (1.0, 2.0))
def test_das_forces_fast_path(interp, points, fc_scale):
    """FORCES through the fast path (per-frame table, proven voxels; the rest on
    the general per-voxel code), deep enough that most voxels carry the proof,
    both demodulation phase paths (theta = 2 pi and 4 pi), against the oracle."""
    bp = small_params(S=1024, C=32, T=32, points=points, das="FORCES")
    bp.center_frequency *= fc_scale
    raw = small_raw(bp, n_points=12, n_speckle=200)
    bf, ref = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], raw, interpolation=interp)
    check_volume(bf.frame(0)[0], ref["frame"], f"FORCES fast path interp={interp} {points} fc x {fc_scale}")


@pytest.mark.parametrize("interp", (1, 2))
def test_das_forces_fast_path_without_demodulation(interp):
    bp = small_params(S=512, C=16, T=16, points=(24, 2, 40), D=1, das="FORCES")
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["DAS"]], raw, kaiser=None, interpolation=interp)
    check_volume(bf.frame(0)[0], ref["frame"], f"FORCES fast path, no demodulation, interp={interp}")
