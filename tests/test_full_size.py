"""GPU parity at the benchmark workloads' full sizes, through the C ABI, against
the CPU oracle (the reference's semantics) on the same seeded int16 RF.

- Plane workload: HERCULES, T = C = 128 transmits and receive channels, S = 2048
  samples, 64-tap Kaiser, decimation 2, linear interpolation, the whole
  128 x 1 x 128 x-z plane.
- Decode at T = C = 128, S = 2048: bit-exact (the FWHT kernel of order 128
  that the benchmarks run).
- 3D workload: 128 x 128 x 256 cubic volume through the HERCULES fast path
  with its channel groups, compared on stratified voxel runs (the oracle's voxel
  ranges); then 16 frames through Sum and MinMax, both bit-exact against the
  oracle's Sum and MinMax of the GPU's own frames.
- Precision workload front end: S = 4096, 128 taps; FP32 against the oracle,
  FP16 / BF16 (tensor-core FIR) against the FP64 restatement, with the plane.
- FORCES at the batched workload's largest size (128 x 128 x 256 cubic,
  T = C = 128, S = 2048) through its fast path, on stratified voxel runs.

Tolerances: decode, Sum and MinMax bit-exact; the float stages NRMSE <= -80 dB
and max |err| <= 1e-4 of the peak against the oracle; FP16 <= -65 dB and BF16
<= -48 dB against FP64.
"""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi, synth
from ogl_beamforming_cuda_gb300.client import Beamformer
from bf_cases import check_volume, oracle_for, fp64_front_end, nrmse
import oracle.bf_oracle as O

pytestmark = pytest.mark.gpu
SH = abi.SHADER
PIPE = [SH["Decode"], SH["Demodulate"], SH["DAS"]]
PRECISION_BOUND = {1: -65.0, 2: -48.0}


def plane_params(samples=2048, filter_length=64, interpolate=0):
    return synth.make_parameters(samples=samples, channels=128, transmits=128, points=(128, 1, 128), decimation=2,
                                 f_number=1.0, interpolate=interpolate, filter_length=filter_length)


def plane_raw(bp, seed):
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    pos, amp = synth.scatterers(seed, 20)
    return synth.encode_and_quantise(synth.decoded_traces(bp, pos, amp, device=dev), seed).cpu().numpy()


def test_plane_workload_whole_plane_linear():
    bp = plane_params()
    kaiser = synth.kaiser_spec(64)
    raw = plane_raw(bp, 11)
    bf = Beamformer().configure(bp, PIPE, kaiser=kaiser, interpolation=2)
    bf.push(raw)
    bf.synchronize()
    vol, dims = bf.frame(0)
    assert dims == (128, 1, 128)
    orc = oracle_for(bf, bp, PIPE, kaiser=kaiser)
    orc.interpolation = 2
    ref = orc.compute(raw)
    check_volume(bf.channel_data(), ref["channel_data"], "plane workload: demodulated channel data")
    db = check_volume(vol, ref["frame"], "plane workload: 128 x 128 plane, linear")
    print(f"plane workload: {db:.1f} dB")


def test_decode_order_128_full_size_bit_exact():
    bp = plane_params()
    raw = plane_raw(bp, 12)
    bf = Beamformer().configure(bp, [SH["Decode"]])
    bf.push(raw)
    bf.synchronize()
    orc = oracle_for(bf, bp, [SH["Decode"]])
    ref = orc.compute(raw)["channel_data"]
    got = bf.channel_data()
    assert got.size == ref.size
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def volume_params():
    return synth.make_parameters(samples=2048, channels=128, transmits=128, points=(128, 128, 256), decimation=2,
                                 f_number=1.0, interpolate=1, frames=16, filter_length=64)


def test_volume_workload_stratified_voxels_sum_and_min_max():
    import torch
    bp = volume_params()
    pipe = synth.default_pipeline(sum_and_minmax=True)
    kaiser = synth.kaiser_spec(64)
    dims = (128, 128, 256)
    V = int(np.prod(dims))
    pos, amp = synth.scatterers(5, 200, 4000)
    traces = synth.decoded_traces(bp, pos, amp, device="cuda")
    bf = Beamformer().configure(bp, pipe, kaiser=kaiser)
    orc = oracle_for(bf, bp, pipe, kaiser=kaiser)
    frames = []
    raw0 = None
    for k in range(16):
        raw = synth.encode_and_quantise(traces, 100 + k).cpu().numpy()
        if k == 0:
            raw0 = raw
        bf.push(raw)
        bf.synchronize()
        frames.append(bf.frame(0)[0].copy())
    del traces
    torch.cuda.empty_cache()

    # DAS of the first frame on stratified voxel runs (shallow and deep, central
    # and edge voxels) against the oracle on the oracle's own channel data
    orc.shaders = [SH["Decode"], SH["Demodulate"]]
    front = orc.compute(raw0)
    plan = O.plan(bp, pipe, [0] * len(pipe), abi.DATA_KIND["Int16"],
                  [(0, kaiser[3], kaiser[2], kaiser[0], kaiser[1]), None, None, None])
    rf = front["channel_data"][: plan.rf_size // 4]
    ranges, per = 16, 384
    stratum = V // ranges
    rng = np.random.default_rng(3)
    got, exp = [], []
    out = np.zeros(2 * V, np.float32)
    for i in range(ranges):
        v0 = stratum * i + int(rng.integers(0, stratum - per))
        O.das(plan.das, rf, dims, orc.sparse, orc.focal, fast=True, voxel_begin=v0, voxel_end=v0 + per, out=out)
        got.append(frames[0][2 * v0: 2 * (v0 + per)])
        exp.append(out[2 * v0: 2 * (v0 + per)].copy())
    db = check_volume(np.concatenate(got), np.concatenate(exp), "3D workload: stratified voxels, cubic")
    print(f"3D workload, {ranges * per} voxels: {db:.1f} dB")

    # Sum of the 16 frames and the MinMax pyramid of the last, bit-exact
    averaged, _ = bf.frame(1)
    expect = O.sum_frames(frames, np.float32(1.0) / np.float32(16), dims)
    assert np.array_equal(averaged.view(np.uint32), expect.view(np.uint32)), "16-frame Sum not bit-exact"
    levels = O.min_max(frames[-1], dims)
    off = 0
    for lvl in range(1, O.frame_mips(dims)):
        g, _ = bf.frame(0, lvl)
        assert np.array_equal(g, levels[off:off + g.size], equal_nan=True), f"mip {lvl}"
        off += g.size


@pytest.mark.parametrize("precision", (0, 1, 2))
def test_precision_workload_front_end(precision):
    bp = plane_params(samples=4096, filter_length=128, interpolate=0)
    kaiser = synth.kaiser_spec(128)
    raw = plane_raw(bp, 13)
    bf = Beamformer().configure(bp, PIPE, kaiser=kaiser, interpolation=2)
    assert bf.lib.beamformer_gb300_set_filter_precision(precision)
    try:
        bf.push(raw)
        bf.synchronize()
        chan = bf.channel_data()
        vol = bf.frame(0)[0]
    finally:
        assert bf.lib.beamformer_gb300_set_filter_precision(0)
    orc = oracle_for(bf, bp, PIPE, kaiser=kaiser)
    orc.interpolation = 2
    ref = orc.compute(raw, want_stages=precision != 0)
    if precision == 0:
        check_volume(chan, ref["channel_data"], "S = 4096, 128 taps: demodulated channel data (FP32)")
        check_volume(vol, ref["frame"], "S = 4096, 128 taps: plane (FP32)")
        return
    dem64, n = fp64_front_end(ref, kaiser, 128)
    p = ref["plan"]
    vol64 = O.das(p.das, dem64[: p.rf_size // 4], (128, 1, 128), orc.sparse, orc.focal, fast=True, f64=True,
                  interpolation=2)
    e_dem, e_vol = nrmse(chan[:n], dem64[:n]), nrmse(vol, vol64)
    print(f"precision {precision}: demodulated {e_dem:.1f} dB, plane {e_vol:.1f} dB against FP64")
    assert e_dem <= PRECISION_BOUND[precision], e_dem
    assert e_vol <= PRECISION_BOUND[precision], e_vol


def test_volume_workload_every_block_staged(monkeypatch):
    """The 3D workload's DAS reads every term from shared-memory windows: with
    OGL_BF_DAS_STAGED=require a block that could not stage would write NaN
    instead of running the unstaged code. FP32 against the oracle on stratified
    voxels; the FP16 table (DAS precision 1) against FP32 within -50 dB."""
    monkeypatch.setenv("OGL_BF_DAS_STAGED", "require")
    bp = volume_params()
    bp.output_points[3] = 1
    pipe = PIPE
    kaiser = synth.kaiser_spec(64)
    dims = (128, 128, 256)
    raw = synth.acquisition(bp, 17, n_points=200, n_speckle=2000, device="cuda")
    bf = Beamformer().configure(bp, pipe, kaiser=kaiser)
    vols = {}
    try:
        for prec in (0, 1):
            assert bf.lib.beamformer_gb300_set_das_precision(prec)
            bf.push(raw)
            bf.synchronize()
            vols[prec] = bf.frame(0)[0].copy()
    finally:
        bf.lib.beamformer_gb300_set_das_precision(0)
    assert np.all(np.isfinite(vols[0])) and np.all(np.isfinite(vols[1]))
    assert nrmse(vols[1], vols[0]) <= -50.0
    orc = oracle_for(bf, bp, pipe, kaiser=kaiser)
    orc.shaders = [SH["Decode"], SH["Demodulate"]]
    front = orc.compute(raw)
    plan = O.plan(bp, pipe, [0] * len(pipe), abi.DATA_KIND["Int16"],
                  [(0, kaiser[3], kaiser[2], kaiser[0], kaiser[1]), None, None, None])
    rf = front["channel_data"][: plan.rf_size // 4]
    V, per = int(np.prod(dims)), 256
    out = np.zeros(2 * V, np.float32)
    got, got16, exp = [], [], []
    for i in range(8):
        v0 = (V // 8) * i + 4096 * (i % 4)
        O.das(plan.das, rf, dims, orc.sparse, orc.focal, fast=True, voxel_begin=v0, voxel_end=v0 + per, out=out)
        got.append(vols[0][2 * v0: 2 * (v0 + per)])
        got16.append(vols[1][2 * v0: 2 * (v0 + per)])
        exp.append(out[2 * v0: 2 * (v0 + per)].copy())
    check_volume(np.concatenate(got), np.concatenate(exp), "3D workload, staged blocks only")
    # the FP16 table against the oracle itself (not only against the FP32 volume)
    assert nrmse(np.concatenate(got16), np.concatenate(exp)) <= -50.0


def test_forces_volume_full_size_stratified():
    """FORCES at the batched workload's largest size: 128 x 128 x 256 cubic volume,
    T = C = 128, S = 2048, through the FORCES fast path (per-frame table,
    in-range proof) with its channel groups; stratified voxel runs against the
    oracle."""
    bp = synth.make_parameters(samples=2048, channels=128, transmits=128, points=(128, 128, 256), decimation=2,
                               f_number=1.0, interpolate=1, das_id="FORCES", filter_length=64)
    bp.output_points[3] = 1
    kaiser = synth.kaiser_spec(64)
    dims = (128, 128, 256)
    raw = synth.acquisition(bp, 23, n_points=60, n_speckle=600, device="cuda")
    bf = Beamformer().configure(bp, PIPE, kaiser=kaiser)
    bf.push(raw)
    bf.synchronize()
    vol = bf.frame(0)[0].copy()
    assert np.all(np.isfinite(vol))
    orc = oracle_for(bf, bp, PIPE, kaiser=kaiser)
    orc.shaders = [SH["Decode"], SH["Demodulate"]]
    front = orc.compute(raw)
    plan = O.plan(bp, PIPE, [0] * len(PIPE), abi.DATA_KIND["Int16"],
                  [(0, kaiser[3], kaiser[2], kaiser[0], kaiser[1]), None, None, None])
    rf = front["channel_data"][: plan.rf_size // 4]
    V, per = int(np.prod(dims)), 128
    out = np.zeros(2 * V, np.float32)
    got, exp = [], []
    for i in range(8):
        v0 = (V // 8) * i + 8192 * (i % 4) + 64
        O.das(plan.das, rf, dims, orc.sparse, orc.focal, fast=True, voxel_begin=v0, voxel_end=v0 + per, out=out)
        got.append(vol[2 * v0: 2 * (v0 + per)])
        exp.append(out[2 * v0: 2 * (v0 + per)].copy())
    check_volume(np.concatenate(got), np.concatenate(exp), "FORCES 128 x 128 x 256, stratified voxels")

