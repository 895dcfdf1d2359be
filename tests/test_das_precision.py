"""DAS precision 1: the HERCULES interpolation table in FP16 (coefficients scaled
by a power of two from the frame's largest channel-data magnitude, segments
evaluated in packed FP16), the sample index from an approximate square root and
one FMA, a degree-3 apodization; FP32 sums. Checked against the oracle (the
reference's FP32 arithmetic) on identical seeded int16 RF, for every
interpolation, plane and volume tiles, both demodulation phase paths
(theta = 2 pi and 4 pi), data without demodulation, voxels outside the in-range
proof and input amplitudes far from full scale.

Bound: NRMSE <= -50 dB against the oracle (the mixed-precision metric allows
-40 dB; FP16 keeps 11 significant bits of each coefficient)."""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from ogl_beamforming_cuda_gb300.client import Beamformer
from bf_cases import small_params, small_raw, oracle_for, nrmse

pytestmark = pytest.mark.gpu
SH = abi.SHADER
KAISER = (5.65, 5e6, 25e6, 32)
BOUND_DB = -50.0


@pytest.fixture(autouse=True)
def fp32_afterwards():
    yield
    Beamformer().lib.beamformer_gb300_set_das_precision(0)


def half_vs_oracle(bp, pipe, raw, interp, kaiser=KAISER):
    bf = Beamformer().configure(bp, pipe, kaiser=kaiser, interpolation=interp)
    assert bf.lib.beamformer_gb300_set_das_precision(1)
    bf.push(raw)
    bf.synchronize()
    vol = bf.frame(0)[0].copy()
    orc = oracle_for(bf, bp, pipe, kaiser=kaiser)
    orc.interpolation = interp
    ref = orc.compute(raw)["frame"]
    assert np.all(np.isfinite(vol))
    return nrmse(vol, ref), vol, ref


@pytest.mark.parametrize("interp", (0, 1, 2))
@pytest.mark.parametrize("points", ((48, 1, 64), (16, 8, 32)))
@pytest.mark.parametrize("fc_scale", (1.0, 2.0))
def test_half_table_against_oracle(interp, points, fc_scale):
    bp = small_params(S=2048, C=16, T=16, points=points, D=2)
    bp.center_frequency *= fc_scale
    raw = small_raw(bp, n_points=12, n_speckle=300)
    db, _, _ = half_vs_oracle(bp, [SH["Decode"], SH["Demodulate"], SH["DASFast"]], raw, interp)
    print(f"interp={interp} points={points} fc x {fc_scale}: {db:.1f} dB")
    assert db <= BOUND_DB, db


@pytest.mark.parametrize("interp", (0, 1, 2))
def test_half_table_without_demodulation(interp):
    bp = small_params(S=512, C=16, T=16, points=(16, 4, 24), D=1)
    raw = small_raw(bp)
    db, _, _ = half_vs_oracle(bp, [SH["Decode"], SH["DASFast"]], raw, interp, kaiser=None)
    assert db <= BOUND_DB, db


@pytest.mark.parametrize("interp", (0, 1, 2))
def test_half_table_outside_the_proof(interp):
    """Voxels from the array plane (depth 0: the IEEE square root) to beyond the
    last sample (per-term range tests, nearest indices clamped to the table)."""
    bp = small_params(S=512, C=16, T=16, points=(12, 4, 40), D=2)
    bp.output_min_coordinate[2] = 0.0
    bp.output_max_coordinate[2] = 12e-3
    raw = small_raw(bp, n_points=10, n_speckle=200)
    db, vol, ref = half_vs_oracle(bp, [SH["Decode"], SH["Demodulate"], SH["DASFast"]], raw, interp)
    assert db <= BOUND_DB, db


@pytest.mark.parametrize("shift", (0, 7, 12))
def test_half_table_scale_follows_the_data(shift):
    """Quiet input (amplitudes divided by 2^shift, down to a few LSB): the
    power-of-two table scale keeps the FP16 coefficients in their normal range."""
    bp = small_params(S=1024, C=16, T=16, points=(16, 4, 32), D=2)
    raw = small_raw(bp, n_points=12, n_speckle=300)
    raw = (raw.astype(np.int32) >> shift).astype(np.int16)
    db, _, _ = half_vs_oracle(bp, [SH["Decode"], SH["Demodulate"], SH["DASFast"]], raw, 1)
    assert db <= BOUND_DB, db


def test_half_table_zero_input_is_zero():
    bp = small_params(S=512, C=16, T=16, points=(16, 4, 16), D=2)
    raw = np.zeros_like(small_raw(bp))
    bf = Beamformer().configure(bp, [SH["Decode"], SH["Demodulate"], SH["DASFast"]], kaiser=KAISER, interpolation=1)
    assert bf.lib.beamformer_gb300_set_das_precision(1)
    bf.push(raw)
    bf.synchronize()
    assert not np.any(bf.frame(0)[0])


@pytest.mark.parametrize("interp", (0, 1))
def test_batch_with_half_table(interp):
    """The batched variant with FP16 tables, each acquisition with its own scale:
    every volume against the oracle (FORCES acquisitions keep the FP32 path)."""
    from test_batch import make_batch, PIPE
    params, raws, rf, out = make_batch(40)
    bf = Beamformer().configure(params[0], PIPE, kaiser=KAISER, interpolation=interp)
    assert bf.lib.beamformer_gb300_set_das_precision(1)
    bf.beamform_batch(params, [t.data_ptr() for t in rf], [t.numel() * 2 for t in rf], [t.data_ptr() for t in out])
    for i, (bp, raw) in enumerate(zip(params, raws)):
        orc = oracle_for(bf, bp, PIPE, kaiser=KAISER)
        orc.interpolation = interp
        db = nrmse(out[i].cpu().numpy(), orc.compute(raw)["frame"])
        assert db <= BOUND_DB, (i, db)


def test_mixed_pipeline_through_the_reference_abi():
    """The whole mixed pipeline (FP16 decode output + tensor-core FIR, FP16 DAS
    table) through beamform_data_synchronized with a 4-frame Sum, against the
    oracle's FP32 pipeline on the same frames."""
    bp = small_params(S=1024, C=32, T=32, points=(16, 4, 32), D=2, frames=4)
    pipe = [SH["Decode"], SH["Demodulate"], SH["DAS"], SH["Sum"]]
    raws = [small_raw(bp, seed=60 + k, n_points=12, n_speckle=300) for k in range(4)]
    bf = Beamformer().configure(bp, pipe, kaiser=KAISER, interpolation=1)
    bf.set_precision(filter=1, das=1)
    try:
        for raw in raws[:-1]:
            bf.push(raw)
        vol = bf.beamform(raws[-1])
    finally:
        bf.set_precision(filter=0, das=0)
    orc = oracle_for(bf, bp, pipe, kaiser=KAISER)
    orc.interpolation = 1
    ref = None
    for raw in raws:
        ref = orc.compute(raw)["averaged"]
    db = nrmse(vol, ref)
    print(f"mixed pipeline, 4-frame sum: {db:.1f} dB")
    assert db <= BOUND_DB, db
