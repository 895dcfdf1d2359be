"""Precision variant: the Decode output rounded once to FP16 or BF16 and the
demodulating FIR run as a Toeplitz contraction on the tensor cores (FP32
accumulate), beside the FP32 pipeline. Every stage's error is measured against
the FP64 restatement of the oracle on identical seeded int16 RF."""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from ogl_beamforming_cuda_gb300.client import Beamformer
from bf_cases import small_params, small_raw, oracle_for, fp64_front_end, nrmse
import oracle.bf_oracle as O

pytestmark = pytest.mark.gpu
SH = abi.SHADER
PIPE = [SH["Decode"], SH["Demodulate"], SH["DAS"]]

# error bounds against FP64 (dB): FP32 is the reference arithmetic; FP16 keeps
# 11 significant bits of each decoded sample and tap, BF16 8
BOUND = {0: -85.0, 1: -65.0, 2: -48.0}


def run(bp, raw, kaiser, precision, interpolation=-1):
    bf = Beamformer().configure(bp, PIPE, kaiser=kaiser, interpolation=interpolation)
    assert bf.lib.beamformer_gb300_set_filter_precision(precision)
    bf.push(raw)
    bf.synchronize()
    return bf


@pytest.mark.parametrize("S,C,L,D", [(1024, 32, 64, 2), (2048, 32, 128, 2), (1024, 16, 64, 1), (1024, 16, 64, 4),
                                     (1024, 16, 37, 2)])
def test_precision_stages_against_fp64(S, C, L, D):
    bp = small_params(S=S, C=C, T=C, points=(48, 1, 64), D=D)
    raw = small_raw(bp, n_points=12, n_speckle=200)
    kaiser = (5.65, 5e6, 25e6, L)
    bf0 = run(bp, raw, kaiser, 0)
    orc = oracle_for(bf0, bp, PIPE, kaiser=kaiser)
    ref = orc.compute(raw, want_stages=True)
    dem64, n = fp64_front_end(ref, kaiser, C)
    p = ref["plan"]
    vol64 = O.das(p.das, dem64[: p.rf_size // 4], (48, 1, 64), orc.sparse, orc.focal, fast=True, f64=True)
    for prec in (0, 1, 2):
        bf = bf0 if prec == 0 else run(bp, raw, kaiser, prec)
        e_dem = nrmse(bf.channel_data()[:n], dem64[:n])
        e_vol = nrmse(bf.frame(0)[0], vol64)
        print(f"S={S} C={C} L={L} D={D} precision={prec}: demod {e_dem:.1f} dB, volume {e_vol:.1f} dB vs FP64")
        assert e_dem <= BOUND[prec], (prec, e_dem)
        assert e_vol <= BOUND[prec], (prec, e_vol)


def test_precision_needs_decode_then_demodulate():
    bp = small_params(S=512, C=16, T=16, D=2)
    raw = small_raw(bp)
    bf = Beamformer().configure(bp, [SH["Demodulate"], SH["Decode"], SH["DAS"]], kaiser=(5.65, 5e6, 25e6, 32))
    assert bf.lib.beamformer_gb300_set_filter_precision(1)
    ok = bf.lib.beamformer_push_data_with_compute(raw.ctypes.data, raw.nbytes, 0)
    assert ok == 0 and bf.lib.beamformer_get_last_error() == abi.ERR["UNSUPPORTED"]
    assert bf.lib.beamformer_gb300_set_filter_precision(0)
