"""CudaHilbert stage: the analytic signal of every channel row (the reference
runs it in its external cuda_toolkit plugin, beamformer.c:567-570; its source is
not part of the reference, so the oracle restates the FFT definition)."""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from oracle.bf_oracle import analytic_signal
from bf_cases import small_params, small_raw, run_both, check_volume

SH = abi.SHADER


def test_oracle_analytic_signal_definition():
    n = np.arange(256)
    for k in (1, 17, 127):
        z = analytic_signal(np.cos(2 * np.pi * k * n / 256))
        assert np.allclose(z, np.exp(2j * np.pi * k * n / 256), atol=1e-12)
    x = np.random.default_rng(2).standard_normal((4, 100))
    z = analytic_signal(x)
    assert np.allclose(z.real, x, atol=1e-12)
    # the spectrum of the analytic signal has no negative frequencies
    assert np.max(np.abs(np.fft.fft(z)[:, 51:])) < 1e-9


def test_oracle_analytic_signal_matches_scipy():
    sig = pytest.importorskip("scipy.signal")
    for n in (64, 63, 2):
        x = np.random.default_rng(n).standard_normal((3, n))
        assert np.max(np.abs(analytic_signal(x) - sig.hilbert(x))) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("S,C,T", [(512, 16, 16), (2048, 8, 8), (16384, 2, 2), (16, 4, 4)])
def test_hilbert_stage_against_oracle(S, C, T):
    bp = small_params(S=S, C=C, T=T, D=1)
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["CudaHilbert"]], raw)
    n = 2 * S * C * T
    check_volume(bf.channel_data()[:n], ref["channel_data"][:n], f"CudaHilbert S={S}")


@pytest.mark.gpu
@pytest.mark.parametrize("interp", (0, 1))
def test_hilbert_then_das_against_oracle(interp):
    bp = small_params(S=512, C=16, T=16, points=(16, 2, 20), D=1, interp=interp)
    raw = small_raw(bp)
    bf, ref = run_both(bp, [SH["Decode"], SH["CudaHilbert"], SH["DASFast"]], raw)
    check_volume(bf.frame(0)[0], ref["frame"], f"Decode -> CudaHilbert -> DAS interp={interp}")


@pytest.mark.gpu
def test_hilbert_dropped_with_demodulate():
    """The planner keeps CudaHilbert only without a Demodulate stage (beamformer.c:325)."""
    bp = small_params(S=512, C=16, T=16, D=2)
    raw = small_raw(bp)
    a, _ = run_both(bp, [SH["Decode"], SH["CudaHilbert"], SH["Demodulate"], SH["DAS"]], raw)
    va = a.frame(0)[0].copy()
    b, _ = run_both(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], raw)
    assert np.array_equal(va.view(np.uint32), b.frame(0)[0].view(np.uint32))


@pytest.mark.gpu
def test_hilbert_needs_power_of_two_rows():
    from ogl_beamforming_cuda_gb300.client import Beamformer
    bp = small_params(S=384, C=8, T=8, D=1)
    raw = small_raw(bp)
    bf = Beamformer().configure(bp, [SH["Decode"], SH["CudaHilbert"]])
    ok = bf.lib.beamformer_push_data_with_compute(raw.ctypes.data, raw.nbytes, 0)
    assert ok == 0 and bf.lib.beamformer_get_last_error() == abi.ERR["UNSUPPORTED"]
