"""Waits and their limits on the GPU (the reference's timeout convention,
ogl_beamformer_lib_base.h:36-44: -1 waits without limit, 0 checks once, N waits
up to N ms). Every wait here ends: the limits are hit only by a compute that is
still running, never by a stuck one."""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi, synth
from ogl_beamforming_cuda_gb300.client import Beamformer

pytestmark = pytest.mark.gpu
SH = abi.SHADER


def _slow_pipeline():
    """A cubic 128 x 128 x 256 volume from 64 x 64 transmits and channels of 512
    samples: about 10 ms of DAS per frame from 4 MB of RF, long against the 0 and
    1 ms limits below and against one upload."""
    bp = synth.make_parameters(samples=512, channels=64, transmits=64, points=(128, 128, 256), decimation=2,
                               interpolate=1)
    raw = synth.acquisition(bp, 3, n_points=10, n_speckle=200)
    bf = Beamformer().configure(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]], kaiser=synth.kaiser_spec(64))
    bf.lib.beamformer_set_global_timeout(-1)
    bf.push(raw)
    bf.synchronize()
    return bf, raw


def test_synchronize_limits():
    bf, raw = _slow_pipeline()
    L = bf.lib
    bf.push(raw)
    assert L.beamformer_gb300_synchronize(0) == 0
    assert L.beamformer_get_last_error() == abi.ERR["SYNC_VARIABLE"]
    assert L.beamformer_gb300_synchronize(-1) == 1
    bf.push(raw)
    assert L.beamformer_gb300_synchronize(1) == 0
    assert L.beamformer_get_last_error() == abi.ERR["SYNC_VARIABLE"]
    assert L.beamformer_gb300_synchronize(10000) == 1
    v0 = bf.frame(0)[0].copy()
    bf.push(raw)
    bf.synchronize()
    assert np.array_equal(v0.view(np.uint32), bf.frame(0)[0].view(np.uint32))


def test_rf_ring_full_with_zero_timeout():
    """Three RF slots: with a 0 ms limit a push whose slot still feeds a running
    compute fails with SYNC_VARIABLE instead of waiting; with -1 it waits."""
    bf, raw = _slow_pipeline()
    L = bf.lib
    L.beamformer_set_global_timeout(0)
    ok = []
    for _ in range(16):
        ok.append(L.beamformer_push_data_with_compute(raw.ctypes.data, raw.nbytes, 0))
        if not ok[-1]:
            break
    assert ok[:3] == [1, 1, 1] and ok[-1] == 0, ok
    assert L.beamformer_get_last_error() == abi.ERR["SYNC_VARIABLE"]
    L.beamformer_set_global_timeout(-1)
    assert L.beamformer_push_data_with_compute(raw.ctypes.data, raw.nbytes, 0) == 1
    assert bf.synchronize()


def test_tensor_core_fir_wait_that_runs_out_is_reported(monkeypatch):
    """The tcgen05 FIR's mbarrier waits are bounded. A test hook makes each CTA's
    first wait one on a barrier that nothing arrives at, limited to ~1 ms: the
    wait runs out, the CTA drains the loads it issued and stops, and
    beamformer_gb300_synchronize reports the error word (CUDA_RUNTIME). The next
    compute without the hook runs normally and matches the oracle."""
    from bf_cases import small_params, small_raw, oracle_for
    bp = small_params(S=1024, C=32, T=32, points=(16, 1, 24), D=2)
    raw = small_raw(bp)
    kaiser = (5.65, 5e6, 25e6, 32)
    pipe = [SH["Decode"], SH["Demodulate"], SH["DAS"]]
    bf = Beamformer().configure(bp, pipe, kaiser=kaiser)
    L = bf.lib
    assert L.beamformer_gb300_set_filter_precision(1)
    try:
        monkeypatch.setenv("OGL_BF_TEST_FIR_STALL_CYCLES", "2000000")
        assert L.beamformer_push_data_with_compute(raw.ctypes.data, raw.nbytes, 0) == 1
        assert L.beamformer_gb300_synchronize(-1) == 0
        assert L.beamformer_get_last_error() == abi.ERR["CUDA_RUNTIME"]
        monkeypatch.delenv("OGL_BF_TEST_FIR_STALL_CYCLES")
        bf.push(raw)
        assert L.beamformer_gb300_synchronize(-1) == 1
        vol = bf.frame(0)[0].copy()
    finally:
        L.beamformer_gb300_set_filter_precision(0)
    ref = oracle_for(bf, bp, pipe, kaiser=kaiser).compute(raw)["frame"]
    from conftest import nrmse_db
    assert nrmse_db(vol, ref) <= -60.0
