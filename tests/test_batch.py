"""Batched variant: acquisitions of different transmit and sample counts, output
grids and DAS modes beamformed by one call (front ends per acquisition, one
persistent DAS launch, CUDA graph replay), each checked against the oracle."""
import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from ogl_beamforming_cuda_gb300.client import Beamformer, BeamformerError
from bf_cases import small_params, small_raw, oracle_for, check_volume

pytestmark = pytest.mark.gpu
SH = abi.SHADER
PIPE = [SH["Decode"], SH["Demodulate"], SH["DAS"]]
KAISER = (5.65, 5e6, 25e6, 32)
SPECS = [(256, 16, 16, (16, 3, 20), "HERCULES"), (512, 16, 32, (24, 1, 20), "FORCES"),
         (512, 8, 16, (12, 5, 16), "HERCULES"), (256, 16, 32, (20, 1, 24), "HERCULES"),
         (512, 16, 16, (16, 2, 16), "FORCES"), (256, 16, 16, (8, 8, 16), "HERCULES")]


def make_batch(seed0):
    import torch
    params, raws, rf, out = [], [], [], []
    for i, (S, C, T, pts, mode) in enumerate(SPECS):
        bp = small_params(S=S, C=C, T=T, points=pts, das=mode)
        raw = small_raw(bp, seed=seed0 + i, n_points=6, n_speckle=60)
        params.append(bp)
        raws.append(raw)
        rf.append(torch.from_numpy(raw).cuda())
        out.append(torch.zeros(2 * int(np.prod(pts)), dtype=torch.float32, device="cuda"))
    return params, raws, rf, out


def check_batch(bf, params, raws, out, what):
    for i, (bp, raw) in enumerate(zip(params, raws)):
        orc = oracle_for(bf, bp, PIPE, kaiser=KAISER)
        orc.interpolation = bf.interpolation if hasattr(bf, "interpolation") else -1
        ref = orc.compute(raw)
        check_volume(out[i].cpu().numpy(), ref["frame"], f"{what} acquisition {i} ({SPECS[i][4]} {SPECS[i][3]})")


@pytest.mark.parametrize("interp", (0, 1, 2))
def test_batch_matches_oracle_and_replays(interp):
    params, raws, rf, out = make_batch(20)
    bf = Beamformer().configure(params[0], PIPE, kaiser=KAISER, interpolation=interp)
    bf.interpolation = interp
    args = (params, [t.data_ptr() for t in rf], [t.numel() * 2 for t in rf], [t.data_ptr() for t in out])
    bf.beamform_batch(*args)
    check_batch(bf, params, raws, out, f"batch interp={interp}")
    tiles, ctas, ms = bf.batch_tuning()
    assert ctas > 0 and len(ms) >= 3 and np.all(ms > 0)
    # same buffers, new RF: the captured graph replays on the new contents
    raws2 = []
    for i, (bp, t) in enumerate(zip(params, rf)):
        r = small_raw(bp, seed=100 + i, n_points=6, n_speckle=60)
        t.copy_(__import__("torch").from_numpy(r).cuda())
        raws2.append(r)
    for o in out:
        o.zero_()
    l0 = bf.launches()
    bf.beamform_batch(*args)
    assert bf.launches() > l0
    check_batch(bf, params, raws2, out, f"replay interp={interp}")


def test_batch_rejects_coherency_weighting():
    params, raws, rf, out = make_batch(30)
    params[1].coherency_weighting = 1
    bf = Beamformer().configure(params[0], PIPE, kaiser=KAISER)
    with pytest.raises(BeamformerError):
        bf.beamform_batch(params, [t.data_ptr() for t in rf], [t.numel() * 2 for t in rf], [t.data_ptr() for t in out])
    assert bf.lib.beamformer_get_last_error() == abi.ERR["UNSUPPORTED"]


def test_batch_volume_tiles_staged(monkeypatch):
    """HERCULES tiles of the batch read the FP32 table staged in shared memory, as
    the single launch does: with OGL_BF_DAS_STAGED=require a tile that could not
    stage writes NaN. Two volumes with the 3D workload's voxel size (78 um x 78 um
    x 78 um) and a plane; the batch output equals the plain API's (which may split
    the receive channels into groups, so summation orders differ) to FP32 rounding."""
    import torch
    from ogl_beamforming_cuda_gb300 import synth
    monkeypatch.setenv("OGL_BF_DAS_STAGED", "require")
    lo, hi = np.array((-5e-3, -5e-3, 5e-3)), np.array((5e-3, 5e-3, 25e-3))
    params, rf, out, single = [], [], [], []
    for i, pts in enumerate(((32, 32, 64), (16, 32, 32), (48, 1, 64))):
        mid, half = (lo + hi) / 2, (hi - lo) / 2 * np.asarray(pts) / np.array((128, 128, 256))
        if pts[1] == 1:
            half[1] = 0.0
        bp = synth.make_parameters(samples=2048, channels=128, transmits=128, points=pts,
                                   extent=(tuple(mid - half), tuple(mid + half)), decimation=2, f_number=1.0,
                                   interpolate=1, frames=1, filter_length=64)
        raw = synth.acquisition(bp, 40 + i, n_points=30, n_speckle=300)
        params.append(bp)
        rf.append(torch.from_numpy(raw).cuda())
        out.append(torch.zeros(2 * int(np.prod(pts)), dtype=torch.float32, device="cuda"))
        one = Beamformer().configure(bp, PIPE, kaiser=synth.kaiser_spec(64))
        one.push(raw)
        one.synchronize()
        single.append(one.frame(0)[0].copy())
    bf = Beamformer().configure(params[0], PIPE, kaiser=synth.kaiser_spec(64))
    bf.beamform_batch(params, [t.data_ptr() for t in rf], [t.numel() * 2 for t in rf], [t.data_ptr() for t in out])
    for i, (o, ref) in enumerate(zip(out, single)):
        got = o.cpu().numpy()
        assert np.all(np.isfinite(got)), f"acquisition {i}: a tile did not stage"
        assert np.max(np.abs(got - ref.ravel())) <= 1e-5 * np.max(np.abs(ref)), f"acquisition {i}"

