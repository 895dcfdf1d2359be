"""The CPU oracle against outputs of the reference itself (tests/golden, made by
tests/golden/make_golden.py from the reference's math.c and compute shaders).
Runs everywhere; needs no GPU and no reference checkout."""
import ctypes
import os

import numpy as np
import pytest

from oracle import bf_oracle as O
from ogl_beamforming_cuda_gb300.abi import BeamformerParameters, SHADER, DATA_KIND

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.npz"))


def params(blob):
    bp = BeamformerParameters()
    ctypes.memmove(ctypes.byref(bp), blob.tobytes(), ctypes.sizeof(bp))
    return bp


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128])
def test_sylvester_matches_reference(n):
    assert np.array_equal(O.hadamard(n).ravel(), G[f"hadamard_{n}"])


def scramble_x86(h):
    """What the reference's Kronecker product writes on x86-64 for a 1 x 1 Sylvester
    factor: its store macro advances by 4-int vectors, so block j of row i lands at
    i*n + 16*j/4 (math.c fill_kronecker_sub_matrix with intrinsics.c store_i32x4).
    The 1 x 1 Sylvester factor (value 1) sits right after the matrix in the arena."""
    n = h.shape[0]
    out = np.zeros(n * n + 64, np.int32)
    out[n * n] = 1
    for i in range(n):
        for j in range(0, n, 4):
            o = i * n + 4 * j
            out[o:o + 4] = h[i, j:j + 4]
    return out


@pytest.mark.parametrize("n", [12, 20])
def test_paley_orders_match_reference_tables(n):
    """Our bordered Paley construction reproduces the reference's 12x12 / 20x20
    tables: applying the reference's x86 store pattern to it gives exactly what
    the reference computed."""
    assert np.array_equal(scramble_x86(O.hadamard(n)), G[f"hadamard_{n}"])


@pytest.mark.parametrize("L", [16, 36, 64, 128])
def test_kaiser_matches_reference(L):
    ours = O.kaiser(5e6, 25e6, 5.65, L)
    ref = G[f"kaiser_{L}"]
    assert np.max(np.abs(ours - ref)) <= 2e-7 * np.max(np.abs(ref))


def test_matched_and_i0_match_reference():
    ours = O.matched(12.5e6, 12.5e6, 50e6, 20)
    assert np.max(np.abs(ours - G["matched_20"])) <= 1e-6 * np.max(np.abs(G["matched_20"]))
    for x, y in zip(G["i0_x"], G["i0_y"]):
        assert abs(O.lib().bfo_i0(float(x)) - y) <= 1e-14 * abs(y)


@pytest.mark.parametrize("name", ["hercules_plane", "hercules_vol", "forces"])
def test_voxel_transform_matches_reference(name):
    bp = params(G[f"voxel_{name}_params"])
    assert np.allclose(O.voxel_transform(bp), G[f"voxel_{name}"], rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("label", ["plain", "tofloat"])
def test_decode_matches_reference(label):
    bp = params(G[f"decode_{label}_params"])
    shaders = [SHADER["Decode"]] if label == "plain" else [SHADER["Decode"], SHADER["Demodulate"]]
    p = O.plan(bp, shaders, [0] * len(shaders), DATA_KIND["Int16"], [(0, 8, 25e6, 5.65, 5e6), None, None, None])
    raw, chmap = G["decode_raw"], G["decode_chmap"]
    T = int(bp.dec_data_dim[2])
    H = O.hadamard(T).astype(np.int32).ravel()
    out = np.zeros_like(G[f"decode_{label}_out"])
    O.lib().bfo_decode(ctypes.byref(p.decode), p.shaders[0], 1, 0, O._ptr(raw), raw.nbytes, O._ptr(out), out.nbytes,
                       O._arr(H, ctypes.c_int32), T, O._arr(chmap, ctypes.c_int16), p.decode_dispatch, 2)
    assert np.array_equal(out.view(np.uint32), G[f"decode_{label}_out"].view(np.uint32))
    if label == "tofloat":
        dem = np.zeros_like(out)
        taps = G["demod_taps"]
        O.lib().bfo_filter(ctypes.byref(p.demod), p.shaders[1], O._ptr(out), out.nbytes, O._ptr(dem), dem.nbytes,
                           O._arr(taps, ctypes.c_float), 8, O._arr(chmap, ctypes.c_int16), p.demod_dispatch, 2)
        assert np.array_equal(dem.view(np.uint32), G["demod_out"].view(np.uint32))


@pytest.mark.parametrize("label", ["herc_nearest", "herc_cubic", "forces_cubic"])
def test_das_matches_reference(label):
    bp = params(G[f"das_{label}_params"])
    dims = [int(v) for v in bp.output_points[:3]]
    focal = np.zeros(512, np.float32)
    focal[1::2] = np.inf
    frame = O.das(bp, G[f"das_{label}_rf"], dims, np.arange(256, dtype=np.int16), focal, fast=True)
    assert np.array_equal(frame.view(np.uint32), G[f"das_{label}_out"].view(np.uint32))


def test_sum_and_min_max_match_reference():
    dims = (64, 2, 32)
    frames = [f.copy() for f in G["sum_in"]]
    assert np.array_equal(O.sum_frames(frames, np.float32(1 / 3), dims), G["sum_out"])
    assert np.array_equal(O.min_max(frames[0], dims), G["minmax_out"], equal_nan=True)
