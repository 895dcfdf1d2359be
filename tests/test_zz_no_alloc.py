"""beamformer_gb300_das_no_alloc: delay-and-sum for callers that cannot let the
library allocate device memory while they run (a loop that fixes its memory
budget at start-up, a host whose device memory belongs to its own allocator).
Its partial sums live in a static device array and its focal / sparse tables
travel as kernel parameters.

Through the C ABI, three calls in a row on the same library state:
  1, 2. a plane split into channel groups (partial sums in the static array),
        the same parameters twice;
  3.    other parameters, focal vectors and sparse elements (UHERCULES with a
        permuted sparse table and a cylindrical focal vector) on a volume whose
        default group count would overflow the static array, so the call takes
        fewer groups, down to one;
each checked against the oracle on the same channel data and against the
regular pipeline's frame, within the parity tests' volume tolerance. Collected
last on purpose, so a run that stops at the first failure has run the rest."""
import ctypes

import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from bf_cases import small_params, small_raw, check_volume

pytestmark = pytest.mark.gpu
SH = abi.SHADER
KAISER = (5.65, 5e6, 25e6, 32)
PIPE = [SH["Decode"], SH["Demodulate"], SH["DAS"]]


def das_stage_parameters(bp, pipeline):
    """Parameters as the DAS stage sees them after planning (the oracle's plan),
    and the float count of the channel data that stage reads."""
    from oracle import bf_oracle as O
    spec = [(0, KAISER[3], KAISER[2], KAISER[0], KAISER[1]), None, None, None]
    plan = O.plan(bp, pipeline, [0] * len(pipeline), abi.DATA_KIND["Int16"], spec)
    return plan.das, int(plan.rf_size) // 4


def regular_and_channel_data(bp, focal=None, sparse=None):
    """The regular pipeline's frame and its DAS input, through the C ABI."""
    from ogl_beamforming_cuda_gb300.client import Beamformer
    bf = Beamformer().configure(bp, PIPE, kaiser=KAISER, focal_vectors=focal, sparse_elements=sparse)
    bf.push(small_raw(bp))
    bf.synchronize()
    frame, dims = bf.frame(0)
    das, n = das_stage_parameters(bp, PIPE)
    return bf, frame, dims, np.ascontiguousarray(bf.channel_data()[:n]), das


def no_alloc(lib, das, focal, sparse, channel_dev, out_dev, stream):
    return lib.beamformer_gb300_das_no_alloc(
        ctypes.byref(das), focal.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
        sparse.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), ctypes.c_void_p(channel_dev.data_ptr()),
        channel_dev.numel() * 4, ctypes.c_void_p(out_dev.data_ptr()), stream)


def test_das_no_alloc_against_oracle_three_calls():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    from oracle import bf_oracle as O
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    # calls 1 and 2: a 32 x 1 x 32 plane, split into channel groups
    bp = small_params(S=512, C=32, T=32, points=(32, 1, 32))
    bf, regular, dims, channel, das = regular_and_channel_data(bp)
    oracle = O.das(das, channel, dims, bf.sparse, bf.focal, fast=True)
    channel_dev = torch.from_numpy(channel).cuda()
    out = torch.empty(2 * int(np.prod(dims)), dtype=torch.float32, device="cuda")
    for call in range(2):
        out.fill_(float("nan"))
        ok = no_alloc(bf.lib, das, bf.focal, bf.sparse, channel_dev, out, stream)
        assert ok == 1, bf.lib.beamformer_get_last_error_string()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        check_volume(got, oracle, f"no-alloc DAS against the oracle, call {call + 1}")
        check_volume(got, regular, f"no-alloc DAS against the regular pipeline, call {call + 1}")

    # call 3: other parameters and tables; 128 x 15 x 128 = 245760 voxels, so
    # the static array holds one group's partial sums at most
    bp3 = small_params(S=512, C=32, T=32, points=(128, 15, 128), das="UHERCULES")
    rng = np.random.default_rng(21)
    focal3 = np.zeros(512, np.float32)
    focal3[0], focal3[1] = 4.0, -4.0e-3                     # 4 degrees, virtual source 4 mm behind the array
    focal3[2::2] = rng.uniform(-5, 5, 255)
    focal3[3::2] = np.inf
    sparse3 = np.concatenate([rng.permutation(32), np.arange(32, 256)]).astype(np.int16)
    bf3, regular3, dims3, channel3, das3 = regular_and_channel_data(bp3, focal=focal3, sparse=sparse3)
    oracle3 = O.das(das3, channel3, dims3, sparse3, focal3, fast=True)
    channel3_dev = torch.from_numpy(channel3).cuda()
    out3 = torch.full((2 * int(np.prod(dims3)),), float("nan"), dtype=torch.float32, device="cuda")
    ok = no_alloc(bf3.lib, das3, focal3, sparse3, channel3_dev, out3, stream)
    assert ok == 1, bf3.lib.beamformer_get_last_error_string()
    torch.cuda.synchronize()
    got3 = out3.cpu().numpy()
    assert np.any(oracle3 != 0) and np.any(got3 != 0)
    check_volume(got3, oracle3, "no-alloc DAS against the oracle, call 3 (one channel group)")
    check_volume(got3, regular3, "no-alloc DAS against the regular pipeline, call 3")


def test_das_no_alloc_rejects_missing_buffers(lib):
    torch = pytest.importorskip("torch")
    bp = small_params(S=512, C=32, T=32, points=(32, 1, 32))
    das, _ = das_stage_parameters(bp, PIPE)
    out = torch.zeros(2 * 32 * 32, dtype=torch.float32, device="cuda")
    ok = lib.beamformer_gb300_das_no_alloc(ctypes.byref(das), None, None, None, 0, ctypes.c_void_p(out.data_ptr()),
                                           None)
    assert ok == 0
    assert lib.beamformer_get_last_error() == abi.ERR["INVALID_ACCESS"]
    assert not torch.any(out)
