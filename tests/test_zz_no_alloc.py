"""beamformer_gb300_das_no_alloc: delay-and-sum for callers that cannot let the
library allocate device memory (its partial sums live in a static device array).

Checks, through the C ABI, that two calls in a row give the volume the regular
pipeline entry point gives for the same channel data (within the volume
tolerance of the parity tests), and that a volume needing more partial-sum
space than the static array holds is rejected. Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from ogl_beamforming_cuda_gb300 import abi
from bf_cases import small_params, small_raw, check_volume

pytestmark = pytest.mark.gpu
SH = abi.SHADER
KAISER = (5.65, 5e6, 25e6, 32)


def das_stage_parameters(bp, pipeline):
    """Parameters as the DAS stage sees them after planning (the oracle's plan)."""
    from oracle import bf_oracle as O
    spec = [(0, KAISER[3], KAISER[2], KAISER[0], KAISER[1]), None, None, None]
    return O.plan(bp, pipeline, [0] * len(pipeline), abi.DATA_KIND["Int16"], spec).das


def test_das_no_alloc_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    from ogl_beamforming_cuda_gb300.client import Beamformer
    bp = small_params(S=512, C=32, T=32, points=(32, 1, 32))     # a plane: split into channel groups
    pipe = [SH["Decode"], SH["Demodulate"], SH["DAS"]]
    bf = Beamformer().configure(bp, pipe, kaiser=KAISER)
    bf.push(small_raw(bp))
    bf.synchronize()
    expected, dims = bf.frame(0)
    channel = torch.from_numpy(bf.channel_data()).cuda()
    das = das_stage_parameters(bp, pipe)
    out = torch.empty(2 * int(np.prod(dims)), dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        out.fill_(float("nan"))
        ok = bf.lib.beamformer_gb300_das_no_alloc(
            ctypes.byref(das), bf.focal.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            bf.sparse.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), ctypes.c_void_p(channel.data_ptr()),
            channel.numel() * 4, ctypes.c_void_p(out.data_ptr()), stream)
        assert ok == 1, bf.lib.beamformer_get_last_error_string()
        torch.cuda.synchronize()
        check_volume(out.cpu().numpy(), expected, f"no-alloc DAS, call {call + 1}")


def test_das_no_alloc_rejects_partial_sums_beyond_capacity(lib):
    torch = pytest.importorskip("torch")
    bp = small_params(S=512, C=32, T=32, points=(128, 15, 128))   # two channel groups x 245760 voxels
    das = das_stage_parameters(bp, [SH["Decode"], SH["Demodulate"], SH["DAS"]])
    channel = torch.zeros(2 * 128 * 32 * 32, dtype=torch.float32, device="cuda")
    out = torch.zeros(2 * 128 * 15 * 128, dtype=torch.float32, device="cuda")
    ok = lib.beamformer_gb300_das_no_alloc(ctypes.byref(das), None, None, ctypes.c_void_p(channel.data_ptr()),
                                           channel.numel() * 4, ctypes.c_void_p(out.data_ptr()), None)
    assert ok == 0
    assert lib.beamformer_get_last_error() == abi.ERR["BUFFER_OVERFLOW"]
    assert not torch.any(out)
