"""Shared cases for the parity tests: one acquisition pushed through the C-ABI
library and through the CPU oracle with identical state."""
import numpy as np

from ogl_beamforming_cuda_gb300 import abi, synth
from ogl_beamforming_cuda_gb300.client import Beamformer
from oracle.bf_oracle import OraclePipeline

NRMSE_DB = -80.0        # volume tolerance (float stages)
MAXABS_FRAC = 1e-4      # max |err| relative to the reference peak


def small_params(S=512, C=32, T=32, points=(24, 1, 20), D=2, das="HERCULES", interp=0, f_number=1.0,
                 frames=1, coherency=0):
    bp = synth.make_parameters(samples=S, channels=C, transmits=T, points=points,
                               extent=((-1.5e-3, -1.5e-3, 1.0e-3), (1.5e-3, 1.5e-3, 3.5e-3)),
                               decimation=D, f_number=f_number, interpolate=interp, das_id=das, frames=frames)
    bp.coherency_weighting = coherency
    return bp


def small_raw(bp, seed=3, n_points=8, n_speckle=40):
    pos, amp = synth.scatterers(seed, n_points, n_speckle, box=((-1.5e-3, -1.5e-3, 1.2e-3), (1.5e-3, 1.5e-3, 3.3e-3)))
    return synth.encode_and_quantise(synth.decoded_traces(bp, pos, amp), seed).numpy()


def oracle_for(bf, bp, pipeline, kaiser=None, data_kind=abi.DATA_KIND["Int16"]):
    """An oracle holding the same state the client pushed to the library."""
    orc = OraclePipeline()
    orc.bp = bp
    orc.shaders = list(pipeline)
    orc.data_kind = data_kind
    if kaiser is not None:
        orc.create_kaiser(kaiser[0], kaiser[1], kaiser[2], kaiser[3], 0)
    orc.chmap, orc.focal, orc.sparse = bf.chmap, bf.focal, bf.sparse
    return orc


def run_both(bp, pipeline, raw, data_kind=abi.DATA_KIND["Int16"], kaiser=(5.65, 5e6, 25e6, 32), matched=None,
             chmap=None, focal=None, sparse=None, slots=None, interpolation=-1, want_frames=("frame",)):
    bf = Beamformer().configure(bp, pipeline, data_kind=data_kind, kaiser=kaiser, matched=matched,
                                channel_mapping=chmap, focal_vectors=focal, sparse_elements=sparse,
                                stage_slots=slots, interpolation=interpolation)
    orc = OraclePipeline()
    orc.bp = bp
    orc.shaders = list(pipeline)
    orc.data_kind = data_kind
    if kaiser is not None:
        orc.create_kaiser(kaiser[0], kaiser[1], kaiser[2], kaiser[3], 0)
    if matched is not None:
        orc.create_matched(*matched)
    orc.chmap = bf.chmap
    orc.focal = bf.focal
    orc.sparse = bf.sparse
    orc.interpolation = interpolation
    for st, sl in (slots or {}).items():
        orc.slots[st % 16] = sl
    bf.push(raw)
    bf.synchronize()
    ref = orc.compute(raw)
    return bf, ref


def check_volume(vol, ref, what=""):
    from conftest import nrmse_db
    db = nrmse_db(vol, ref)
    peak = float(np.max(np.abs(ref)))
    assert db <= NRMSE_DB, f"{what}: NRMSE {db:.1f} dB > {NRMSE_DB} dB"
    assert float(np.max(np.abs(np.asarray(vol) - ref))) <= MAXABS_FRAC * max(peak, 1e-30), f"{what}: max-abs"
    return db


def fp64_front_end(ref, kaiser, data_channels):
    """FP64 restatement of the Demodulate stage on the oracle's (exact) decoded
    samples: complex channel data of the stage's output region, float64 pairs."""
    import ctypes
    import oracle.bf_oracle as O
    p = ref["plan"]
    dec = ref["stages"][0][1].astype(np.float64)
    out = np.zeros_like(dec)
    taps = O.kaiser_f64(kaiser[1], kaiser[2], kaiser[0], kaiser[3])
    O.lib().bfo_filter_f64(ctypes.byref(p.demod), abi.SHADER["DemodulateFloat"], O._ptr(dec), dec.size, O._ptr(out),
                           out.size, O._arr(taps, ctypes.c_double), kaiser[3], p.demod_dispatch, O.threads())
    n = 2 * int(p.demod.output_channel_stride) * data_channels
    return out, n


def nrmse(a, b):
    from conftest import nrmse_db
    return nrmse_db(a, b)
