"""Seeded synthetic acquisitions for the row-column (RCA) array workloads.

There is no public dataset for this path; these generators stand in for it with
the shapes, sizes and value distributions of the benchmark configurations:
a 128 + 128 element row-column array (pitch 0.1 mm), HERCULES transmits encoded
with a Sylvester Hadamard matrix, fs 50 MHz, fc 12.5 MHz, c 1540 m/s, int16 RF
laid out [channel][transmit][sample] (rf_raw_dim = {samples * transmits,
channels}).

Echo model: every decoded (transmit t, receive r) trace holds, for each
scatterer p, a Gaussian-windowed two-cycle sinusoid at fc centred at
tau = (d_tx(p) + |q - e_{r,t}|) / c, with d_tx the plane-wave distance and
e_{r,t} = (r * pitch, t * pitch, 0) the HERCULES virtual element, i.e. the delay
model of das.glsl:178-215 so the DAS image focuses. The traces are summed,
Hadamard-encoded across transmits (raw_i = sum_t H[i][t] x_t), given
N(0, (1% of peak)^2) noise and quantised to int16 at about half of full scale.
"""
import math

import numpy as np
import torch

from .abi import BeamformerParameters, SHADER, DATA_KIND, DAS_KIND

FS = 50e6
FC = 12.5e6
C_SOUND = 1540.0
PITCH = 1e-4


def sylvester(n):
    h = np.ones((1, 1), np.int64)
    while h.shape[0] < n:
        h = np.block([[h, h], [h, -h]])
    return h


def make_parameters(samples=2048, channels=128, transmits=128, points=(128, 1, 128), extent=None,
                    decimation=2, f_number=1.0, interpolate=0, das_id="HERCULES", frames=1, filter_length=64):
    """BeamformerParameters for a HERCULES (or FORCES) acquisition of the RCA array."""
    bp = BeamformerParameters()
    X = np.eye(4, dtype=np.float32)
    X[3, 0] = (channels - 1) / 2 * PITCH      # centre the array on the world origin
    X[3, 1] = (transmits - 1) / 2 * PITCH
    bp.xdc_transform[:] = X.ravel().tolist()
    bp.dec_data_dim[:] = [samples, channels, transmits, 1]
    bp.xdc_element_pitch[:] = [PITCH, PITCH]
    bp.rf_raw_dim[:] = [samples * transmits, channels]
    bp.transmit_mode = 1
    bp.decode = 1
    bp.das_shader_id = DAS_KIND[das_id]
    bp.time_offset = 0.0
    lo, hi = extent if extent is not None else ((-5e-3, -5e-3, 5e-3), (5e-3, 5e-3, 25e-3))
    bp.output_min_coordinate[:] = [lo[0], lo[1], lo[2], 0]
    bp.output_max_coordinate[:] = [hi[0], hi[1], hi[2], 0]
    bp.output_points[:] = [points[0], points[1], points[2], frames]
    bp.sampling_frequency = FS
    bp.center_frequency = FC
    bp.speed_of_sound = C_SOUND
    bp.off_axis_pos = 0.0
    bp.beamform_plane = 0
    bp.f_number = f_number
    bp.interpolate = interpolate
    bp.coherency_weighting = 0
    bp.decimation_rate = decimation
    return bp


def default_pipeline(sum_and_minmax=False):
    st = [SHADER["Decode"], SHADER["Demodulate"], SHADER["DAS"]]
    if sum_and_minmax:
        st += [SHADER["Sum"], SHADER["MinMax"]]
    return st


def kaiser_spec(filter_length=64):
    """(beta, cutoff, sampling_frequency, length): low-pass for the decimated baseband."""
    return (5.65, 5e6, FS / 2, filter_length)


def scatterers(seed, n_points, n_speckle=0, box=((-5e-3, -5e-3, 5e-3), (5e-3, 5e-3, 25e-3)), in_plane=0.5):
    """Point targets (unit amplitude) plus speckle (Gaussian amplitudes), world coordinates [m].

    A fraction `in_plane` of the points lies on the x = 0 plane, the plane a 2D
    HERCULES output (beamform_plane 0, one y point) images."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(box[0]), np.asarray(box[1])
    pts = lo + (hi - lo) * rng.random((n_points, 3))
    pts[: int(round(in_plane * n_points)), 0] = 0.0
    amp = np.ones(n_points)
    if n_speckle:
        sp = lo + (hi - lo) * rng.random((n_speckle, 3))
        pts = np.concatenate([pts, sp])
        amp = np.concatenate([amp, 0.1 * rng.standard_normal(n_speckle)])
    return pts.astype(np.float64), amp.astype(np.float64)


def decoded_traces(bp, pos, amp, device="cpu", batch=256):
    """Decoded RF x[t][r][n] (float32 torch tensor) for scatterers at pos (world)."""
    S, C, T = int(bp.dec_data_dim[0]), int(bp.dec_data_dim[1]), int(bp.dec_data_dim[2])
    fs, fc, c = float(bp.sampling_frequency), float(bp.center_frequency), float(bp.speed_of_sound)
    px, py = float(bp.xdc_element_pitch[0]), float(bp.xdc_element_pitch[1])
    X = torch.tensor(np.asarray(bp.xdc_transform[:], np.float64).reshape(4, 4), device=device)  # column-major rows
    dev = torch.device(device)
    x = torch.zeros(T * C * S, dtype=torch.float32, device=dev)
    rx = torch.arange(C, device=dev, dtype=torch.float64) * px
    tx = torch.arange(T, device=dev, dtype=torch.float64) * py
    sigma = 1.0 / fc / 2.5                  # two-cycle Gaussian envelope
    half = int(math.ceil(3 * sigma * fs)) + 1
    k = torch.arange(-half, half + 1, device=dev, dtype=torch.float64)
    P = torch.tensor(pos, device=dev)
    A = torch.tensor(amp, device=dev)
    for b in range(0, P.shape[0], batch):
        p = P[b:b + batch]
        a = A[b:b + batch]
        q = p @ X[:3, :3] + X[3, :3]        # xdc = M * (p, 1), M column-major
        dtx = p[:, 2]                        # plane wave at 0 degrees, transmit rows
        dx = q[:, 0, None, None] - rx[None, None, :]
        dy = q[:, 1, None, None] - tx[None, :, None]
        d = torch.sqrt(dx * dx + dy * dy + q[:, 2, None, None] ** 2)
        tau = (dtx[:, None, None] + d) / c                        # [P, T, C]
        n0 = torch.floor(tau * fs)
        n = n0[..., None] + k                                      # [P, T, C, K]
        tt = n / fs - tau[..., None]
        val = a[:, None, None, None] * torch.cos(2 * math.pi * fc * tt) * torch.exp(-(tt / sigma) ** 2)
        ok = (n >= 0) & (n < S)
        row = (torch.arange(T, device=dev)[:, None] * C + torch.arange(C, device=dev)[None, :]) * S
        idx = row[None, :, :, None] + n.long()
        x.index_put_((idx[ok],), val[ok].float(), accumulate=True)
    return x.view(T, C, S)


def encode_and_quantise(x, seed, noise=0.01):
    """Hadamard-encode decoded traces x[t][r][n], add noise, quantise: int16 raw[r][t][n]."""
    T = x.shape[0]
    H = torch.tensor(sylvester(T), dtype=torch.float64, device=x.device)
    raw = (H @ x.double().reshape(T, -1)).reshape(x.shape)
    g = torch.Generator(device=x.device).manual_seed(int(seed) + 1)
    peak = raw.abs().max().clamp_min(1e-30)
    raw = raw + noise * peak * torch.randn(raw.shape, generator=g, device=x.device, dtype=torch.float64)
    scale = 0.5 * 32767.0 / raw.abs().max().clamp_min(1e-30)
    q = torch.round(raw * scale).clamp(-32768, 32767).to(torch.int16)
    return q.permute(1, 0, 2).contiguous()


def acquisition(bp, seed, n_points=20, n_speckle=0, device="cpu"):
    """int16 raw RF (numpy, [channel][transmit][sample]) for one seeded frame."""
    pos, amp = scatterers(seed, n_points, n_speckle)
    x = decoded_traces(bp, pos, amp, device=device)
    return encode_and_quantise(x, seed).cpu().numpy()


BATCH_GRIDS = ((64, 1, 64), (128, 1, 128), (64, 64, 128), (128, 128, 256))


def batch_workload(seed, count=32, transmits=(32, 64, 128), samples=(1024, 2048, 4096), grids=BATCH_GRIDS,
                   modes=("HERCULES", "FORCES"), interpolate=1, filter_length=64):
    """Seeded mixed batch: per acquisition a transmit count, sample count, output
    grid and DAS mode drawn uniformly from the given sets (128 receive channels)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        T = int(rng.choice(transmits))
        S = int(rng.choice(samples))
        grid = tuple(grids[int(rng.integers(len(grids)))])
        mode = str(rng.choice(modes))
        out.append(make_parameters(samples=S, channels=128, transmits=T, points=grid, decimation=2,
                                   interpolate=interpolate, das_id=mode, filter_length=filter_length))
    return out
