"""The learned variant: DAS over every 4th receive channel followed by a small
3D convolutional U-Net that restores the full-aperture volume. No counterpart in
the reference.

Network (channels-first volumes, the complex DAS output as 2 real channels):
  enc1  conv 2->16, conv 16->16 (ReLU)                  full resolution
  enc2  2x mean pool, conv 16->32, conv 32->32 (ReLU)    1/2
  mid   2x mean pool, conv 32->64, conv 64->64 (ReLU)    1/4
  dec2  2x upsample, concat enc2, conv 96->32, conv 32->32 (ReLU)
  dec1  2x upsample, concat enc1, conv 48->16, conv 16->16 (ReLU)
  out   conv 16->2, plus the input (residual)
All convolutions are 3x3x3. Weights and activations are stored in BF16, gradients
and the master weights in FP32, every product is accumulated in FP32. Forward,
backward (input and weight gradients) and the Adam step run on the library's own
kernels (include/bf_unet.h); torch only holds the device memory.

Input and target are normalised per volume by the RMS of the input, which is the
subsampled DAS scaled by the aperture ratio (128 / 32 = 4).
"""
import ctypes
import math

import numpy as np
import torch

from . import abi, synth

F32, BF16 = 0, 1
LAYERS = (("e1a", 2, 16, True), ("e1b", 16, 16, True), ("e2a", 16, 32, True), ("e2b", 32, 32, True),
          ("m1", 32, 64, True), ("m2", 64, 64, True), ("d2a", 96, 32, True), ("d2b", 32, 32, True),
          ("d1a", 48, 16, True), ("d1b", 16, 16, True), ("out", 16, 2, False))
RX_STEP = 4

# Weight file: a plain versioned little-endian binary (no pickle, readable from C):
# 8-byte magic, u32 version, u32 layer count, then per layer in LAYERS order a
# 16-byte NUL-padded name, u32 cin, u32 cout, f32 w[cout][cin][27], f32 b[cout].
WEIGHTS_MAGIC = b"BFUNETW\0"
WEIGHTS_VERSION = 1


def save_weights(path, state):
    """Write state {layer: (w, b)} (tensors or arrays; every layer of LAYERS)."""
    import struct
    with open(path, "wb") as f:
        f.write(WEIGHTS_MAGIC + struct.pack("<II", WEIGHTS_VERSION, len(LAYERS)))
        for name, cin, cout, _ in LAYERS:
            w, b = state[name]
            w = np.asarray(w.detach().cpu() if hasattr(w, "detach") else w, dtype="<f4").reshape(-1)
            b = np.asarray(b.detach().cpu() if hasattr(b, "detach") else b, dtype="<f4").reshape(-1)
            if w.size != cout * cin * 27 or b.size != cout:
                raise ValueError(f"layer {name}: {w.size} weights / {b.size} biases, expected "
                                 f"{cout * cin * 27} / {cout}")
            f.write(name.encode().ljust(16, b"\0") + struct.pack("<II", cin, cout))
            f.write(w.tobytes())
            f.write(b.tobytes())


def load_weights(path):
    """Read a weight file into {layer: (w float32 [cout*cin*27], b float32 [cout])};
    ValueError for another magic, version, layer table or a short file."""
    import struct
    raw = open(path, "rb").read()
    if raw[:8] != WEIGHTS_MAGIC or len(raw) < 16:
        raise ValueError(f"{path}: not a U-Net weight file")
    version, count = struct.unpack_from("<II", raw, 8)
    if version != WEIGHTS_VERSION or count != len(LAYERS):
        raise ValueError(f"{path}: version {version} with {count} layers, expected version "
                         f"{WEIGHTS_VERSION} with {len(LAYERS)}")
    off, state = 16, {}
    for name, cin, cout, _ in LAYERS:
        if off + 24 > len(raw):
            raise ValueError(f"{path}: truncated at layer {name}")
        fname = raw[off:off + 16].rstrip(b"\0").decode()
        fcin, fcout = struct.unpack_from("<II", raw, off + 16)
        if (fname, fcin, fcout) != (name, cin, cout):
            raise ValueError(f"{path}: layer {fname} ({fcin} -> {fcout}), expected {name} ({cin} -> {cout})")
        off += 24
        nw, nb = cout * cin * 27, cout
        if off + 4 * (nw + nb) > len(raw):
            raise ValueError(f"{path}: truncated at layer {name}")
        w = np.frombuffer(raw, "<f4", nw, off).astype(np.float32)
        b = np.frombuffer(raw, "<f4", nb, off + 4 * nw).astype(np.float32)
        off += 4 * (nw + nb)
        state[name] = (w, b)
    if off != len(raw):
        raise ValueError(f"{path}: {len(raw) - off} trailing bytes")
    return state


def _bind(lib):
    vp, i32, i64, f32, u32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_uint32
    dims = ctypes.POINTER(ctypes.c_int32)
    sig = {
        "bf_unet_conv3d": [vp, i32, i32, vp, vp, vp, vp, i32, i32, dims, i32, vp],
        "bf_unet_conv3d_grad_input": [vp, i32, vp, vp, i32, dims, vp, vp],
        "bf_unet_conv3d_grad_weight": [vp, i32, vp, i32, i32, dims, vp, vp, vp],
        "bf_unet_relu_grad": [vp, vp, i64, vp],
        "bf_unet_avgpool2": [vp, i32, vp, i32, i32, dims, vp],
        "bf_unet_avgpool2_grad": [vp, vp, i32, dims, i32, vp],
        "bf_unet_upsample2": [vp, i32, vp, i32, i32, dims, vp],
        "bf_unet_upsample2_grad": [vp, vp, i32, dims, vp],
        "bf_unet_mse": [vp, vp, vp, vp, i64, vp],
        "bf_unet_adam": [vp, vp, vp, vp, vp, i64, f32, f32, f32, f32, i32, vp],
        "bf_unet_convert": [vp, i32, vp, i32, i64, f32, vp],
        "bf_unet_ema": [vp, vp, vp, i64, f32, vp],
        "bf_synth_traces": [vp, vp, i32, vp, i32, i32, i32, f32, f32, f32, f32, f32, vp],
        "bf_unet_tc_errors": [vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = u32
    return lib


class Kernels:
    """The bf_unet_* entry points of the library on one CUDA stream."""

    def __init__(self, lib=None, stream=None):
        self.lib = _bind(lib or abi.load())
        self.stream = stream if stream is not None else torch.cuda.current_stream().cuda_stream

    @staticmethod
    def _d(dims):
        return (ctypes.c_int32 * 3)(*dims)

    @staticmethod
    def _p(t):
        return ctypes.c_void_p(t.data_ptr()) if t is not None else None

    def _ok(self, r, what):
        if not r:
            raise RuntimeError(f"{what} failed")

    def conv(self, x, cin, w16, b, out, cout, dims, relu, residual=None):
        tx = BF16 if x.dtype == torch.bfloat16 else F32
        to = BF16 if out.dtype == torch.bfloat16 else F32
        self._ok(self.lib.bf_unet_conv3d(self._p(x), tx, cin, self._p(w16), self._p(b), self._p(residual), self._p(out),
                                         to, cout, self._d(dims), int(relu), self.stream), "conv3d")

    def conv_grad_input(self, g, cout, w16, gin, cin, dims, scratch):
        self._ok(self.lib.bf_unet_conv3d_grad_input(self._p(g), cout, self._p(w16), self._p(gin), cin, self._d(dims),
                                                    self._p(scratch), self.stream), "conv3d_grad_input")

    def conv_grad_weight(self, g, cout, x, cin, dims, gw, gb):
        tx = BF16 if x.dtype == torch.bfloat16 else F32
        self._ok(self.lib.bf_unet_conv3d_grad_weight(self._p(g), cout, self._p(x), tx, cin, self._d(dims), self._p(gw),
                                                     self._p(gb), self.stream), "conv3d_grad_weight")

    def relu_grad(self, g, act):
        self._ok(self.lib.bf_unet_relu_grad(self._p(g), self._p(act), g.numel(), self.stream), "relu_grad")

    def pool(self, x, out, c, dims_in):
        tx = BF16 if x.dtype == torch.bfloat16 else F32
        to = BF16 if out.dtype == torch.bfloat16 else F32
        self._ok(self.lib.bf_unet_avgpool2(self._p(x), tx, self._p(out), to, c, self._d(dims_in), self.stream), "pool")

    def pool_grad(self, go, gi, c, dims_in, accumulate):
        self._ok(self.lib.bf_unet_avgpool2_grad(self._p(go), self._p(gi), c, self._d(dims_in), int(accumulate),
                                                self.stream), "pool_grad")

    def up(self, x, out, c, dims_out):
        tx = BF16 if x.dtype == torch.bfloat16 else F32
        to = BF16 if out.dtype == torch.bfloat16 else F32
        self._ok(self.lib.bf_unet_upsample2(self._p(x), tx, self._p(out), to, c, self._d(dims_out), self.stream), "up")

    def up_grad(self, go, gi, c, dims_out):
        self._ok(self.lib.bf_unet_upsample2_grad(self._p(go), self._p(gi), c, self._d(dims_out), self.stream), "up_grad")

    def mse(self, y, t, g, loss):
        self._ok(self.lib.bf_unet_mse(self._p(y), self._p(t), self._p(g), self._p(loss), y.numel(), self.stream), "mse")

    def adam(self, w, g, m, v, w16, lr, step, b1=0.9, b2=0.999, eps=1e-8):
        self._ok(self.lib.bf_unet_adam(self._p(w), self._p(g), self._p(m), self._p(v), self._p(w16), w.numel(), lr, b1,
                                       b2, eps, step, self.stream), "adam")

    def ema(self, e, w, e16, decay):
        self._ok(self.lib.bf_unet_ema(self._p(e), self._p(w), self._p(e16), w.numel(), decay, self.stream), "ema")

    def convert(self, x, y, scale=1.0):
        tx = BF16 if x.dtype == torch.bfloat16 else F32
        ty = BF16 if y.dtype == torch.bfloat16 else F32
        self._ok(self.lib.bf_unet_convert(self._p(x), tx, self._p(y), ty, x.numel(), scale, self.stream), "convert")


class UNet:
    """Parameters (FP32 master, BF16 copy, Adam moments) and the forward and
    backward passes of the network, on the library's kernels."""

    def __init__(self, device="cuda", seed=0, kernels=None):
        self.k = kernels or Kernels()
        self.device = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.p = {}
        for name, cin, cout, relu in LAYERS:
            w = torch.randn(cout * cin * 27, generator=g, dtype=torch.float32) * math.sqrt(2.0 / (cin * 27))
            if name == "out":
                w *= 0.05                      # start close to the identity of the residual path
            w = w.to(self.device)
            L = dict(cin=cin, cout=cout, relu=relu, w=w, w16=torch.empty(w.numel(), dtype=torch.bfloat16, device=self.device),
                     b=torch.zeros(cout, device=self.device), gw=torch.zeros_like(w), gb=torch.zeros(cout, device=self.device),
                     mw=torch.zeros_like(w), vw=torch.zeros_like(w), mb=torch.zeros(cout, device=self.device),
                     vb=torch.zeros(cout, device=self.device),
                     b16=torch.empty(cout, dtype=torch.bfloat16, device=self.device))
            self.k.convert(L["w"], L["w16"])
            self.p[name] = L
        self._reset_average()
        self.scratch = torch.empty(max(L["cin"] * L["cout"] * 27 for L in self.p.values()), dtype=torch.bfloat16,
                                   device=self.device)
        self.step = 0
        self.acts = None

    def _reset_average(self):
        """the moving average of the weights restarts from the current weights"""
        for L in self.p.values():
            L["we"], L["be"] = L["w"].clone(), L["b"].clone()
            L["w16e"] = L["w16"].clone()

    def average(self, decay):
        """one step of the exponential moving average of the weights (bf_unet_ema)"""
        for L in self.p.values():
            self.k.ema(L["we"], L["w"], L["w16e"], decay)
            self.k.ema(L["be"], L["b"], None, decay)

    def _swap_average(self):
        for L in self.p.values():
            L["w16"], L["w16e"] = L["w16e"], L["w16"]
            L["b"], L["be"] = L["be"], L["b"]
            L["w"], L["we"] = L["we"], L["w"]

    def averaged(self):
        """context in which forward() (and state()) use the averaged weights"""
        net = self

        class _Ctx:
            def __enter__(self):
                net._swap_average()
                return net

            def __exit__(self, *exc):
                net._swap_average()
                return False
        return _Ctx()

    def state(self):
        return {n: (L["w"].clone(), L["b"].clone()) for n, L in self.p.items()}

    def load(self, state):
        for n, (w, b) in state.items():
            self.p[n]["w"].copy_(torch.as_tensor(w))
            self.p[n]["b"].copy_(torch.as_tensor(b))
            self.k.convert(self.p[n]["w"], self.p[n]["w16"])
        self._reset_average()

    def save_file(self, path):
        save_weights(path, self.state())

    def load_file(self, path):
        self.load(load_weights(path))

    def _buf(self, c, dims, dtype=torch.bfloat16):
        return torch.empty((c, dims[2], dims[1], dims[0]), dtype=dtype, device=self.device)

    def _conv(self, name, x, out, dims, residual=None):
        L = self.p[name]
        self.k.conv(x, L["cin"], L["w16"], L["b"], out, L["cout"], dims, L["relu"], residual)

    def forward(self, x16, x32, dims):
        """x16: [2][D][H][W] bf16 input, x32: the same in f32 (the residual);
        dims = (W, H, D), each divisible by 4. Returns y [2][D][H][W] f32."""
        d1, d2, d4 = tuple(dims), tuple(v // 2 for v in dims), tuple(v // 4 for v in dims)
        A = {}
        A["e1a"] = self._buf(16, d1)
        self._conv("e1a", x16, A["e1a"], d1)
        A["c1"] = self._buf(48, d1)
        A["e1"] = A["c1"][32:48]
        self._conv("e1b", A["e1a"], A["e1"], d1)
        A["p1"] = self._buf(16, d2)
        self.k.pool(A["e1"], A["p1"], 16, d1)
        A["e2a"] = self._buf(32, d2)
        self._conv("e2a", A["p1"], A["e2a"], d2)
        A["c2"] = self._buf(96, d2)
        A["e2"] = A["c2"][64:96]
        self._conv("e2b", A["e2a"], A["e2"], d2)
        A["p2"] = self._buf(32, d4)
        self.k.pool(A["e2"], A["p2"], 32, d2)
        A["m1"] = self._buf(64, d4)
        self._conv("m1", A["p2"], A["m1"], d4)
        A["m2"] = self._buf(64, d4)
        self._conv("m2", A["m1"], A["m2"], d4)
        self.k.up(A["m2"], A["c2"][0:64], 64, d2)
        A["d2a"] = self._buf(32, d2)
        self._conv("d2a", A["c2"], A["d2a"], d2)
        A["d2b"] = self._buf(32, d2)
        self._conv("d2b", A["d2a"], A["d2b"], d2)
        self.k.up(A["d2b"], A["c1"][0:32], 32, d1)
        A["d1a"] = self._buf(16, d1)
        self._conv("d1a", A["c1"], A["d1a"], d1)
        A["d1b"] = self._buf(16, d1)
        self._conv("d1b", A["d1a"], A["d1b"], d1)
        y = self._buf(2, d1, torch.float32)
        self._conv("out", A["d1b"], y, d1, residual=x32)
        A["x16"] = x16
        self.acts, self.dims = A, (d1, d2, d4)
        return y

    def _grads(self, name, g, x, dims, g_in=None):
        """Weight/bias gradients of layer `name` (output gradient g, input x) and,
        when g_in is given, the input gradient."""
        L = self.p[name]
        self.k.conv_grad_weight(g, L["cout"], x, L["cin"], dims, L["gw"], L["gb"])
        if g_in is not None:
            self.k.conv_grad_input(g, L["cout"], L["w16"], g_in, L["cin"], dims, self.scratch)

    def backward(self, gy):
        A = self.acts
        d1, d2, d4 = self.dims
        for L in self.p.values():
            L["gw"].zero_()
            L["gb"].zero_()
        G = lambda c, dims: self._buf(c, dims, torch.float32)
        g = G(16, d1)
        self._grads("out", gy, A["d1b"], d1, g)
        self.k.relu_grad(g, A["d1b"])
        g2 = G(16, d1)
        self._grads("d1b", g, A["d1a"], d1, g2)
        self.k.relu_grad(g2, A["d1a"])
        gc1 = G(48, d1)
        self._grads("d1a", g2, A["c1"], d1, gc1)
        g = G(32, d2)
        self.k.up_grad(gc1[0:32], g, 32, d1)
        self.k.relu_grad(g, A["d2b"])
        g2 = G(32, d2)
        self._grads("d2b", g, A["d2a"], d2, g2)
        self.k.relu_grad(g2, A["d2a"])
        gc2 = G(96, d2)
        self._grads("d2a", g2, A["c2"], d2, gc2)
        g = G(64, d4)
        self.k.up_grad(gc2[0:64], g, 64, d2)
        self.k.relu_grad(g, A["m2"])
        g2 = G(64, d4)
        self._grads("m2", g, A["m1"], d4, g2)
        self.k.relu_grad(g2, A["m1"])
        g = G(32, d4)
        self._grads("m1", g2, A["p2"], d4, g)
        ge2 = gc2[64:96]                       # skip gradient + the pooled path
        self.k.pool_grad(g, ge2, 32, d2, True)
        self.k.relu_grad(ge2, A["e2"])
        g2 = G(32, d2)
        self._grads("e2b", ge2, A["e2a"], d2, g2)
        self.k.relu_grad(g2, A["e2a"])
        g = G(16, d2)
        self._grads("e2a", g2, A["p1"], d2, g)
        ge1 = gc1[32:48]
        self.k.pool_grad(g, ge1, 16, d1, True)
        self.k.relu_grad(ge1, A["e1"])
        g2 = G(16, d1)
        self._grads("e1b", ge1, A["e1a"], d1, g2)
        self.k.relu_grad(g2, A["e1a"])
        self._grads("e1a", g2, A["x16"], d1)

    def adam(self, lr):
        self.step += 1
        for L in self.p.values():
            self.k.adam(L["w"], L["gw"], L["mw"], L["vw"], L["w16"], lr, self.step)
            self.k.adam(L["b"], L["gb"], L["mb"], L["vb"], L["b16"], lr, self.step)


# ------------------------------------------------------------------------------------------
# training data: seeded phantoms beamformed by the plain pipeline, full and subsampled aperture

BOX = ((-5e-3, -5e-3, 5e-3), (5e-3, 5e-3, 25e-3))


def phantom(seed, max_speckle=30000):
    """Point scatterers, speckle regions of random density (Gaussian amplitudes)
    and 1-5 mm anechoic spherical cysts (speckle removed), world coordinates [m]."""
    rng = np.random.default_rng(seed)
    lo, hi = np.array(BOX[0]), np.array(BOX[1])
    n_pts = int(rng.integers(5, 31))
    pts = lo + (hi - lo) * rng.random((n_pts, 3))
    amp = [rng.uniform(0.5, 2.0, n_pts)]
    pos = [pts]
    n_reg = int(rng.integers(1, 4))
    sp = []
    for _ in range(n_reg):
        c = lo + (hi - lo) * rng.random(3)
        rad = rng.uniform(2e-3, 6e-3, 3)
        n = int(max_speckle / n_reg * rng.uniform(0.2, 1.0))
        u = rng.standard_normal((n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        sp.append(c + u * (rng.random((n, 1)) ** (1.0 / 3.0)) * rad)
    sp = np.concatenate(sp)
    sp = sp[np.all((sp >= lo) & (sp <= hi), axis=1)]
    for _ in range(int(rng.integers(1, 4))):
        c = lo + (hi - lo) * (0.15 + 0.7 * rng.random(3))
        r = rng.uniform(0.5e-3, 2.5e-3)
        sp = sp[np.linalg.norm(sp - c, axis=1) > r]
    pos.append(sp)
    amp.append(0.3 * rng.standard_normal(len(sp)))
    return np.concatenate(pos).astype(np.float32), np.concatenate(amp).astype(np.float32)


def synth_rf(bp, pos, amp, seed, kernels):
    """int16 raw RF [channel][transmit][sample] (device) of a phantom: traces by
    bf_synth_traces, Hadamard encoding, noise and quantisation as synth.py."""
    S, C, T = int(bp.dec_data_dim[0]), int(bp.dec_data_dim[1]), int(bp.dec_data_dim[2])
    X = np.asarray(bp.xdc_transform[:], np.float32).reshape(4, 4)
    q = torch.from_numpy(pos + np.array([X[3, 0], X[3, 1], 0.0], np.float32)).cuda()
    a = torch.from_numpy(amp).cuda()
    x = torch.zeros(T * C * S, dtype=torch.float32, device="cuda")
    ok = kernels.lib.bf_synth_traces(ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(a.data_ptr()), len(amp),
                                     ctypes.c_void_p(x.data_ptr()), S, C, T, float(bp.xdc_element_pitch[0]),
                                     float(bp.xdc_element_pitch[1]), float(bp.sampling_frequency),
                                     float(bp.center_frequency), float(bp.speed_of_sound), kernels.stream)
    if not ok:
        raise RuntimeError("bf_synth_traces failed")
    return synth.encode_and_quantise(x.view(T, C, S), seed)


def learned_parameters(points=(128, 128, 256)):
    """The acquisition (128 tx, 128 rx, 2048 samples, decimation 2) on the 3D grid."""
    return synth.make_parameters(samples=2048, points=points, decimation=2, interpolate=0, frames=1,
                                 filter_length=64)


class PairMaker:
    """Full-aperture and every-4th-channel DAS of one acquisition through the
    library (decode -> demodulate -> linear DAS), as channels-first float32."""

    def __init__(self, bp, kernels):
        from .client import Beamformer
        self.bp, self.k = bp, kernels
        self.bf = Beamformer().configure(bp, [abi.SHADER["Decode"], abi.SHADER["Demodulate"], abi.SHADER["DAS"]],
                                         kaiser=synth.kaiser_spec(64), interpolation=2)
        self.dims = tuple(int(v) for v in bp.output_points[:3])
        n = int(np.prod(self.dims))
        self.frame = torch.empty(2 * n, dtype=torch.float32, device="cuda")

    def das(self, raw, rx_step):
        L = self.bf.lib
        if not L.beamformer_gb300_set_receive_subsampling(rx_step):
            raise RuntimeError("set_receive_subsampling failed")
        self.bf.push_device(raw.data_ptr(), raw.numel() * 2)
        d = (ctypes.c_int32 * 3)()
        if not L.beamformer_gb300_export_frame(0, 0, ctypes.cast(self.frame.data_ptr(), ctypes.POINTER(ctypes.c_float)),
                                               self.frame.numel() * 4, d):
            raise RuntimeError("export_frame failed")
        W, H, D = self.dims
        return self.frame.view(D, H, W, 2).permute(3, 0, 1, 2).contiguous()

    def pair(self, raw):
        """(input, target, scale): RX_STEP x subsampled DAS and the full DAS,
        both divided by the RMS of the input."""
        sub = self.das(raw, RX_STEP) * float(RX_STEP)
        full = self.das(raw, 1)
        self.bf.lib.beamformer_gb300_set_receive_subsampling(1)
        scale = float(torch.sqrt(torch.mean(sub * sub)).item()) or 1.0
        return sub / scale, full / scale, scale


def nrmse_db(y, t):
    return float(20 * torch.log10(torch.sqrt(torch.mean((y - t) ** 2)) / torch.sqrt(torch.mean(t * t))).item())


def make_dataset(n, seed0, points=(128, 128, 256), max_speckle=30000, kernels=None):
    """n pairs as bf16 tensors [n][2][D][H][W] (input, target) on the GPU."""
    k = kernels or Kernels()
    bp = learned_parameters(points)
    pm = PairMaker(bp, k)
    W, H, D = pm.dims
    X = torch.empty((n, 2, D, H, W), dtype=torch.bfloat16, device="cuda")
    Y = torch.empty((n, 2, D, H, W), dtype=torch.bfloat16, device="cuda")
    for i in range(n):
        pos, amp = phantom(seed0 + i, max_speckle)
        raw = synth_rf(bp, pos, amp, seed0 + i, k)
        x, y, _ = pm.pair(raw)
        k.convert(x, X[i])
        k.convert(y, Y[i])
    return X, Y, pm.dims


def lr_schedule(s, steps, lr, warmup=None, floor=0.05):
    """learning rate of step s: linear warm-up over the first `warmup` steps
    (steps / 10 by default), then a cosine decay from lr to floor * lr"""
    warmup = max(1, steps // 10) if warmup is None else max(1, warmup)
    ramp = min(1.0, (s + 1) / warmup)
    t = min(1.0, max(0.0, (s - warmup) / max(1, steps - warmup)))
    return lr * ramp * (floor + (1.0 - floor) * 0.5 * (1.0 + math.cos(math.pi * t)))


def train(X, Y, steps, crop=(64, 64, 64), lr=5e-4, seed=0, log_every=100, net=None, kernels=None, ema=0.999,
          eval_fn=None, eval_every=0):
    """Adam on random crops (one per step) of the pairs, the learning rate from
    lr_schedule, and an exponential moving average of the weights (decay `ema`
    from the first step: the average starts at the initial network, whose output
    is close to its input, and moves to the trained weights over about
    1 / (1 - ema) steps). Returns the network, whose averaged weights are the
    ones to evaluate (UNet.averaged), the logged losses (mean training loss over
    each logging window) and, when eval_fn is given, the curve
    [(step, eval_fn(net))] with the averaged weights every `eval_every` steps and
    after the last."""
    k = kernels or Kernels()
    net = net or UNet(seed=seed, kernels=k)
    curve = []
    rng = np.random.default_rng(seed)
    n, _, D, H, W = X.shape
    cx, cy, cz = crop
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    x32 = torch.empty((2, cz, cy, cx), dtype=torch.float32, device="cuda")
    t32 = torch.empty_like(x32)
    gy = torch.empty_like(x32)
    losses, window = [], 0
    for s in range(steps):
        i = int(rng.integers(n))
        z0 = int(rng.integers(0, (D - cz) // 4 + 1)) * 4
        y0 = int(rng.integers(0, (H - cy) // 4 + 1)) * 4
        x0 = int(rng.integers(0, (W - cx) // 4 + 1)) * 4
        xc = X[i, :, z0:z0 + cz, y0:y0 + cy, x0:x0 + cx].contiguous()
        k.convert(xc, x32)
        k.convert(Y[i, :, z0:z0 + cz, y0:y0 + cy, x0:x0 + cx].contiguous(), t32)
        y = net.forward(xc, x32, crop)
        k.mse(y, t32, gy, loss)             # accumulates over the logging window
        window += 1
        net.backward(gy)
        net.adam(lr_schedule(s, steps, lr))
        net.average(ema)
        if log_every and (s % log_every == 0 or s == steps - 1):
            losses.append((s, float(loss.item()) / window))
            loss.zero_()
            window = 0
        if eval_fn is not None and ((eval_every and (s + 1) % eval_every == 0) or s == steps - 1):
            if not curve or curve[-1][0] != s + 1:
                with net.averaged():
                    curve.append((s + 1, eval_fn(net)))
    if eval_fn is not None:
        return net, losses, curve
    return net, losses


def evaluate(net, X, Y, dims, kernels=None):
    """Per held-out pair: NRMSE (dB) of the subsampled DAS and of the network
    output against the full-aperture DAS."""
    k = kernels or Kernels()
    base, learned = [], []
    x32 = torch.empty(X.shape[1:], dtype=torch.float32, device="cuda")
    t32 = torch.empty_like(x32)
    for i in range(X.shape[0]):
        k.convert(X[i], x32)
        k.convert(Y[i], t32)
        y = net.forward(X[i], x32, dims)
        base.append(nrmse_db(x32, t32))
        learned.append(nrmse_db(y, t32))
    return np.array(base), np.array(learned)


def time_layers(layers, reps=5, forms=("",), seed=0):
    """Mean CUDA-event milliseconds of BF16 convolution layers [(cin, cout, (W, H, D))]
    with random inputs and weights, for each OGL_BF_UNET_TC form in `forms`
    ("" = the default form; "simt" = the direct kernel)."""
    import os
    k = Kernels()
    g = torch.Generator(device="cuda").manual_seed(seed)
    res = {}
    for cin, cout, dims in layers:
        W, H, D = dims
        x = torch.randn((cin, D, H, W), device="cuda", generator=g).to(torch.bfloat16)
        w = (torch.randn(cout * cin * 27, device="cuda", generator=g) * 0.05).to(torch.bfloat16)
        b = torch.zeros(cout, device="cuda")
        out = torch.empty((cout, D, H, W), device="cuda", dtype=torch.bfloat16)
        for form in forms:
            saved = {v: os.environ.get(v) for v in ("OGL_BF_UNET_TC", "OGL_BF_UNET_SIMT")}
            os.environ["OGL_BF_UNET_SIMT"] = "1" if form == "simt" else "0"
            os.environ["OGL_BF_UNET_TC"] = "" if form == "simt" else form
            try:
                k.conv(x, cin, w, b, out, cout, dims, True)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    k.conv(x, cin, w, b, out, cout, dims, True)
                e1.record()
                torch.cuda.synchronize()
            finally:
                for v, val in saved.items():
                    if val is None:
                        os.environ.pop(v, None)
                    else:
                        os.environ[v] = val
            res[f"{cin}->{cout} {W}x{H}x{D} {form or 'default'}"] = e0.elapsed_time(e1) / reps
    if k.lib.bf_unet_tc_errors(k.stream):
        raise RuntimeError("a tensor-core convolution's bounded wait ran out")
    return res


def _main(argv=None):
    """python -m ogl_beamforming_cuda_gb300.learned conv CIN COUT W H D [--reps N] [--forms a,b]:
    times one BF16 convolution layer; python -m ... forward W H D [--reps N]: times the
    whole network's forward pass (random weights). Prints one JSON line."""
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="python -m ogl_beamforming_cuda_gb300.learned")
    ap.add_argument("what", choices=["conv", "forward"])
    ap.add_argument("sizes", type=int, nargs="+")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--forms", default="")
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    if a.what == "conv":
        cin, cout, W, H, D = a.sizes
        print(json.dumps(time_layers([(cin, cout, (W, H, D))], a.reps, tuple(a.forms.split(",")))))
        return 0
    W, H, D = a.sizes
    net = UNet()
    x32 = torch.randn((2, D, H, W), device="cuda")
    x16 = x32.to(torch.bfloat16)
    net.forward(x16, x32, (W, H, D))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        net.forward(x16, x32, (W, H, D))
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"unet_forward_ms": e0.elapsed_time(e1) / a.reps, "dims": [W, H, D],
                      "tc_errors": int(net.k.lib.bf_unet_tc_errors(net.k.stream))}))
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
