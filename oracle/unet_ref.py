"""CPU restatement (numpy, float64) of the learned variant's kernels: 3 x 3 x 3
"same" convolutions and their gradients, 2 x mean pooling, nearest 2 x
upsampling and the MSE loss. Test infrastructure: tests compare the GPU kernels
of include/bf_unet.h against these on small tensors.

Layout as the kernels: channels-first [C][D][H][W]; weights [Cout][Cin][3][3][3]
with the tap (kz, ky, kx) applied to the input at offset (kz - 1, ky - 1, kx - 1).
"""
import numpy as np


def _pad(x):
    return np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))


def conv3d(x, w, b=None, relu=False, residual=None):
    """out[co] = relu?(b[co] + sum_ci sum_k w[co, ci, k] x[ci, v + k - 1]) + residual[co]."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64).reshape(w.shape[0], w.shape[1], 3, 3, 3)
    cout = w.shape[0]
    _, D, H, W = x.shape
    xp = _pad(x)
    out = np.zeros((cout, D, H, W))
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                patch = xp[:, kz:kz + D, ky:ky + H, kx:kx + W]          # [cin, D, H, W]
                out += np.einsum("oc,cdhw->odhw", w[:, :, kz, ky, kx], patch)
    if b is not None:
        out += np.asarray(b, np.float64)[:, None, None, None]
    if relu:
        out = np.maximum(out, 0.0)
    if residual is not None:
        out += residual
    return out


def conv3d_grad_input(g, w):
    """d(sum g * conv3d(x, w)) / dx."""
    g = np.asarray(g, np.float64)
    w = np.asarray(w, np.float64).reshape(w.shape[0], w.shape[1], 3, 3, 3)
    cin = w.shape[1]
    _, D, H, W = g.shape
    gp = _pad(g)
    out = np.zeros((cin, D, H, W))
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                # x[v] meets g[v - (k - 1)]: window starting at 2 - k in the padded gradient
                patch = gp[:, 2 - kz:2 - kz + D, 2 - ky:2 - ky + H, 2 - kx:2 - kx + W]
                out += np.einsum("oc,odhw->cdhw", w[:, :, kz, ky, kx], patch)
    return out


def conv3d_grad_weight(g, x):
    """(d/dw, d/db) of sum g * conv3d(x, w, b): [Cout][Cin][27], [Cout]."""
    g = np.asarray(g, np.float64)
    x = np.asarray(x, np.float64)
    _, D, H, W = x.shape
    xp = _pad(x)
    gw = np.zeros((g.shape[0], x.shape[0], 3, 3, 3))
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                patch = xp[:, kz:kz + D, ky:ky + H, kx:kx + W]
                gw[:, :, kz, ky, kx] = np.einsum("odhw,cdhw->oc", g, patch)
    return gw.reshape(g.shape[0], x.shape[0], 27), g.sum(axis=(1, 2, 3))


def avgpool2(x):
    c, D, H, W = x.shape
    return np.asarray(x, np.float64).reshape(c, D // 2, 2, H // 2, 2, W // 2, 2).mean(axis=(2, 4, 6))


def upsample2(x):
    return np.repeat(np.repeat(np.repeat(np.asarray(x, np.float64), 2, axis=1), 2, axis=2), 2, axis=3)


def mse(y, t):
    d = np.asarray(y, np.float64) - np.asarray(t, np.float64)
    return float(np.mean(d * d)), 2.0 * d / d.size


class Network:
    """float64 restatement of the learned variant's U-Net (same layers and data
    flow as ogl_beamforming_cuda_gb300.learned.UNet). `params` maps a layer name
    to (w [Cout][Cin][27], b [Cout]); `round_bf16` rounds an array to bfloat16 and
    is applied where the kernels store an activation in BF16."""

    def __init__(self, params, round_bf16=lambda a: a):
        self.p = params
        self.R = round_bf16

    def _c(self, name, x, relu=True, residual=None):
        w, b = self.p[name]
        return conv3d(x, w, b, relu=relu, residual=residual)

    def forward(self, x):
        R, A = self.R, {}
        A["x"] = x
        A["e1a"] = R(self._c("e1a", x))
        A["e1"] = R(self._c("e1b", A["e1a"]))
        A["p1"] = R(avgpool2(A["e1"]))
        A["e2a"] = R(self._c("e2a", A["p1"]))
        A["e2"] = R(self._c("e2b", A["e2a"]))
        A["p2"] = R(avgpool2(A["e2"]))
        A["m1"] = R(self._c("m1", A["p2"]))
        A["m2"] = R(self._c("m2", A["m1"]))
        A["c2"] = np.concatenate([upsample2(A["m2"]), A["e2"]])
        A["d2a"] = R(self._c("d2a", A["c2"]))
        A["d2b"] = R(self._c("d2b", A["d2a"]))
        A["c1"] = np.concatenate([upsample2(A["d2b"]), A["e1"]])
        A["d1a"] = R(self._c("d1a", A["c1"]))
        A["d1b"] = R(self._c("d1b", A["d1a"]))
        self.A = A
        return self._c("out", A["d1b"], relu=False, residual=x)

    def backward(self, gy):
        A, G = self.A, {}

        def layer(name, g, x):
            G[name] = conv3d_grad_weight(g, x)
            return conv3d_grad_input(g, self.p[name][0])

        g = layer("out", gy, A["d1b"]) * (A["d1b"] > 0)
        g = layer("d1b", g, A["d1a"]) * (A["d1a"] > 0)
        gc1 = layer("d1a", g, A["c1"])
        g = 8.0 * avgpool2(gc1[:32]) * (A["d2b"] > 0)
        g = layer("d2b", g, A["d2a"]) * (A["d2a"] > 0)
        gc2 = layer("d2a", g, A["c2"])
        g = 8.0 * avgpool2(gc2[:64]) * (A["m2"] > 0)
        g = layer("m2", g, A["m1"]) * (A["m1"] > 0)
        g = layer("m1", g, A["p2"])
        g = (gc2[64:] + upsample2(g) / 8.0) * (A["e2"] > 0)
        g = layer("e2b", g, A["e2a"]) * (A["e2a"] > 0)
        g = layer("e2a", g, A["p1"])
        g = (gc1[32:] + upsample2(g) / 8.0) * (A["e1"] > 0)
        g = layer("e1b", g, A["e1a"]) * (A["e1a"] > 0)
        layer("e1a", g, A["x"])
        return G
