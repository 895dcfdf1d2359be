"""Learned variant: the U-Net kernels against the numpy restatement (forward,
input and weight gradients, pooling, upsampling, loss), the whole network's
gradient against a float64 reference of the same network, and training on
pipeline-made pairs improving on the subsampled DAS it starts from."""
import numpy as np
import pytest
import torch

from oracle import unet_ref as U

pytestmark = pytest.mark.gpu


def bf16(a):
    """round to bfloat16 (nearest even), returned as float64"""
    t = torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16)
    return t.float().numpy().astype(np.float64)


@pytest.fixture(scope="module")
def k():
    from ogl_beamforming_cuda_gb300.learned import Kernels
    torch.cuda.set_device(0)
    return Kernels()


def dev(a, dtype):
    return torch.from_numpy(np.asarray(a, np.float32)).to(device="cuda", dtype=dtype).contiguous()


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("cin,cout,dims,relu", [(5, 11, (40, 12, 10), True), (16, 8, (32, 8, 8), False),
                                                (2, 16, (24, 20, 9), True)])
def test_conv_forward(k, cin, cout, dims, relu):
    rng = np.random.default_rng(cin * 100 + cout)
    W, H, D = dims
    x = bf16(rng.standard_normal((cin, D, H, W)))
    w = bf16(rng.standard_normal((cout, cin, 27)) * 0.2)
    b = rng.standard_normal(cout).astype(np.float32)
    r = rng.standard_normal((cout, D, H, W)).astype(np.float32)
    out = torch.empty((cout, D, H, W), dtype=torch.float32, device="cuda")
    k.conv(dev(x, torch.bfloat16), cin, dev(w.ravel(), torch.bfloat16), dev(b, torch.float32), out, cout, dims, relu,
           residual=dev(r, torch.float32))
    ref = U.conv3d(x, w, b, relu=relu, residual=r)
    assert rel(out.cpu().numpy(), ref) < 2e-6


@pytest.mark.parametrize("cin,cout,dims,out_type", [(96, 32, (24, 12, 10), torch.bfloat16),
                                                    (64, 64, (20, 9, 7), torch.float32),
                                                    (48, 16, (33, 5, 6), torch.bfloat16)])
def test_conv_forward_tensor_cores_against_direct(k, monkeypatch, cin, cout, dims, out_type):
    """BF16 inputs run as a tcgen05 implicit GEMM: the wide layers of the network,
    voxel counts that are not a multiple of the 128-voxel tile, in the slab form
    (the default) and the gathering form, against the direct FP32 kernel
    (OGL_BF_UNET_SIMT=1) and the float64 restatement; no bounded wait runs out."""
    rng = np.random.default_rng(cin + cout)
    W, H, D = dims
    x = bf16(rng.standard_normal((cin, D, H, W)))
    w = bf16(rng.standard_normal((cout, cin, 27)) * 0.05)
    b = rng.standard_normal(cout).astype(np.float32)
    outs = []
    for simt, form in (("0", "slab"), ("0", "gather"), ("1", "slab")):
        monkeypatch.setenv("OGL_BF_UNET_SIMT", simt)
        monkeypatch.setenv("OGL_BF_UNET_TC", form)
        out = torch.empty((cout, D, H, W), dtype=out_type, device="cuda")
        k.conv(dev(x, torch.bfloat16), cin, dev(w.ravel(), torch.bfloat16), dev(b, torch.float32), out, cout, dims, True)
        outs.append(out.float().cpu().numpy())
    assert k.lib.bf_unet_tc_errors(k.stream) == 0
    ref = U.conv3d(x, w, b, relu=True)
    tol = 1e-5 if out_type == torch.float32 else 8e-3         # BF16 outputs keep 8 significant bits
    for o in outs:
        assert rel(o, ref) < tol


@pytest.mark.parametrize("cin,cout,dims,out_type,residual", [(2, 16, (128, 2, 3), torch.bfloat16, False),
                                                             (48, 16, (32, 8, 6), torch.bfloat16, False),
                                                             (96, 32, (64, 4, 5), torch.float32, False),
                                                             (64, 64, (16, 16, 4), torch.bfloat16, False),
                                                             (16, 2, (256, 2, 3), torch.float32, True),
                                                             (40, 24, (8, 32, 3), torch.float32, True)])
def test_conv_forward_tma_tiles(k, monkeypatch, cin, cout, dims, out_type, residual):
    """Volumes whose rows tile by 128 voxels, where all three tensor-core forms
    apply (slab, TMA boxes per tap with zero fill at the faces, gather): against
    each other, the direct FP32 kernel and the float64 restatement; no bounded
    wait runs out."""
    rng = np.random.default_rng(cin * 7 + cout)
    W, H, D = dims
    x = bf16(rng.standard_normal((cin, D, H, W)))
    w = bf16(rng.standard_normal((cout, cin, 27)) * 0.05)
    b = rng.standard_normal(cout).astype(np.float32)
    r = bf16(rng.standard_normal((cout, D, H, W))) if residual else None
    outs = []
    for simt, form in (("0", "slab"), ("0", "tma"), ("0", "gather"), ("1", "slab")):
        monkeypatch.setenv("OGL_BF_UNET_SIMT", simt)
        monkeypatch.setenv("OGL_BF_UNET_TC", form)
        out = torch.empty((cout, D, H, W), dtype=out_type, device="cuda")
        k.conv(dev(x, torch.bfloat16), cin, dev(w.ravel(), torch.bfloat16), dev(b, torch.float32), out, cout, dims, True,
               residual=None if r is None else dev(r, out_type))
        outs.append(out.float().cpu().numpy())
    assert k.lib.bf_unet_tc_errors(k.stream) == 0
    ref = U.conv3d(x, w, b, relu=True, residual=r)
    # FP32 sums of up to 27 x 96 products in three different orders; BF16 outputs keep 8 bits
    tol = 1e-5 if out_type == torch.float32 else 8e-3
    for o in outs:
        assert rel(o, ref) < tol
    if out_type == torch.float32:
        for o in outs[1:3]:
            assert np.abs(outs[0] - o).max() <= 1e-5 * np.abs(ref).max()


def test_conv_forward_full_resolution_slab_against_direct(k, monkeypatch):
    """The network's largest layer at full size (48 -> 16 channels, 128 x 128 x 256):
    the slab form (tensor cores) against the direct FP32 kernel, every voxel; FP32
    sums of 1296 products each in two orders."""
    g = torch.Generator(device="cuda").manual_seed(5)
    cin, cout, dims = 48, 16, (128, 128, 256)
    W, H, D = dims
    x = torch.randn((cin, D, H, W), device="cuda", generator=g).to(torch.bfloat16)
    w = (torch.randn(cout * cin * 27, device="cuda", generator=g) * 0.05).to(torch.bfloat16)
    b = torch.randn(cout, device="cuda", generator=g)
    outs = []
    for simt in ("0", "1"):
        monkeypatch.setenv("OGL_BF_UNET_SIMT", simt)
        monkeypatch.delenv("OGL_BF_UNET_TC", raising=False)
        out = torch.empty((cout, D, H, W), dtype=torch.float32, device="cuda")
        k.conv(x, cin, w, b, out, cout, dims, True)
        outs.append(out)
    assert k.lib.bf_unet_tc_errors(k.stream) == 0
    diff = (outs[0] - outs[1]).abs().max().item()
    assert diff <= 1e-5 * outs[1].abs().max().item()


def test_conv_grad_input(k, monkeypatch):
    """the direct kernel (FP32 products)"""
    monkeypatch.setenv("OGL_BF_UNET_SIMT", "1")
    rng = np.random.default_rng(7)
    cin, cout, dims = 12, 9, (33, 10, 11)
    W, H, D = dims
    g = rng.standard_normal((cout, D, H, W)).astype(np.float32)
    w = bf16(rng.standard_normal((cout, cin, 27)) * 0.2)
    out = torch.empty((cin, D, H, W), dtype=torch.float32, device="cuda")
    scratch = torch.empty(cin * cout * 27, dtype=torch.bfloat16, device="cuda")
    k.conv_grad_input(dev(g, torch.float32), cout, dev(w.ravel(), torch.bfloat16), out, cin, dims, scratch)
    assert rel(out.cpu().numpy(), U.conv3d_grad_input(g, w)) < 2e-6


@pytest.mark.parametrize("cin,cout,dims,form", [(16, 32, (32, 8, 6), "slab"), (48, 16, (128, 2, 3), "tma"),
                                                (2, 16, (16, 16, 4), "slab"), (12, 9, (33, 10, 11), "slab")])
def test_conv_grad_input_tensor_cores(k, monkeypatch, cin, cout, dims, form):
    """The output gradient is rounded to BF16 and the input gradient runs on the
    tensor cores (slab form; TMA form where rows tile by 128 voxels), FP32
    accumulation: it equals the float64 input gradient of the rounded output
    gradient to FP32 summation error, and the direct FP32 kernel
    (OGL_BF_UNET_SIMT=1) to BF16 rounding."""
    monkeypatch.setenv("OGL_BF_UNET_TC", form)
    rng = np.random.default_rng(cin * 3 + cout)
    W, H, D = dims
    g = rng.standard_normal((cout, D, H, W)).astype(np.float32)
    w = bf16(rng.standard_normal((cout, cin, 27)) * 0.2)
    scratch = torch.empty(cin * cout * 27, dtype=torch.bfloat16, device="cuda")
    outs = []
    for simt in ("0", "1"):
        monkeypatch.setenv("OGL_BF_UNET_SIMT", simt)
        out = torch.empty((cin, D, H, W), dtype=torch.float32, device="cuda")
        k.conv_grad_input(dev(g, torch.float32), cout, dev(w.ravel(), torch.bfloat16), out, cin, dims, scratch)
        outs.append(out.cpu().numpy())
    assert k.lib.bf_unet_tc_errors(k.stream) == 0
    assert rel(outs[0], U.conv3d_grad_input(bf16(g), w)) < 1e-5
    assert rel(outs[1], U.conv3d_grad_input(g, w)) < 2e-6
    assert rel(outs[0], outs[1]) < 8e-3


def test_conv_grad_weight(k):
    rng = np.random.default_rng(8)
    cin, cout, dims = 10, 9, (36, 10, 7)
    W, H, D = dims
    g = rng.standard_normal((cout, D, H, W)).astype(np.float32)
    x = bf16(rng.standard_normal((cin, D, H, W)))
    gw = torch.zeros(cout * cin * 27, dtype=torch.float32, device="cuda")
    gb = torch.zeros(cout, dtype=torch.float32, device="cuda")
    k.conv_grad_weight(dev(g, torch.float32), cout, dev(x, torch.bfloat16), cin, dims, gw, gb)
    rw, rb = U.conv3d_grad_weight(g, x)
    assert rel(gw.cpu().numpy().reshape(cout, cin, 27), rw) < 1e-5
    assert rel(gb.cpu().numpy(), rb) < 1e-5


def test_pool_upsample_and_loss(k):
    rng = np.random.default_rng(9)
    c, dims = 3, (8, 6, 4)
    W, H, D = dims
    x = rng.standard_normal((c, D, H, W)).astype(np.float32)
    p = torch.empty((c, D // 2, H // 2, W // 2), dtype=torch.float32, device="cuda")
    k.pool(dev(x, torch.float32), p, c, dims)
    assert rel(p.cpu().numpy(), U.avgpool2(x)) < 1e-6
    u = torch.empty((c, D, H, W), dtype=torch.float32, device="cuda")
    k.up(p, u, c, dims)
    assert rel(u.cpu().numpy(), U.upsample2(p.cpu().numpy())) < 1e-7
    # gradients: adjoints of the linear maps
    go = rng.standard_normal((c, D // 2, H // 2, W // 2)).astype(np.float32)
    gi = torch.full((c, D, H, W), 1.0, dtype=torch.float32, device="cuda")
    k.pool_grad(dev(go, torch.float32), gi, c, dims, True)
    assert rel(gi.cpu().numpy(), 1.0 + U.upsample2(go) / 8.0) < 1e-6
    gu = torch.empty((c, D // 2, H // 2, W // 2), dtype=torch.float32, device="cuda")
    k.up_grad(dev(x, torch.float32), gu, c, dims)
    assert rel(gu.cpu().numpy(), 8.0 * U.avgpool2(x)) < 1e-6
    y, t = rng.standard_normal(1000).astype(np.float32), rng.standard_normal(1000).astype(np.float32)
    g = torch.empty(1000, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    k.mse(dev(y, torch.float32), dev(t, torch.float32), g, loss)
    rl, rg = U.mse(y, t)
    assert abs(loss.item() - rl) < 1e-5 * rl and rel(g.cpu().numpy(), rg) < 1e-6


def test_network_gradient_matches_reference(k):
    """Whole-network weight gradients against unet_ref.Network (float64, with the
    activations rounded to bf16 where the kernels store them)."""
    from ogl_beamforming_cuda_gb300.learned import UNet
    rng = np.random.default_rng(10)
    dims = (16, 8, 8)
    W, H, D = dims
    net = UNet(seed=3, kernels=k)
    x = bf16(rng.standard_normal((2, D, H, W)))
    t = rng.standard_normal((2, D, H, W)).astype(np.float32)
    y = net.forward(dev(x, torch.bfloat16), dev(x, torch.float32), dims)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    gy = torch.empty_like(y)
    k.mse(y, dev(t, torch.float32), gy, loss)
    net.backward(gy)
    ref = U.Network({n: (bf16(L["w16"].float().cpu().numpy()).reshape(L["cout"], L["cin"], 27),
                         L["b"].cpu().numpy().astype(np.float64)) for n, L in net.p.items()}, round_bf16=bf16)
    ry = ref.forward(x)
    assert rel(y.cpu().numpy(), ry) < 2e-3
    rl, rgy = U.mse(ry, t)
    grads = ref.backward(rgy)
    # BF16 activations (8 significant bits) round differently where the FP32 and
    # float64 sums straddle a rounding boundary, and the differences compound
    # through the layers: the gradients agree to about 1 % (relative L2); a wrong
    # kernel or data flow gives errors of order 1
    for n, L in net.p.items():
        gw = L["gw"].cpu().numpy().reshape(L["cout"], L["cin"], 27)
        assert rel_l2(gw, grads[n][0]) < 3e-2, n
        assert rel_l2(L["gb"].cpu().numpy(), grads[n][1]) < 3e-2, n


def test_training_improves_on_subsampled_das():
    """Pairs from the plain pipeline (subsampled and full-aperture DAS of seeded
    phantoms); after a short training the network is closer to the full-aperture
    volume than its input on held-out phantoms."""
    from ogl_beamforming_cuda_gb300 import learned as Lm
    torch.cuda.set_device(0)
    k = Lm.Kernels()
    X, Y, dims = Lm.make_dataset(48, 1000, points=(32, 32, 64), max_speckle=20000, kernels=k)
    Xt, Yt, _ = Lm.make_dataset(8, 900000, points=(32, 32, 64), max_speckle=20000, kernels=k)
    # 1500 Adam steps (warm-up and cosine decay from 1e-3, averaged weights); the
    # float atomics of the weight gradient make each short training take its own path
    mean_db = lambda n: float(np.mean(Lm.evaluate(n, Xt, Yt, dims, kernels=k)[1]))
    net, losses, curve = Lm.train(X, Y, 1500, crop=(32, 32, 32), lr=1e-3, log_every=100, kernels=k, ema=0.995,
                                  eval_fn=mean_db, eval_every=500)
    with net.averaged():
        base, learned = Lm.evaluate(net, Xt, Yt, dims, kernels=k)
    gain = float(np.mean(base - learned))
    print(f"held-out NRMSE vs full aperture: subsampled {base.mean():.1f} dB, network {learned.mean():.1f} dB, "
          f"gain {gain:.1f} dB; curve {curve}")
    assert gain > 0.5
    assert np.all(np.isfinite(learned))
    assert [c[0] for c in curve] == [500, 1000, 1500]
    assert curve[-1][1] == pytest.approx(float(np.mean(learned)), abs=1e-3)
    assert curve[-1][1] < curve[0][1]

