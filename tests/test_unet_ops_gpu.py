"""The U-Net kernels of the learned warm start (kw_unet.cu) against a plain
PyTorch FP32 reference on the CPU, one operation at a time.

Inputs are bf16 (the network's storage type); the reference gets the same
bf16 values in float32, so the comparison measures the kernels' accumulation
(FP32 on the tensor cores) and, for bf16 outputs, their final rounding.
Tolerances: 1e-5 relative L2 for f32 outputs, 4e-3 for bf16 outputs (the
bf16 unit roundoff is 2^-9)."""
import pytest

pytestmark = pytest.mark.gpu

F32_TOL = 1e-5
BF16_TOL = 4e-3


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def rel(a, b):
    a = a.detach().double().cpu()
    b = b.detach().double().cpu()
    return float((a - b).norm() / max(float(b.norm()), 1e-300))


def bf(shape, seed, scale=1.0):
    import torch

    g = torch.Generator().manual_seed(seed)
    return (scale * torch.randn(shape, generator=g)).to(torch.bfloat16)


def to_nchw(x):
    return x.float().permute(0, 3, 1, 2)


def w_torch(w):
    """(cout, 9, cin) -> torch conv weight (cout, cin, 3, 3)."""
    cout, _, cin = w.shape
    return w.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (256, 256, 640), (300, 72, 136), (1000, 200, 1152)])
def test_gemm_on_tensor_cores(M, N, K):
    import torch

    from kwave_gb300 import unet_ops as U

    A, B = bf((M, K), 1), bf((N, K), 2)
    got = U.gemm(A.cuda(), B.cuda())
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T
    e = rel(got, ref)
    print(f"gemm {M}x{N}x{K}: {e:.2e}")
    assert e <= F32_TOL


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (256, 64, 192), (384, 40, 320), (1152, 256, 4096)])
def test_gemm_on_mn_major_tiles(M, N, K):
    """The MN-major operand layout of the weight gradients, as a plain GEMM."""
    import torch

    from kwave_gb300 import unet_ops as U

    A, B = bf((K, M), 3), bf((K, N), 4)
    got = U.gemm_mn(A.cuda(), B.cuda())
    torch.cuda.synchronize()
    e = rel(got, A.float().T @ B.float())
    print(f"gemm MN-major {M}x{N}x{K}: {e:.2e}")
    assert e <= F32_TOL


def ref_conv(x1, w, bias=None, x2=None, relu=False):
    import torch
    import torch.nn.functional as F

    x = to_nchw(x1)
    if x2 is not None:
        x = torch.cat([x, F.interpolate(to_nchw(x2), scale_factor=2, mode="nearest")], dim=1)
    y = F.conv2d(x, w_torch(w), None if bias is None else bias.float(), padding=1)
    if relu:
        y = torch.relu(y)
    return y.permute(0, 2, 3, 1)


@pytest.mark.parametrize("concat", [False, True])
def test_conv3x3_forward(concat):
    import torch

    from kwave_gb300 import unet_ops as U

    nb, H, W = 2, 16, 12
    x1 = bf((nb, H, W, 16), 3)
    x2 = bf((nb, H // 2, W // 2, 24), 4) if concat else None
    cin = 16 + (24 if concat else 0)
    w = bf((32, 9, cin), 5, 0.2)
    bias = torch.randn(32, generator=torch.Generator().manual_seed(6))
    yb, yf = U.conv3x3(x1.cuda(), w.cuda(), bias.cuda(), relu=True, x2=None if x2 is None else x2.cuda(),
                       y=torch.empty((nb, H, W, 32), dtype=torch.bfloat16, device="cuda"),
                       yf=torch.empty((nb, H, W, 32), dtype=torch.float32, device="cuda"))
    torch.cuda.synchronize()
    ref = ref_conv(x1, w, bias, x2, relu=True)
    e32, e16 = rel(yf, ref), rel(yb, ref)
    print(f"conv3x3 concat={concat}: f32 {e32:.2e} bf16 {e16:.2e}")
    assert e32 <= F32_TOL and e16 <= BF16_TOL


@pytest.mark.parametrize("W,c1,c2,cout", [(128, 32, 0, 32), (128, 16, 32, 48), (256, 64, 0, 96)])
def test_conv3x3_halo_tiles(W, c1, c2, cout):
    """Rows of a multiple of 128 pixels with 16-channel inputs run on halo
    tiles (the nine taps as nine shifted views of one shared-memory halo):
    forward with and without the upsampled concatenation, against torch."""
    import torch

    from kwave_gb300 import unet_ops as U

    nb, H = 2, 6
    x1 = bf((nb, H, W, c1), 30)
    x2 = bf((nb, H // 2, W // 2, c2), 31) if c2 else None
    w = bf((cout, 9, c1 + c2), 32, 0.15)
    bias = torch.randn(cout, generator=torch.Generator().manual_seed(33))
    _, yf = U.conv3x3(x1.cuda(), w.cuda(), bias.cuda(), relu=True, x2=None if x2 is None else x2.cuda(),
                      yf=torch.empty((nb, H, W, cout), dtype=torch.float32, device="cuda"))
    torch.cuda.synchronize()
    e = rel(yf, ref_conv(x1, w, bias, x2, relu=True))
    print(f"halo conv W={W} c1={c1} c2={c2} cout={cout}: {e:.2e}")
    assert e <= F32_TOL


@pytest.mark.parametrize("nb,H,W,c1,cout", [(4, 64, 256, 32, 32), (2, 128, 128, 64, 64), (1, 20, 384, 16, 8),
                                           (2, 40, 128, 32, 128), (3, 7, 128, 16, 16), (1, 9, 256, 32, 160)])
def test_conv3x3_persistent_tma(nb, H, W, c1, cout):
    """One full-resolution input on rows of a multiple of 128 pixels runs on
    the persistent TMA-fed kernel (k_conv_tma): more tiles than CTAs (the
    halo ring and the two TMEM accumulators wrap around), tiles of two image
    rows (even heights, up to 128 output channels) and of one (odd heights,
    160 channels), 1-4 channel groups, 8-160 output channels, bf16 and f32
    outputs, against torch."""
    import torch

    from kwave_gb300 import unet_ops as U

    x1 = bf((nb, H, W, c1), 40)
    w = bf((cout, 9, c1), 41, 0.15)
    bias = torch.randn(cout, generator=torch.Generator().manual_seed(42))
    yb, yf = U.conv3x3(x1.cuda(), w.cuda(), bias.cuda(), relu=True,
                       y=torch.empty((nb, H, W, cout), dtype=torch.bfloat16, device="cuda"),
                       yf=torch.empty((nb, H, W, cout), dtype=torch.float32, device="cuda"))
    torch.cuda.synchronize()
    ref = ref_conv(x1, w, bias, relu=True)
    e32, e16 = rel(yf, ref), rel(yb, ref)
    print(f"persistent conv {nb}x{H}x{W} {c1}->{cout}: f32 {e32:.2e} bf16 {e16:.2e}")
    assert e32 <= F32_TOL and e16 <= BF16_TOL


def test_conv3x3_data_and_weight_gradients():
    """Data gradient as the flipped-weight convolution, weight and bias
    gradients, against torch autograd of the same convolution (concatenated
    upsampled input included)."""
    import torch

    from kwave_gb300 import unet_ops as U

    nb, H, W = 2, 16, 20
    x1, x2 = bf((nb, H, W, 8), 7), bf((nb, H // 2, W // 2, 16), 8)
    w = bf((48, 9, 24), 9, 0.2)
    dz = bf((nb, H, W, 48), 10)
    # reference
    xr1 = to_nchw(x1).requires_grad_(True)
    xr2 = to_nchw(x2).requires_grad_(True)
    wr = w_torch(w).requires_grad_(True)
    br = torch.zeros(48, requires_grad=True)
    import torch.nn.functional as F

    xin = torch.cat([xr1, F.interpolate(xr2, scale_factor=2, mode="nearest")], dim=1)
    y = F.conv2d(xin, wr, br, padding=1)
    y.backward(to_nchw(dz))
    # data gradient: convolution of dz with the flipped, transposed weights
    wt = U.flip_weights(w.cuda())
    _, dcat = U.conv3x3(dz.cuda(), wt, yf=torch.empty((nb, H, W, 24), dtype=torch.float32, device="cuda"))
    # the full-resolution part of the concatenation gradient is xr1's gradient itself
    e_d1 = rel(dcat[..., :8], xr1.grad.permute(0, 2, 3, 1))
    d1, d2 = U.split_concat_grad(dcat.to(torch.bfloat16).contiguous(), 8)
    e_d2 = rel(d2, xr2.grad.permute(0, 2, 3, 1))
    dw = torch.zeros((48, 9, 24), dtype=torch.float32, device="cuda")
    U.conv3x3_wgrad(x1.cuda(), dz.cuda(), dw, x2=x2.cuda())
    db = torch.zeros(48, dtype=torch.float32, device="cuda")
    U.bias_grad(dz.cuda(), db)
    torch.cuda.synchronize()
    e_w = rel(dw.reshape(48, 3, 3, 24).permute(0, 3, 1, 2), wr.grad)
    e_b = rel(db, br.grad)
    print(f"data grad {e_d1:.2e}, upsampled-branch grad {e_d2:.2e}, weight grad {e_w:.2e}, bias grad {e_b:.2e}")
    assert e_d1 <= F32_TOL and e_w <= F32_TOL and e_b <= F32_TOL and e_d2 <= BF16_TOL


def test_weight_gradient_large_pixel_split():
    """The weight gradient split over many CTAs (partial tiles added with
    red.add) at a full-resolution layer's size."""
    import torch

    from kwave_gb300 import unet_ops as U

    nb, H, W = 2, 128, 128
    x1, dz = bf((nb, H, W, 32), 11), bf((nb, H, W, 32), 12)
    dw = torch.zeros((32, 9, 32), dtype=torch.float32, device="cuda")
    U.conv3x3_wgrad(x1.cuda(), dz.cuda(), dw)
    torch.cuda.synchronize()
    import torch.nn.functional as F

    wr = torch.zeros((32, 32, 3, 3), requires_grad=True)
    F.conv2d(to_nchw(x1), wr, padding=1).backward(to_nchw(dz))
    e = rel(dw.reshape(32, 3, 3, 32).permute(0, 3, 1, 2), wr.grad)
    print(f"weight grad 2x128x128x32: {e:.2e}")
    assert e <= F32_TOL


def test_pool_relu_loss_adam():
    import torch
    import torch.nn.functional as F

    from kwave_gb300 import unet_ops as U

    x = bf((2, 8, 12, 16), 13)
    y = U.avgpool2(x.cuda())
    ref = F.avg_pool2d(to_nchw(x), 2).permute(0, 2, 3, 1)
    assert rel(y, ref) <= BF16_TOL
    dy = bf((2, 4, 6, 16), 14)
    add = bf((2, 8, 12, 16), 15)
    dx = U.avgpool2_bwd(dy.cuda(), add=add.cuda())
    xr = to_nchw(x).requires_grad_(True)
    F.avg_pool2d(xr, 2).backward(to_nchw(dy))
    assert rel(dx, xr.grad.permute(0, 2, 3, 1) + add.float()) <= BF16_TOL
    yy, gg = bf((4096,), 16), bf((4096,), 17)
    dz = U.relu_grad(gg.cuda(), yy.cuda())
    assert torch.equal(dz.cpu(), torch.where(yy.float() > 0, gg, torch.zeros_like(gg)))
    out = torch.randn((64, 16), generator=torch.Generator().manual_seed(18))
    img = torch.randn(64, generator=torch.Generator().manual_seed(22))
    tgt = torch.randn(64, generator=torch.Generator().manual_seed(19))
    dout = torch.empty((64, 16), dtype=torch.bfloat16, device="cuda")
    loss = torch.zeros(1, device="cuda")
    U.mse_grad(out.cuda(), img.cuda(), 0.7, tgt.cuda(), dout, 0.5, loss)
    e = U.residual_out(out.cuda(), img.cuda(), 0.7)
    torch.cuda.synchronize()
    est = out[:, 0] + 0.7 * img
    assert rel(e, est) <= F32_TOL
    assert abs(float(loss) - float(((est - tgt) ** 2).sum())) <= 1e-4 * float(((est - tgt) ** 2).sum())
    assert rel(dout[:, 0], 0.5 * (est - tgt)) <= BF16_TOL and float(dout[:, 1:].abs().max()) == 0.0
    # Adam against torch.optim.Adam over three steps
    w0 = torch.randn(1000, generator=torch.Generator().manual_seed(20))
    grads = [torch.randn(1000, generator=torch.Generator().manual_seed(21 + i)) for i in range(3)]
    wr = w0.clone().requires_grad_(True)
    opt = torch.optim.Adam([wr], lr=1e-2)
    w, m, v = w0.cuda(), torch.zeros(1000, device="cuda"), torch.zeros(1000, device="cuda")
    wb = torch.empty(1000, dtype=torch.bfloat16, device="cuda")
    for i, g in enumerate(grads):
        wr.grad = g.clone()
        opt.step()
        U.adam(w, m, v, g.cuda(), wb, 1e-2, i + 1)
    torch.cuda.synchronize()
    assert rel(w, wr) <= F32_TOL and rel(wb, wr) <= BF16_TOL
