"""Thin torch-tensor wrappers of the U-Net kernels in libkwave_gb300
(kw_unet.cu, declared in include/kwave_gb300.h).  Tensors are CUDA tensors
owned by the caller: activations bf16 NHWC, parameters and gradients f32.
torch only allocates memory here; every operation is one of the library's
kernels, enqueued on torch's current stream."""
from __future__ import annotations

import ctypes as C

from . import _lib as K


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _st():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _lib():
    return K.lib()


def _contig(*ts):
    for t in ts:
        if t is not None and not t.is_contiguous():
            raise ValueError("kwave_gb300 U-Net kernels take contiguous tensors")


def gemm(A, B, out=None):
    """C = A @ B.T in f32 on the tensor cores (A: (M, K) bf16, B: (N, K) bf16)."""
    import torch

    _contig(A, B)
    M, Kd = A.shape
    N = B.shape[0]
    C_ = out if out is not None else torch.empty((M, N), dtype=torch.float32, device=A.device)
    K.check(_lib().kw_umma_gemm(_p(A), _p(B), _p(C_), M, N, Kd, _st()))
    return C_


def gemm_mn(A, B, out=None):
    """C = A.T @ B in f32 on the tensor cores from MN-major tiles (A: (K, M),
    B: (K, N) bf16, M and N multiples of 8)."""
    import torch

    _contig(A, B)
    Kd, M = A.shape
    N = B.shape[1]
    C_ = out if out is not None else torch.empty((M, N), dtype=torch.float32, device=A.device)
    K.check(_lib().kw_umma_gemm_mn(_p(A), _p(B), _p(C_), M, N, Kd, _st()))
    return C_


def conv3x3(x1, w, bias=None, relu=False, x2=None, y=None, yf=None):
    """3x3 same convolution of x1 (nb, H, W, c1) [+ upsampled x2 (nb, H/2,
    W/2, c2)] with w (cout, 9, c1 + c2) bf16; returns (y bf16, yf f32) as
    requested (bf16 by default)."""
    import torch

    _contig(x1, x2, w, bias)
    nb, H, W, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[3]
    cout = w.shape[0]
    if y is None and yf is None:
        y = torch.empty((nb, H, W, cout), dtype=torch.bfloat16, device=x1.device)
    K.check(_lib().kw_conv3x3(_p(x1), c1, _p(x2), c2, nb, H, W, _p(w), _p(bias), cout, int(bool(relu)), _p(y), _p(yf),
                              _st()))
    return y, yf


def conv3x3_wgrad(x1, dz, dw, x2=None):
    """dw (cout, 9, c1 + c2) f32 += weight gradient of conv3x3 for output gradient dz."""
    _contig(x1, x2, dz, dw)
    nb, H, W, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[3]
    K.check(_lib().kw_conv3x3_wgrad(_p(x1), c1, _p(x2), c2, nb, H, W, _p(dz), dz.shape[3], _p(dw), _st()))
    return dw


def flip_weights(w, wt=None):
    import torch

    cout, _, cin = w.shape
    wt = wt if wt is not None else torch.empty((cin, 9, cout), dtype=w.dtype, device=w.device)
    K.check(_lib().kw_unet_flip_weights(_p(w), _p(wt), cout, cin, _st()))
    return wt


def avgpool2(x):
    import torch

    nb, H, W, Cc = x.shape
    y = torch.empty((nb, H // 2, W // 2, Cc), dtype=x.dtype, device=x.device)
    K.check(_lib().kw_unet_avgpool2(_p(x), _p(y), nb, H, W, Cc, _st()))
    return y


def avgpool2_bwd(dy, add=None):
    import torch

    nb, h2, w2, Cc = dy.shape
    dx = torch.empty((nb, 2 * h2, 2 * w2, Cc), dtype=dy.dtype, device=dy.device)
    K.check(_lib().kw_unet_avgpool2_bwd(_p(dy), _p(dx), nb, 2 * h2, 2 * w2, Cc, _p(add), _st()))
    return dx


def relu_grad(dy, y):
    import torch

    dz = torch.empty_like(dy)
    K.check(_lib().kw_unet_relu_grad(_p(dy), _p(y), _p(dz), dy.numel(), _st()))
    return dz


def split_concat_grad(dcat, c1, add1=None):
    import torch

    nb, H, W, Cc = dcat.shape
    c2 = Cc - c1
    d1 = torch.empty((nb, H, W, c1), dtype=dcat.dtype, device=dcat.device)
    d2 = torch.empty((nb, H // 2, W // 2, c2), dtype=dcat.dtype, device=dcat.device)
    K.check(_lib().kw_unet_split_concat_grad(_p(dcat), nb, H, W, c1, c2, _p(d1), _p(add1), _p(d2), _st()))
    return d1, d2


def bias_grad(dz, db):
    K.check(_lib().kw_unet_bias_grad(_p(dz), _p(db), dz.numel() // dz.shape[-1], dz.shape[-1], _st()))
    return db


def mse_grad(out, img, s, target, dout, scale, loss):
    """loss += sum (out[..., 0] + s img - target)^2; dout = scale (...) in channel 0."""
    _contig(out, img, target, dout)
    K.check(_lib().kw_unet_mse_grad(_p(out), out.shape[-1], _p(img), C.c_float(s), _p(target), _p(dout),
                                     target.numel(), C.c_float(scale), _p(loss), _st()))


def residual_out(out, img, s, e=None):
    """e = out[..., 0] + s img (f32)."""
    import torch

    _contig(out, img)
    e = e if e is not None else torch.empty(img.shape, dtype=torch.float32, device=img.device)
    K.check(_lib().kw_unet_residual_out(_p(out), out.shape[-1], _p(img), C.c_float(s), _p(e), img.numel(), _st()))
    return e


def adam(w, m, v, g, wb, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    K.check(_lib().kw_unet_adam(_p(w), _p(m), _p(v), _p(g), _p(wb), w.numel(), C.c_float(lr), C.c_float(b1),
                                C.c_float(b2), C.c_float(eps), int(step), _st()))


def image_to_nhwc(img, x, scale):
    K.check(_lib().kw_unet_image_to_nhwc(_p(img), _p(x), img.numel(), x.shape[-1], C.c_float(scale), _st()))
