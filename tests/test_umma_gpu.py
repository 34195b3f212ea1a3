"""tcgen05 tensor-core kernels of the U-Net warm starter against plain PyTorch
FP32 references of the same ops (inputs are BF16, so the references see the
exact same values; tolerance: relative L2 1e-2 for BF16 outputs, 1e-4 for
FP32 outputs)."""
import numpy as np
import pytest
import torch
import torch.nn.functional as Fnn

from synkrotomo_gb300 import runtime as rt

pytestmark = pytest.mark.gpu


def _bf16(t):
    return t.to(torch.bfloat16).contiguous()


def _p(t):
    return rt._ptr(t)


def _rel(a, b):
    a = a.double()
    b = b.double()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


@pytest.mark.parametrize("M,N,K", [(128, 32, 64), (256, 64, 192), (384, 128, 512), (128, 256, 128), (256, 96, 256)])
def test_gemm_bf16(gpu, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = _bf16(torch.randn(M, K, device="cuda", generator=g))
    B = _bf16(torch.randn(N, K, device="cuda", generator=g))
    C = torch.full((M, N), float("nan"), device="cuda")
    ctx = rt.context()
    ctx.check(ctx.lib.synk_gemm_bf16(ctx.handle, _p(A), _p(B), _p(C), M, N, K), "gemm")
    ctx.sync()
    ref = A.float() @ B.float().T
    assert _rel(C, ref) < 1e-4


def _conv_ref(x, w, b=None):
    # x NHWC float, w [Cout][9*Cin] (tap-major) -> NHWC
    Bn, H, W, Cin = x.shape
    Cout = w.shape[0]
    wk = w.reshape(Cout, 3, 3, Cin).permute(0, 3, 1, 2)
    y = Fnn.conv2d(x.permute(0, 3, 1, 2), wk, b, padding=1)
    return y.permute(0, 2, 3, 1)


@pytest.mark.parametrize("Bn,H,W,Cin,Cout", [(2, 16, 128, 32, 32), (1, 64, 64, 64, 128), (2, 32, 32, 96, 256),
                                             (1, 128, 256, 32, 64), (2, 8, 256, 96, 32), (1, 8, 128, 192, 64),
                                             (1, 4, 128, 64, 96), (1, 4, 256, 128, 192), (1, 4, 128, 32, 256)])
def test_conv3x3_forward_bias_relu(gpu, Bn, H, W, Cin, Cout):
    g = torch.Generator(device="cuda").manual_seed(Cin * Cout + H)
    x = _bf16(torch.randn(Bn, H, W, Cin, device="cuda", generator=g))
    w = _bf16(0.1 * torch.randn(Cout, 9 * Cin, device="cuda", generator=g))
    bias = torch.randn(Cout, device="cuda", generator=g)
    y = torch.zeros(Bn, H, W, Cout, dtype=torch.bfloat16, device="cuda")
    ctx = rt.context()
    rc = ctx.lib.synk_conv3x3_bf16(ctx.handle, _p(x), Cin, 0, Cin, Bn, H, W, _p(w), _p(bias), _p(y), Cout, 0, Cout,
                                   1, None, 0, 0)
    ctx.check(rc, "conv")
    ctx.sync()
    ref = torch.relu(_conv_ref(x.float(), w.float(), bias))
    assert _rel(y.float(), ref) < 1e-2


def test_conv3x3_channel_slices(gpu):
    # input read from channels [32, 96) of a 128-channel buffer, output written
    # to channels [64, 96) of a 96-channel buffer (the U-Net's concatenations)
    Bn, H, W = 1, 32, 64
    g = torch.Generator(device="cuda").manual_seed(7)
    xbuf = _bf16(torch.randn(Bn, H, W, 128, device="cuda", generator=g))
    w = _bf16(0.1 * torch.randn(32, 9 * 64, device="cuda", generator=g))
    bias = torch.zeros(32, device="cuda")
    ybuf = torch.zeros(Bn, H, W, 96, dtype=torch.bfloat16, device="cuda")
    ctx = rt.context()
    rc = ctx.lib.synk_conv3x3_bf16(ctx.handle, _p(xbuf), 128, 32, 64, Bn, H, W, _p(w), _p(bias), _p(ybuf), 96, 64, 32,
                                   4, None, 0, 0)
    ctx.check(rc, "conv")
    ctx.sync()
    ref = _conv_ref(xbuf[..., 32:96].float(), w.float())
    assert _rel(ybuf[..., 64:96].float(), ref) < 1e-2
    assert float(ybuf[..., :64].float().abs().max()) == 0.0


def test_conv3x3_backward_data_with_relu_mask(gpu):
    Bn, H, W, Cin, Cout = 2, 32, 64, 64, 32
    g = torch.Generator(device="cuda").manual_seed(11)
    x = _bf16(torch.relu(torch.randn(Bn, H, W, Cin, device="cuda", generator=g)))     # a post-ReLU activation
    w = _bf16(0.1 * torch.randn(Cout, 9 * Cin, device="cuda", generator=g))
    dy = _bf16(torch.randn(Bn, H, W, Cout, device="cuda", generator=g))
    # reference: d/dx of sum(dy * conv(x)), masked by x > 0
    xr = x.float().clone().requires_grad_(True)
    y = _conv_ref(xr, w.float())
    y.backward(dy.float())
    ref = xr.grad * (x.float() > 0)
    # ours: the same convolution of dy with tap-flipped, transposed weights
    wt = w.float().reshape(Cout, 9, Cin).flip(1).permute(2, 1, 0).reshape(Cin, 9 * Cout)
    wt = _bf16(wt)
    dx = torch.zeros(Bn, H, W, Cin, dtype=torch.bfloat16, device="cuda")
    ctx = rt.context()
    rc = ctx.lib.synk_conv3x3_bf16(ctx.handle, _p(dy), Cout, 0, Cout, Bn, H, W, _p(wt), None, _p(dx), Cin, 0, Cin, 2,
                                   _p(x), Cin, 0)
    ctx.check(rc, "dgrad")
    ctx.sync()
    assert _rel(dx.float(), ref) < 1e-2


@pytest.mark.parametrize("Bn,H,W,Cin,Cout,ksplit", [(2, 16, 128, 32, 32, 4), (1, 32, 32, 96, 256, 2),
                                                    (2, 64, 64, 64, 128, 8)])
def test_conv3x3_weight_gradient(gpu, Bn, H, W, Cin, Cout, ksplit):
    g = torch.Generator(device="cuda").manual_seed(Cin + Cout + ksplit)
    x = _bf16(torch.randn(Bn, H, W, Cin, device="cuda", generator=g))
    dy = _bf16(torch.randn(Bn, H, W, Cout, device="cuda", generator=g))
    wr = torch.zeros(Cout, 9 * Cin, device="cuda", requires_grad=True)
    y = _conv_ref(x.float(), wr)
    y.backward(dy.float())
    ref = wr.grad
    cw = 64 if W >= 64 else 32

    def blocked(t):   # [B][H][W][C] -> [B][H][W/cw][C][cw]
        Bq, Hq, Wq, Cq = t.shape
        return t.reshape(Bq, Hq, Wq // cw, cw, Cq).permute(0, 1, 2, 4, 3).contiguous()

    dyT = blocked(dy)
    xs = torch.zeros(3, Bn, H, W, Cin, dtype=torch.bfloat16, device="cuda")
    xs[0, :, :, 1:] = x[:, :, :-1]     # kx = 0: x[w - 1]
    xs[1] = x
    xs[2, :, :, :-1] = x[:, :, 1:]     # kx = 2: x[w + 1]
    xT3 = torch.stack([blocked(xs[k]) for k in range(3)])
    dw = torch.zeros(Cout, 9 * Cin, device="cuda")
    ctx = rt.context()
    rc = ctx.lib.synk_conv3x3_wgrad_bf16(ctx.handle, _p(dyT), _p(xT3), _p(dw), Cin, Cout, Bn, H, W, ksplit)
    ctx.check(rc, "wgrad")
    ctx.sync()
    assert _rel(dw, ref) < 1e-4


@pytest.mark.parametrize("W,Cin,Cout,xoff,ldx", [(128, 64, 32, 32, 128), (256, 32, 96, 64, 96)])
def test_conv3x3_row_strip_slices_and_backward_data(gpu, W, Cin, Cout, xoff, ldx):
    """Rows of 128k pixels take the row-strip path: channel slices of a wider
    input buffer, and the backward-data form with the ReLU mask."""
    Bn, H = 1, 8
    g = torch.Generator(device="cuda").manual_seed(W + Cin)
    xbuf = _bf16(torch.relu(torch.randn(Bn, H, W, ldx, device="cuda", generator=g)))
    x = xbuf[..., xoff:xoff + Cin]
    w = _bf16(0.1 * torch.randn(Cout, 9 * Cin, device="cuda", generator=g))
    bias = torch.randn(Cout, device="cuda", generator=g)
    y = torch.zeros(Bn, H, W, Cout, dtype=torch.bfloat16, device="cuda")
    ctx = rt.context()
    rc = ctx.lib.synk_conv3x3_bf16(ctx.handle, _p(xbuf), ldx, xoff, Cin, Bn, H, W, _p(w), _p(bias), _p(y), Cout, 0,
                                   Cout, 4, None, 0, 0)
    ctx.check(rc, "conv")
    ctx.sync()
    assert _rel(y.float(), _conv_ref(x.float(), w.float(), bias)) < 1e-2
    # backward data: dx = conv(dy, flipped transposed w) * (x > 0), written into a slice
    dy = _bf16(torch.randn(Bn, H, W, Cout, device="cuda", generator=g))
    xr = x.float().clone().requires_grad_(True)
    _conv_ref(xr, w.float()).backward(dy.float())
    ref = xr.grad * (x.float() > 0)
    wt = _bf16(w.float().reshape(Cout, 9, Cin).flip(1).permute(2, 1, 0).reshape(Cin, 9 * Cout))
    dxbuf = torch.zeros(Bn, H, W, ldx, dtype=torch.bfloat16, device="cuda")
    rc = ctx.lib.synk_conv3x3_bf16(ctx.handle, _p(dy), Cout, 0, Cout, Bn, H, W, _p(wt), None, _p(dxbuf), ldx, xoff,
                                   Cin, 2, _p(xbuf), ldx, xoff)
    ctx.check(rc, "dgrad")
    ctx.sync()
    assert _rel(dxbuf[..., xoff:xoff + Cin].float(), ref) < 1e-2
    rest = torch.cat([dxbuf[..., :xoff], dxbuf[..., xoff + Cin:]], dim=-1)
    assert float(rest.float().abs().max()) == 0.0
