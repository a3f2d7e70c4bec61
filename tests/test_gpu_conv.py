"""GPU: the BF16 implicit-GEMM 3x3x3 convolutions (agb_conv3_*) against
torch's CPU convolution in FP64 with circular padding, on the same
BF16-rounded inputs.  Forward, weight gradient and data gradient (forward
with the flipped weights) are each checked, as is a finite-difference
gradient check of a two-layer network through the kernels."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def lib():
    from alamo_gb300._lib import lib as L
    return L()


def cells(n):
    return (ctypes.c_int * 3)(*n)


def vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def to_ncdhw(x_cl, n, c):
    """[voxel][C] (voxel = x + n0 (y + n1 z)) -> (1, C, z, y, x)."""
    return x_cl.reshape(n[2], n[1], n[0], c).permute(3, 0, 1, 2).unsqueeze(0)


def torch_w(w_ours, cin, cout):
    """[27][cout][cin], tap = kx + 3 ky + 9 kz -> (cout, cin, kz, ky, kx)."""
    return w_ours.reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)


def ref_conv(x_cl, w_ours, bias, n, cin, cout, relu):
    x = to_ncdhw(x_cl.double(), n, cin)
    xp = torch.nn.functional.pad(x, (1, 1, 1, 1, 1, 1), mode="circular")
    y = torch.nn.functional.conv3d(xp, torch_w(w_ours.double(), cin, cout), bias.double() if bias is not None else None)
    if relu:
        y = torch.relu(y)
    return y[0].permute(1, 2, 3, 0).reshape(-1, cout)


def rand_bf16(shape, scale, gen):
    return (torch.randn(shape, generator=gen, dtype=torch.float32) * scale).to(torch.bfloat16)


@pytest.mark.parametrize("n,cin,cout,relu", [((16, 4, 2), 16, 16, False), ((32, 8, 4), 48, 16, True),
                                             ((16, 8, 6), 32, 32, True), ((32, 4, 4), 16, 48, False),
                                             ((16, 4, 2), 16, 8, False)])
def test_conv3_forward(gpu_lib, n, cin, cout, relu):
    gen = torch.Generator().manual_seed(cin * 7 + cout)
    V = n[0] * n[1] * n[2]
    x = rand_bf16((V, cin), 1.0, gen)
    w = rand_bf16((27, cout, cin), 0.1, gen)
    b = torch.randn(cout, generator=gen) * 0.1
    out = torch.zeros(V, cout, dtype=torch.float32, device="cuda")
    assert lib().agb_conv3_forward(cells(n), cin, cout, vp(x.cuda()), vp(w.cuda()), vp(b.cuda()), vp(out), 1,
                                   int(relu), None) == 0
    torch.cuda.synchronize()
    ref = ref_conv(x.float(), w.float(), b, n, cin, cout, relu)
    err = (out.cpu().double() - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


@pytest.mark.parametrize("n,cin,cout", [((16, 4, 2), 16, 16), ((32, 8, 4), 48, 16), ((16, 8, 6), 32, 32)])
def test_conv3_gradients(gpu_lib, n, cin, cout):
    gen = torch.Generator().manual_seed(cin + 100 * cout)
    V = n[0] * n[1] * n[2]
    x = rand_bf16((V, cin), 1.0, gen)
    w = rand_bf16((27, cout, cin), 0.1, gen)
    dy = rand_bf16((V, cout), 1.0, gen)
    # torch reference: gradients of sum(dy * conv(x, w)) in FP64
    xr = to_ncdhw(x.double(), n, cin).clone().requires_grad_(True)
    wr = torch_w(w.double(), cin, cout).clone().requires_grad_(True)
    y = torch.nn.functional.conv3d(torch.nn.functional.pad(xr, (1, 1, 1, 1, 1, 1), mode="circular"), wr)
    (y * to_ncdhw(dy.double(), n, cout)).sum().backward()
    dw_ref = wr.grad.permute(2, 3, 4, 0, 1).reshape(27, cout, cin)
    dx_ref = xr.grad[0].permute(1, 2, 3, 0).reshape(V, cin)
    db_ref = dy.double().sum(0)
    # ours
    dw = torch.zeros(27, cout, cin, dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    assert lib().agb_conv3_wgrad(cells(n), cin, cout, vp(x.cuda()), vp(dy.cuda()), vp(dw), vp(db), None) == 0
    wt = torch.zeros(27, cin, cout, dtype=torch.bfloat16, device="cuda")
    assert lib().agb_conv3_flip(cin, cout, vp(w.cuda()), vp(wt), None) == 0
    dx = torch.zeros(V, cin, dtype=torch.float32, device="cuda")
    assert lib().agb_conv3_forward(cells(n), cout, cin, vp(dy.cuda()), vp(wt), None, vp(dx), 1, 0, None) == 0
    torch.cuda.synchronize()
    for got, ref in ((dw, dw_ref), (db, db_ref), (dx, dx_ref)):
        err = (got.cpu().double() - ref).abs().max().item() / ref.abs().max().item()
        assert err < 1e-5, err


def test_relu_backward_and_adam(gpu_lib):
    gen = torch.Generator().manual_seed(5)
    y = rand_bf16((1000,), 1.0, gen).cuda()
    dy = rand_bf16((1000,), 1.0, gen).cuda()
    expect = torch.where(y.float() > 0, dy.float(), torch.zeros_like(dy.float()))
    assert lib().agb_relu_backward(1000, vp(y), vp(dy), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(dy.float(), expect)
    w = torch.randn(100, generator=gen).cuda()
    g = torch.randn(100, generator=gen).cuda()
    m = torch.zeros(100, device="cuda")
    v = torch.zeros(100, device="cuda")
    wb = torch.zeros(100, dtype=torch.bfloat16, device="cuda")
    w0 = w.clone()
    assert lib().agb_adam_step(100, vp(w), vp(g), vp(m), vp(v), vp(wb), 1e-2, 0.9, 0.999, 1e-8, 1, None) == 0
    torch.cuda.synchronize()
    # first Adam step moves every weight by lr * sign(g) (bias-corrected moments)
    assert torch.allclose(w - w0, -1e-2 * torch.sign(g), atol=1e-6)
    assert torch.equal(wb, w.to(torch.bfloat16))
