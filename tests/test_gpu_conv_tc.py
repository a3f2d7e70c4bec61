"""GPU: the tensor-core (tcgen05) 3x3x3 convolution agb_conv3_tc against
torch's CPU convolution in FP64 with zero padding, on the same BF16-rounded
inputs: channel slices of wider channels-last buffers in and out, boxes whose
x extent is not a multiple of the kernel's 128-voxel line, every supported
output width, bias, ReLU, BF16 and FP32 output.  Output channels outside the
written slice must be left as they were."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def lib():
    from alamo_gb300._lib import lib as L
    return L()


def vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def ref_conv0(x, w, bias, n, cin, cout, relu):
    """x [voxel][cin] (voxel = x + n0 (y + n1 z)), w [27][cout][cin] (tap =
    kx + 3 ky + 9 kz): zero-padded cross-correlation, FP64."""
    xt = x.double().reshape(n[2], n[1], n[0], cin).permute(3, 0, 1, 2).unsqueeze(0)
    wt = w.double().reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
    y = torch.nn.functional.conv3d(xt, wt, bias.double() if bias is not None else None, padding=1)
    if relu:
        y = torch.relu(y)
    return y[0].permute(1, 2, 3, 0).reshape(-1, cout)


CASES = [((130, 5, 4), 16, 16), ((17, 9, 7), 48, 64), ((128, 3, 3), 32, 32), ((40, 6, 5), 16, 48),
         ((257, 2, 2), 64, 16), ((9, 4, 3), 96, 32)]


@pytest.mark.parametrize("n,cin,cout", CASES)
@pytest.mark.parametrize("out_f32,relu", [(False, True), (True, False)])
def test_conv3_tc_matches_torch(gpu_lib, n, cin, cout, out_f32, relu):
    from alamo_gb300._lib import check
    L = lib()
    gen = torch.Generator().manual_seed(n[0] + cin * 7 + cout)
    V = n[0] * n[1] * n[2]
    in_cs, in_c0 = cin + 16, 8          # the input is a slice of a wider buffer
    out_cs, out_c0 = cout + 24, 16      # and so is the output
    xin = (torch.randn((V, in_cs), generator=gen) * 1.0).to(torch.bfloat16)
    w = (torch.randn((27, cout, cin), generator=gen) * 0.1).to(torch.bfloat16)
    b = (torch.randn(cout, generator=gen) * 0.1).float()
    odt = torch.float32 if out_f32 else torch.bfloat16
    out = torch.full((V, out_cs), 7.0, dtype=odt).cuda()
    d_in, d_w, d_b = xin.cuda(), w.cuda(), b.cuda()
    d_wp = torch.empty(27 * cout * cin, dtype=torch.bfloat16, device="cuda")
    check(L.agb_conv3_tc_pack(cin, cout, vp(d_w), cout, 0, vp(d_wp), None))
    for rep in range(2):
        check(L.agb_conv3_tc((ctypes.c_int * 3)(*n), cin, cout, vp(d_in), in_cs, in_c0, vp(d_wp), vp(d_b), vp(out),
                             out_cs, out_c0, int(out_f32), int(relu), None))
        torch.cuda.synchronize()
        flag = ctypes.c_int(0)
        check(L.agb_conv3_tc_error(ctypes.byref(flag)))
        assert flag.value == 0
        got = out.cpu().double()
        ref = ref_conv0(xin[:, in_c0:in_c0 + cin], w, b, n, cin, cout, relu)
        scale = max(float(ref.abs().max()), 1e-30)
        tol = 1e-5 if out_f32 else 1e-2   # FP32 accumulation; BF16 output rounding (2^-8)
        err = float((got[:, out_c0:out_c0 + cout] - ref).abs().max()) / scale
        assert err < tol, (rep, err)
        assert bool((got[:, :out_c0] == 7.0).all()) and bool((got[:, out_c0 + cout:] == 7.0).all())


def test_conv3_tc_rejects_bad_arguments(gpu_lib):
    from alamo_gb300._lib import AGB_BADARG
    L = lib()
    t = torch.zeros(64 * 32, dtype=torch.bfloat16, device="cuda")
    n = (4, 4, 4)
    # cin not a multiple of 16, cout unsupported, slice outside the stride
    assert L.agb_conv3_tc((ctypes.c_int * 3)(*n), 8, 16, vp(t), 32, 0, vp(t), None, vp(t), 32, 0, 0, 0,
                          None) == AGB_BADARG
    assert L.agb_conv3_tc((ctypes.c_int * 3)(*n), 16, 24, vp(t), 32, 0, vp(t), None, vp(t), 32, 0, 0, 0,
                          None) == AGB_BADARG
    assert L.agb_conv3_tc((ctypes.c_int * 3)(*n), 16, 16, vp(t), 32, 24, vp(t), None, vp(t), 32, 0, 0, 0,
                          None) == AGB_BADARG
