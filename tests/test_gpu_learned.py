"""GPU: the learned correction (the library's U-Net and its training kernels).

* The forward pass (agb_unet_forward) and the weight gradients of the
  backward pass (chained from agb_conv3_wgrad0, flipped-weight data gradients
  on the tensor cores, grid transfers and ReLU masks) against torch's FP64
  CPU autograd on the same graph: zero-padded 3x3x3 convolutions, P^T / 8
  down (a stride-2 convolution with the [1/2, 1, 1/2]^3 stencil) and P up
  (its transpose), skip concatenations, every stored activation rounded to
  BF16 as the kernels store it.
* A few Adam steps on multigrid samples lower the loss.
* The operator probed into a sparse matrix (operator_matrix) equals Fapply.
* Trained on the GCR gain (train_gain), the network removes, on held-out
  residuals of unseen problems, a clearly larger share of what the
  multigrid direction leaves than the untrained network does: the gain the
  network brings over the method without it, per GCR step.
* A mixed-precision solve with the network attached converges to the
  oracle's solution, and the network's directions are tried.
"""
import numpy as np
import pytest

import oracle as O
from helpers import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def torch_unet(net, feat, g0):
    """The U-Net restated in torch FP64 from the network's BF16 weights; returns
    (output [V][16], list of the weight tensors (leaves with gradients))."""
    F = torch.nn.functional
    Wt, Bt = [], []
    for l in range(len(net.w)):
        ci, co = net.cin[l], net.cout[l]
        w = net.wb[l].double().cpu().reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2).contiguous().requires_grad_(True)
        b = net.b[l].double().cpu().clone().requires_grad_(True)
        Wt.append(w)
        Bt.append(b)
    k1 = torch.tensor([0.5, 1.0, 0.5], dtype=torch.float64)
    K = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :])

    def bf(x):   # stored as BF16 (straight-through for the gradient)
        return x + (x.to(torch.bfloat16).double() - x).detach()

    def conv(l, x, relu=True):
        y = F.conv3d(x, Wt[l], Bt[l], padding=1)
        return bf(torch.relu(y)) if relu else y

    def down(x):
        C = x.shape[1]
        return bf(F.conv3d(x, K.expand(C, 1, 3, 3, 3), stride=2, padding=1, groups=C) / 8.0)

    def up(x):
        C = x.shape[1]
        return bf(F.conv_transpose3d(x, K.expand(C, 1, 3, 3, 3), stride=2, padding=1, groups=C))

    x = feat.double().cpu().reshape(g0[2], g0[1], g0[0], 16).permute(3, 0, 1, 2).unsqueeze(0)
    a1 = conv(0, x)
    s0 = conv(1, a1)
    b1 = conv(2, down(s0))
    s1 = conv(3, b1)
    c2 = conv(5, conv(4, down(s1)))
    d1 = conv(6, torch.cat([up(c2), s1], dim=1))
    e1 = conv(7, d1)
    f0 = conv(8, torch.cat([up(e1), s0], dim=1))
    out = conv(10, conv(9, f0), relu=False)
    return out[0].permute(1, 2, 3, 0).reshape(-1, 16), Wt, Bt


def make_net_and_features(n=16, seed=3):
    from alamo_gb300 import Elastic
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import TensionTest
    from alamo_gb300.learned import UNet, features
    ddw, _, _ = M.voronoi_cubic(n, ngrains=5, seed=seed)
    op = Elastic([n] * 3, None, "majorminor")
    op.SetBC(TensionTest("uniaxial_stress", disp=0.01))
    op.SetModel(ddw)
    r = np.random.default_rng(seed).standard_normal(3 * op.nodes(0))
    feat, rms = features(op, r)
    net = UNet(seed=seed)
    return op, net, feat, rms, r, ddw


def test_unet_forward_and_gradients_match_torch(gpu_lib):
    from alamo_gb300.learned import cosine_loss
    op, net, feat, rms, r, ddw = make_net_and_features()
    g0 = (17, 17, 17)
    assert net.nparams() == 366336 + sum(net.cout)
    # features: r / rms in channels 0-2, half logs of the moduli, the boundary flag
    f = feat.double().cpu().numpy()
    assert np.allclose(f[:, 0], r[:17 ** 3] / rms, rtol=1e-2, atol=1e-2)
    assert f[0, 9] == 1.0 and f[17 * 17 * 8 + 17 * 8 + 8, 9] == 0.0
    c = ddw.reshape(-1, 21)
    assert np.allclose(f[:, 3], 0.5 * np.log(c[:, 0]), rtol=1e-2, atol=1e-2)
    out = net.forward(g0, feat).clone()
    ref, Wt, Bt = torch_unet(net, feat, g0)
    e = float((out.double().cpu() - ref.detach()).abs().max() / ref.detach().abs().max())
    assert e < 2e-2, e
    target = torch.randn(17 ** 3, 3, generator=torch.Generator().manual_seed(5)).cuda()
    loss, dout = cosine_loss(out, target)
    gw, gb = net.backward(g0, dout)
    lt, _ = cosine_loss(ref, target.cpu())
    c_ = ref[:, :3]
    t_ = target.double().cpu()
    ce = (c_ * t_).sum()
    L = 1.0 - ce * ce / ((c_ * c_).sum() * (t_ * t_).sum())
    L.backward()
    assert abs(float(L) - loss) < 1e-2
    for l in range(len(Wt)):
        gref = Wt[l].grad.permute(2, 3, 4, 0, 1).reshape(27, net.cout[l], net.cin[l])
        eg = rel_err(gw[l].double().cpu().numpy(), gref.numpy())
        eb = rel_err(gb[l].double().cpu().numpy(), Bt[l].grad.numpy())
        print("layer %d: weight gradient rel err %.2e, bias %.2e" % (l, eg, eb))
        assert eg < 5e-2 and eb < 5e-2, (l, eg, eb)
    op.close()


def test_training_lowers_the_loss(gpu_lib):
    from alamo_gb300.learned import UNet, train, training_samples
    smp = training_samples(count=2, n=16, seed=11)
    net = UNet(seed=1)
    hist = train(net, smp, 16, steps=60, lr=1e-3, warmup=10)
    assert np.mean(hist[-10:]) < np.mean(hist[:10]), (hist[:10], hist[-10:])


def test_learned_mixed_solve_matches_oracle(gpu_lib):
    from alamo_gb300 import Elastic, Linear
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import TensionTest
    from alamo_gb300.learned import UNet, learned_stats
    from helpers import tension_bc_arrays
    n = 32
    ddw, _, _ = M.voronoi_cubic(n, ngrains=12, seed=21)
    bt, bv = tension_bc_arrays(0.01)
    g = O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bt, bc_val=bv)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, None, np.zeros(3 * N), b)
    xo, _ = O.solve(g, ddw, rhs, tol_rel=1e-8, tol_abs=0.0)
    op = Elastic([n] * 3, None, "majorminor")
    op.SetBC(TensionTest("uniaxial_stress", disp=0.01))
    op.SetModel(ddw)
    net = UNet(seed=2)
    s = Linear(op, precision=1, krylov=8)
    net.attach(s, min_gain=0.0, max_fail=1000)   # keep every direction: exercises the GCR with them
    x = np.zeros(3 * N)
    s.solve(x, rhs, 1e-8, 0.0)
    tried, kept, _ = learned_stats(s)
    assert s.report.status == 0 and tried > 0 and kept > 0
    r = O.residual(g, ddw, x, rhs)
    assert np.abs(r).max() <= 1e-8 * max(np.abs(rhs).max(), s.report.res0) * 1.000001
    assert rel_err(x, xo) < 1e-6
    s.Clear()
    op.close()


def test_operator_matrix_equals_fapply(gpu_lib):
    from alamo_gb300 import Elastic
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import TensionTest
    from alamo_gb300.learned import operator_matrix
    n = 12
    ddw, _, _ = M.voronoi_cubic(n, ngrains=4, seed=8)
    op = Elastic([n] * 3, None, "majorminor")
    op.SetBC(TensionTest("uniaxial_stress", disp=0.01))
    op.SetModel(ddw)
    A = operator_matrix(op)
    x = torch.randn(3 * op.nodes(0), dtype=torch.float64, device="cuda")
    f = torch.empty_like(x)
    op.Fapply(0, x, out=f)
    assert float((A @ x - f).abs().max() / f.abs().max()) < 1e-13
    op.close()


def test_gain_training_beats_untrained_network(gpu_lib):
    from alamo_gb300.learned import UNet, gain_samples, gcr_gain, train_gain
    n = 32
    train = gain_samples(count=4, n=n, seed=31)
    held = gain_samples(count=2, n=n, seed=97)
    net = UNet(seed=4)

    def mean_gain():
        g = []
        for p in held:
            for feat, r, rms, w in p["items"]:
                out = net.forward((n + 1,) * 3, feat)
                z = out[:, :3].double().t().reshape(-1) * rms * p["h2"]
                g.append(gcr_gain(p["A"], p["W"], z, r, w))
        return float(np.mean(g))

    before = mean_gain()
    train_gain(net, train, n, steps=600, lr=1e-3, warmup=30)
    after = mean_gain()
    print("held-out gain on top of the multigrid direction: untrained %.4f, trained %.4f" % (before, after))
    assert after > 0.03 and after > 5 * before, (before, after)
