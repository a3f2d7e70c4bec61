"""GPU: the learned correction (alamo_gb300.learned, agb_learned_*).

* The network's gradients through the conv kernels against torch's CPU
  autograd in FP64 on the same BF16-rounded weights, inputs and activations.
* GCR with V-cycle directions against the oracle's solution of the same
  periodic RVE.
* Training reduces the loss, and the learned GCR converges to the same
  solution; the ablation (same problem, same GCR, without the network) is
  reported side by side.
"""
import sys

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def ref_forward(x_cl, ws, bs, n, layers):
    """FP64 CPU forward with the kernels' BF16 rounding of hidden activations."""
    F = torch.nn.functional
    x = x_cl.double().reshape(n[2], n[1], n[0], -1).permute(3, 0, 1, 2).unsqueeze(0)
    for l, (ci, co) in enumerate(layers):
        w = ws[l].double().reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)
        x = F.conv3d(F.pad(x, (1, 1, 1, 1, 1, 1), mode="circular"), w, bs[l].double())
        if l < len(layers) - 1:
            x = torch.relu(x).to(torch.bfloat16).double()
    return x[0].permute(1, 2, 3, 0).reshape(-1, layers[-1][1])


def test_network_gradients_match_cpu_autograd(gpu_lib):
    from alamo_gb300.learned import ConvNet
    layers = ((16, 32), (32, 16), (16, 16))
    n = (16, 4, 4)
    V = n[0] * n[1] * n[2]
    net = ConvNet(layers, seed=3)
    for l in range(len(layers)):
        net.b[l].normal_(0, 0.05)
    g = torch.Generator().manual_seed(11)
    feat = (torch.randn(V, 16, generator=g)).to(torch.bfloat16)
    target = torch.randn(V, 16, generator=g) * 0.1
    out = net.forward(n, feat.cuda())
    dout = (out - target.cuda()) * (2.0 / out.numel())
    gw, gb = net.backward(n, dout)
    # reference: the same loss in FP64 through torch autograd on the CPU
    ws = [w.detach().cpu().to(torch.bfloat16).double().requires_grad_(True) for w in net.w]
    bs = [b.detach().cpu().double().requires_grad_(True) for b in net.b]
    y = ref_forward(feat, ws, bs, n, layers)
    loss = ((y - target.double()) ** 2).mean()
    loss.backward()
    assert (out.cpu().double() - y.detach()).abs().max() <= 1e-2 * y.detach().abs().max()
    for l in range(len(layers)):
        for got, ref in ((gw[l], ws[l].grad), (gb[l], bs[l].grad)):
            err = (got.cpu().double() - ref).abs().max().item() / ref.abs().max().item()
            assert err < 3e-2, (l, err)


def rve(q, n, seed=4242):
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import Constant, Elastic
    _, ddw, F0 = M.rve_problem(q, seed=seed, edges=(n,))
    op = Elastic([n] * 3, None, "isotropic", periodic=(1, 1, 1))
    op.SetBC(Constant())
    op.SetModel(ddw)
    N = (n + 1) ** 3
    rhs = op.NewtonRHS(np.zeros(3 * N), np.zeros(3 * N), F0=np.tile(np.asarray(F0).reshape(9), N))
    return op, ddw, rhs


def zero_mean(u, n):
    a = u.reshape(3, n + 1, n + 1, n + 1)
    m = a[:, :n, :n, :n].reshape(3, -1).mean(axis=1)
    return (a - m[:, None, None, None]).reshape(-1)


def test_vcycle_gcr_matches_oracle(gpu_lib):
    from alamo_gb300.learned import LearnedSolver
    n = 32
    op, ddw, rhs = rve(2, n)
    s = LearnedSolver(op, None, restart=8)
    x = np.zeros_like(rhs)
    s.solve(x, rhs, 1e-9, 0.0)
    assert s.report.status == 0
    g = O.make_grid([n] * 3, sym=O.ISO, periodic=(1, 1, 1))
    xo, rep = O.solve(g, ddw, rhs, tol_rel=1e-10, tol_abs=0.0, params=O.default_params(max_fmg_iter=0))
    assert rep.status == 0
    err = np.abs(zero_mean(x, n) - xo).max() / np.abs(xo).max()
    assert err < 1e-6, err
    s.close()
    op.close()


def test_training_and_learned_gcr(gpu_lib, capsys):
    from alamo_gb300.learned import ConvNet, LearnedSolver, train, train_highpass, training_pairs
    n = 32
    pairs = training_pairs(n=n, count=2, seed=777)
    net_e = ConvNet(seed=2)
    hist = train(net_e, pairs, n, steps=40, lr=2e-3)
    assert np.mean(hist[-4:]) < np.mean(hist[:4]), (hist[:4], hist[-4:])
    net = ConvNet(seed=1)
    hist = train_highpass(net, pairs, n, steps=150, lr=5e-5)
    assert np.mean(hist[-4:]) < 0.8 * hist[0], (hist[:4], hist[-4:])
    with capsys.disabled():
        sys.stderr.write("\nhigh-pass loss: first %.4g last %.4g\n" % (np.mean(hist[:4]), np.mean(hist[-4:])))
    op, ddw, rhs = rve(5, n)
    base = LearnedSolver(op, None, restart=16)
    xb = np.zeros_like(rhs)
    base.solve(xb, rhs, 1e-8, 0.0)
    lrn = LearnedSolver(op, net, restart=16)
    xl = np.zeros_like(rhs)
    lrn.solve(xl, rhs, 1e-8, 0.0)
    assert base.report.status == 0 and lrn.report.status == 0
    err = np.abs(xl - xb).max() / np.abs(xb).max()
    assert err < 1e-6, err
    with capsys.disabled():
        sys.stderr.write("\nablation (32^3 RVE, GCR restart 16): V-cycle %d steps %.1f ms; V-cycle+learned %d steps "
                         "(%d fallbacks) %.1f ms\n" % (base.report.iterations, base.report.solve_ms,
                                                       lrn.report.iterations, lrn.report.refinements,
                                                       lrn.report.solve_ms))
    # GCR minimises over every stored direction: the learned ones cannot slow it
    assert lrn.report.iterations <= base.report.iterations + 1
    base.close()
    lrn.close()
    op.close()
