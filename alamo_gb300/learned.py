"""Learned correction for the multigrid-preconditioned GCR solve of periodic
isotropic RVEs (agb_learned_* and agb_conv3_* in the C ABI).

The network is a stack of 3x3x3 convolutions over the finest level, run by
this project's BF16 implicit-GEMM kernels (forward, data and weight
gradients) with Adam on FP32 master weights; torch tensors only hold device
memory here.  It is trained to map the residual left by one V-cycle,
r1 = r - A V(r), to the error that remains, e1 = A^{-1} r - V(r); inside
agb_learned_solve every GCR iteration adds the V-cycle direction V(r) and
then the learned direction N(r1) on the residual it left, and GCR minimises
the residual over all stored directions (a learned direction that does not
help leaves the V-cycle directions to carry the solve: the fallback).

    ConvNet        layers, forward/backward through the kernels, Adam, export
    training_pairs samples (features, residual, error target) from solves of
                   periodic RVEs
    train          Adam on the error of the correction
    train_highpass Adam on the high-frequency part of that error
    LearnedSolver  agb_learned_solve with or without the network (ablation)
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .elastic import Elastic, Linear, _ptr, default_params

FEAT = 16
DEFAULT_LAYERS = ((16, 32), (32, 32), (32, 16), (16, 16))   # (cin, cout); hidden ReLU, last linear


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _cells(n):
    return (ctypes.c_int * 3)(*[int(v) for v in n])


class ConvNet:
    def __init__(self, layers=DEFAULT_LAYERS, seed=0):
        import torch
        self.torch = torch
        self.layers = [tuple(int(v) for v in l) for l in layers]
        if self.layers[0][0] != FEAT or self.layers[-1][1] != FEAT:
            raise ValueError("the first layer takes %d channels and the last gives %d" % (FEAT, FEAT))
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.wb, self.mw, self.vw, self.mb, self.vb = [], [], [], [], [], [], []
        for l, (ci, co) in enumerate(self.layers):
            fan_in = 27 * ci
            scale = (2.0 / fan_in) ** 0.5 if l < len(self.layers) - 1 else 0.1 * (1.0 / fan_in) ** 0.5
            w = (torch.randn(27, co, ci, generator=g) * scale).cuda()
            self.w.append(w)
            self.b.append(torch.zeros(co, device="cuda"))
            self.wb.append(w.to(torch.bfloat16))
            self.mw.append(torch.zeros_like(w))
            self.vw.append(torch.zeros_like(w))
            self.mb.append(torch.zeros(co, device="cuda"))
            self.vb.append(torch.zeros(co, device="cuda"))
        self.step = 0
        self.out_scale = 1.0   # the model's correction is out_scale x the last layer's output

    # -- forward / backward through the conv kernels ----------------------
    def forward(self, n, feat):
        """feat: CUDA BF16 [V][16]; returns the FP32 output [V][16] and keeps
        the activations for backward."""
        torch = self.torch
        V = n[0] * n[1] * n[2]
        self.acts = [feat]
        x = feat
        for l, (ci, co) in enumerate(self.layers):
            last = l == len(self.layers) - 1
            out = torch.empty(V, co, dtype=torch.float32 if last else torch.bfloat16, device="cuda")
            check(lib().agb_conv3_forward(_cells(n), ci, co, _vp(x), _vp(self.wb[l]), _vp(self.b[l]), _vp(out),
                                          int(last), int(not last), None))
            if not last:
                self.acts.append(out)
            x = out
        return x

    def backward(self, n, dout):
        """dout: FP32 [V][16] gradient of the loss w.r.t. the output; returns
        the weight and bias gradients (FP32) of every layer."""
        torch = self.torch
        V = n[0] * n[1] * n[2]
        gw, gb = [None] * len(self.layers), [None] * len(self.layers)
        dy = dout.to(torch.bfloat16)
        for l in range(len(self.layers) - 1, -1, -1):
            ci, co = self.layers[l]
            x = self.acts[l]
            gw[l] = torch.zeros(27, co, ci, device="cuda")
            gb[l] = torch.zeros(co, device="cuda")
            check(lib().agb_conv3_wgrad(_cells(n), ci, co, _vp(x), _vp(dy), _vp(gw[l]), _vp(gb[l]), None))
            if l == 0:
                break
            wt = torch.empty(27, ci, co, dtype=torch.bfloat16, device="cuda")
            check(lib().agb_conv3_flip(ci, co, _vp(self.wb[l]), _vp(wt), None))
            dx = torch.empty(V, ci, dtype=torch.bfloat16, device="cuda")
            check(lib().agb_conv3_forward(_cells(n), co, ci, _vp(dy), _vp(wt), None, _vp(dx), 0, 0, None))
            check(lib().agb_relu_backward(V * ci, _vp(x), _vp(dx), None))   # x = ReLU output of layer l-1
            dy = dx
        return gw, gb

    def adam(self, gw, gb, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        for l in range(len(self.layers)):
            check(lib().agb_adam_step(self.w[l].numel(), _vp(self.w[l]), _vp(gw[l]), _vp(self.mw[l]),
                                      _vp(self.vw[l]), _vp(self.wb[l]), lr, b1, b2, eps, self.step, None))
            check(lib().agb_adam_step(self.b[l].numel(), _vp(self.b[l]), _vp(gb[l]), _vp(self.mb[l]),
                                      _vp(self.vb[l]), None, lr, b1, b2, eps, self.step, None))

    # -- export -----------------------------------------------------------
    def export(self):
        """(cin, cout, weights FP32 host, biases FP32 host) for agb_learned_create;
        out_scale is folded into the last (linear) layer."""
        cin = [c for c, _ in self.layers]
        cout = [c for _, c in self.layers]
        last = len(self.layers) - 1
        w = np.concatenate([t.detach().cpu().numpy().reshape(-1) * (self.out_scale if l == last else 1.0)
                            for l, t in enumerate(self.w)]).astype(np.float32)
        b = np.concatenate([t.detach().cpu().numpy().reshape(-1) * (self.out_scale if l == last else 1.0)
                            for l, t in enumerate(self.b)]).astype(np.float32)
        return cin, cout, w, b

    def state(self):
        return {"layers": self.layers, "w": [t.cpu().numpy() for t in self.w], "b": [t.cpu().numpy() for t in self.b]}


class LearnedHandle:
    """agb_learned: the network as the solver uses it (BF16 weights on the device)."""

    def __init__(self, net):
        cin, cout, w, b = net.export()
        h = ctypes.c_void_p()
        check(lib().agb_learned_create(len(cin), (ctypes.c_int * len(cin))(*cin), (ctypes.c_int * len(cout))(*cout),
                                       w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                       b.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().agb_learned_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# training data and training
# ---------------------------------------------------------------------------
def unique_rms(v, n):
    a = v.reshape(3, n + 1, n + 1, n + 1)[:, :n, :n, :n]
    return float(np.sqrt(np.mean(a * a)))


def features(n, r, ddw, scale):
    """BF16 features [n^3][16] of a residual in the reference layout."""
    import torch
    rd = torch.from_numpy(np.ascontiguousarray(r)).cuda()
    dd = ddw if hasattr(ddw, "data_ptr") else torch.from_numpy(np.ascontiguousarray(ddw)).cuda()
    feat = torch.empty(n ** 3, FEAT, dtype=torch.bfloat16, device="cuda")
    check(lib().agb_learned_features(_cells((n, n, n)), _vp(rd), _vp(dd), float(scale), _vp(feat), None))
    return feat


def training_pairs(n=64, count=8, seed=4242, rng_seed=1, contrast_max=100.0):
    """Training samples on n^3 periodic RVEs: for each RVE and each of two
    right-hand sides (its eigenstrain load and a random load), r1 = r -
    A V(r) after one FP64 V-cycle and e1 = A^{-1} r - V(r).  Each sample is a
    dict: op (the RVE's operator, kept for the residual loss), feat (BF16
    network features of r1), rhat (r1 / s at the unique nodes, [V][3]),
    target (e1 / (s h^2), [V][16]); s = RMS of r1."""
    import torch
    from . import microstructure as M
    rng = np.random.default_rng(rng_seed)
    pairs = []
    for q in range(count):
        _, ddw, F0 = M.rve_problem_device(q, seed=seed, edges=(n,), contrast_max=contrast_max)
        op = Elastic([n] * 3, None, "isotropic", periodic=(1, 1, 1))
        op.SetBC(_periodic_bc())
        op.SetModel(ddw)
        N = (n + 1) ** 3
        F0n = np.tile(np.asarray(F0).reshape(9), N)
        b_eig = op.NewtonRHS(np.zeros(3 * N), np.zeros(3 * N), F0=F0n)
        rnd = rng.standard_normal((3, n, n, n))
        b_rnd = np.pad(rnd, ((0, 0), (0, 1), (0, 1), (0, 1)), mode="wrap").reshape(-1) * np.abs(b_eig).max()
        for b in (b_eig, b_rnd):
            b = b - _unique_mean(b, n)
            one = Linear(op, fixed_iter=1, max_iter=1, max_fmg_iter=0)
            x1 = np.zeros(3 * N)
            one.solve(x1, b, 1e-30, 0.0, raise_on_fail=False)
            one.Clear()
            r1 = op.solutionResidual(0, x1, b)
            r1 = r1 - _unique_mean(r1, n)
            full = Linear(op, max_fmg_iter=0, precision=1)
            xs = np.zeros(3 * N)
            full.solve(xs, b, 1e-10, 0.0)
            full.Clear()
            e1 = xs - x1
            e1 = e1 - _unique_mean(e1, n)
            s = unique_rms(r1, n)
            h2 = (1.0 / n) ** 2
            feat = features(n, r1, ddw, s)
            t = e1.reshape(3, n + 1, n + 1, n + 1)[:, :n, :n, :n].reshape(3, -1).T / (s * h2)
            target = torch.zeros(n ** 3, FEAT, device="cuda")
            target[:, :3] = torch.from_numpy(np.ascontiguousarray(t)).float().cuda()
            rhat = _from_reference(torch.from_numpy(r1 / s).cuda(), n)
            pairs.append({"op": op, "feat": feat, "target": target, "rhat": rhat})
    return pairs


def _unique_mean(v, n):
    a = v.reshape(3, n + 1, n + 1, n + 1)
    m = a[:, :n, :n, :n].reshape(3, -1).mean(axis=1)
    return np.repeat(m, (n + 1) ** 3)


def _periodic_bc():
    from .elastic import Constant
    return Constant()


def train(net, pairs, n, steps=300, lr=2e-3):
    """Adam on the mean squared error of output channels 0-2 against the
    error targets; returns the loss history."""
    V = n ** 3
    net.out_scale = 1.0
    hist = []
    for it in range(steps):
        p = pairs[it % len(pairs)]
        out = net.forward((n, n, n), p["feat"])
        diff = out - p["target"]
        diff[:, 3:] = 0.0
        hist.append(float((diff[:, :3] ** 2).mean()))
        dout = diff * (2.0 / (3 * V))
        gw, gb = net.backward((n, n, n), dout)
        net.adam(gw, gb, lr=lr)
    return hist


def _to_reference(u_cl, n):
    """[V][3] channels-last (V = x + n (y + n z)) -> reference layout SoA over
    (n+1)^3 nodes with the periodic duplicates, float64."""
    import torch
    a = u_cl.reshape(n, n, n, 3).permute(3, 0, 1, 2)
    a = torch.cat([a, a[:, :1]], dim=1)
    a = torch.cat([a, a[:, :, :1]], dim=2)
    a = torch.cat([a, a[:, :, :, :1]], dim=3)
    return a.reshape(-1).double().contiguous()


def _from_reference(v, n):
    """reference layout (3, n+1, n+1, n+1) -> [V][3] at the unique nodes."""
    a = v.reshape(3, n + 1, n + 1, n + 1)[:, :n, :n, :n]
    return a.permute(1, 2, 3, 0).reshape(-1, 3)


def _highpass(op, v):
    """(I - P R) v on the finest level: the part of v that the next coarser
    level cannot represent (R full weighting, P trilinear prolongation;
    R = P^T / 8, so the filter is symmetric)."""
    import torch
    crse = torch.zeros(op.nodes(1) * 3, dtype=torch.float64, device="cuda")
    op.restriction(1, v, crse)
    smooth = torch.zeros_like(v)
    op.interpolation(0, smooth, crse)
    return v - smooth


def train_highpass(net, pairs, n, steps=300, lr=5e-5, warmup=50):
    """Adam on the high-frequency part of the correction's error, in units
    of s: per sample, loss_k = mean |H (c - e1 / (s h^2))|^2 / w_k over the
    unique nodes, c = sigma x the network output, H = I - P R, w_k = mean
    |H t_k|^2 (each sample weighs the same), sigma = RMS of H of the targets
    over the samples (so the output the loss asks for is of order one;
    sigma becomes net.out_scale).  One Adam step per pass over all samples
    (gradients summed), the learning rate ramped up over the first `warmup`
    steps (Adam's first steps move every weight by the full rate at once).  A local correction can only match the part of the
    remaining error that the coarse levels do not represent, and that part
    is what leaves the residual rough.  The gradient is exact (H is
    symmetric).  Returns the history of the mean loss."""
    import torch
    V = n ** 3
    wk = []
    for p in pairs:
        if "t_ref" not in p:
            p["t_ref"] = _to_reference(p["target"][:, :3], n)
        wk.append(float((_from_reference(_highpass(p["op"], p["t_ref"]), n) ** 2).mean()))
    sigma = float(np.sqrt(np.mean(wk))) or 1.0
    net.out_scale = sigma
    hist = []
    for it in range(steps):
        gsum_w, gsum_b, total = None, None, 0.0
        for k, p in enumerate(pairs):
            out = net.forward((n, n, n), p["feat"])
            d = _to_reference(out[:, :3].double() * sigma, n) - p["t_ref"]
            hu = _from_reference(_highpass(p["op"], d), n)
            total += float((hu ** 2).mean()) / wk[k]
            g = _from_reference(_highpass(p["op"], _to_reference(hu, n)), n) * (2.0 * sigma / (3 * V * wk[k]))
            dout = torch.zeros_like(out)
            dout[:, :3] = g.float()
            gw, gb = net.backward((n, n, n), dout)
            if gsum_w is None:
                gsum_w, gsum_b = gw, gb
            else:
                for l in range(len(gw)):
                    gsum_w[l] += gw[l]
                    gsum_b[l] += gb[l]
        hist.append(total / len(pairs))
        net.adam(gsum_w, gsum_b, lr=lr * min(1.0, (it + 1) / float(warmup)))
    return hist


# ---------------------------------------------------------------------------
# solve
# ---------------------------------------------------------------------------
class LearnedSolver:
    """agb_learned_solve on an operator: GCR with V-cycle (+ learned) directions."""

    def __init__(self, op, net=None, restart=8, **params):
        params.setdefault("max_iter", 200)
        self.params = default_params(**params)
        h = ctypes.c_void_p()
        check(lib().agb_solver_create(op.h, ctypes.byref(self.params), ctypes.byref(h)))
        self.h = h
        self.op = op
        self.handle = LearnedHandle(net) if net is not None else None
        self.restart = restart
        self.report = None

    def solve(self, sol, rhs, tol_rel=1e-8, tol_abs=0.0, raise_on_fail=True):
        rep = _lib.AgbSolveReport()
        ps, mem = _ptr(sol)
        pr, _ = _ptr(rhs)
        st = lib().agb_learned_solve(self.h, self.handle.h if self.handle else None, ps, pr, float(tol_rel),
                                     float(tol_abs), int(self.restart), mem, ctypes.byref(rep))
        self.report = rep
        if st != _lib.AGB_OK and raise_on_fail:
            check(st)
        return rep.res_final

    def close(self):
        if getattr(self, "h", None):
            lib().agb_solver_destroy(self.h)
            self.h = None
        if self.handle:
            self.handle.close()
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
