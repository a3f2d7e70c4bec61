"""Learned correction for the mixed-precision multigrid solve (agb_unet_* and
agb_solver_set_learned in the C ABI).  No counterpart in the reference.

The network is the library's three-level convolutional encoder-decoder
(channels 16/32/64, 3x3x3 convolutions on the tensor cores with zero padding,
skip connections, full weighting down and trilinear prolongation up between
nodal grids).  Its forward pass is the library's (agb_unet_forward, the same
code the solver runs); the backward pass here chains the library's gradient
kernels (weight gradients, data gradients as convolutions with flipped
weights, grid transfers and their transposes, ReLU masks), and Adam updates
FP32 master weights with BF16 copies.  torch tensors only hold device memory
and compute the loss.

    UNet             weights, forward, backward, Adam, attach to a solver
    training_samples residuals and errors of multigrid iterates on random
                     cubic polycrystals (the solves the plain multigrid makes)
    train            Adam on the cosine between the network's correction and
                     the error (GCR rescales every direction, so only the
                     direction matters)
    operator_matrix  the finest-level operator of a small box as a sparse
                     matrix, probed through the library's Fapply
    train_gain       Adam on the quantity the solve's GCR keeps a direction
                     for: the weighted cosine between A N(r) and r
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .elastic import Elastic, Linear, _ptr

FEAT = 16


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _i3(g):
    return (ctypes.c_int * 3)(*[int(v) for v in g])


def topology():
    L = lib()
    nl, na = 11, 13
    cin, cout, lev = (ctypes.c_int * nl)(), (ctypes.c_int * nl)(), (ctypes.c_int * nl)()
    check(L.agb_unet_layers(cin, cout, lev))
    alev, ach = (ctypes.c_int * na)(), (ctypes.c_int * na)()
    check(L.agb_unet_acts(alev, ach))
    return list(cin), list(cout), list(lev), list(alev), list(ach)


def grids(g0):
    return [tuple(((int(v) - 1) >> l) + 1 for v in g0) for l in range(3)]


# activation indices (the order of agb_unet_acts)
FEATS, A1, CAT0, P1, B1, CAT1, P2, C1, C2, D1, E1, F0, H0 = range(13)


class UNet:
    def __init__(self, seed=0):
        import torch
        self.torch = torch
        self.cin, self.cout, self.lev, self.alev, self.ach = topology()
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.wb = [], [], []
        self.mw, self.vw, self.mb, self.vb = [], [], [], []
        last = len(self.cin) - 1
        for l, (ci, co) in enumerate(zip(self.cin, self.cout)):
            fan_in = 27 * ci
            scale = (2.0 / fan_in) ** 0.5 if l < last else 0.1 * (1.0 / fan_in) ** 0.5
            w = (torch.randn(27, co, ci, generator=g) * scale).cuda()
            self.w.append(w)
            self.wb.append(w.to(torch.bfloat16))
            self.b.append(torch.zeros(co, device="cuda"))
            for lst in (self.mw, self.vw):
                lst.append(torch.zeros_like(w))
            for lst in (self.mb, self.vb):
                lst.append(torch.zeros(co, device="cuda"))
        self.step = 0
        w_h = np.concatenate([t.cpu().numpy().reshape(-1) for t in self.w]).astype(np.float32)
        b_h = np.concatenate([t.cpu().numpy().reshape(-1) for t in self.b]).astype(np.float32)
        h = ctypes.c_void_p()
        check(lib().agb_unet_create(w_h.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                    b_h.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(h)))
        self.h = h
        self.sync()
        self._acts = None

    def close(self):
        if getattr(self, "h", None):
            lib().agb_learned_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nparams(self):
        return sum(t.numel() for t in self.w) + sum(t.numel() for t in self.b)

    def sync(self):
        """Hand the current BF16 weights and biases to the library's network."""
        n = len(self.w)
        wp = (ctypes.c_void_p * n)(*[t.data_ptr() for t in self.wb])
        bp = (ctypes.c_void_p * n)(*[t.data_ptr() for t in self.b])
        check(lib().agb_unet_set_weights(self.h, wp, bp, None))

    # -- forward / backward --------------------------------------------------
    def acts(self, g0):
        """Activation buffers for a grid of g0 nodes (kept between calls)."""
        torch = self.torch
        key = tuple(g0)
        if self._acts is None or self._acts[0] != key:
            G = grids(g0)
            bufs = [torch.empty(int(np.prod(G[self.alev[a]])) * self.ach[a], dtype=torch.bfloat16, device="cuda")
                    for a in range(len(self.alev))]
            out = torch.empty(int(np.prod(G[0])) * FEAT, dtype=torch.float32, device="cuda")
            self._acts = (key, bufs, out)
        return self._acts[1], self._acts[2]

    def forward(self, g0, feat):
        """feat: BF16 [V][16] on a grid of g0 nodes; returns the FP32 output
        [V][16] (a view of a buffer reused by the next call)."""
        bufs, out = self.acts(g0)
        bufs[FEATS].copy_(feat.reshape(-1))
        ptrs = (ctypes.c_void_p * len(bufs))(*[t.data_ptr() for t in bufs])
        check(lib().agb_unet_forward(self.h, _i3(g0), ptrs, _vp(out), None))
        return out.view(-1, FEAT)

    def _dgrad(self, l, g, dy, dy_cs, dy_c0, out, out_cs, out_c0):
        """out[:, out_c0 : out_c0 + cin_l] = data gradient of layer l at dy."""
        torch = self.torch
        L = lib()
        ci, co = self.cin[l], self.cout[l]
        wt = torch.empty(27 * ci * co, dtype=torch.bfloat16, device="cuda")
        check(L.agb_conv3_flip(ci, co, _vp(self.wb[l]), _vp(wt), None))   # [27][ci][co]
        c0 = 0
        while c0 < ci:
            w = min(64, ci - c0)
            if w == 48 and ci - c0 > 48:
                w = 32
            wp = torch.empty(27 * co * w, dtype=torch.bfloat16, device="cuda")
            check(L.agb_conv3_tc_pack(co, w, _vp(wt), ci, c0, _vp(wp), None))
            check(L.agb_conv3_tc(_i3(g), co, w, _vp(dy), dy_cs, dy_c0, _vp(wp), None, _vp(out), out_cs, out_c0 + c0,
                                 0, 0, None))
            c0 += w

    def _wgrad(self, l, g, x, x_cs, x_c0, dy, dy_cs, dy_c0, gw, gb):
        check(lib().agb_conv3_wgrad0(_i3(g), self.cin[l], self.cout[l], _vp(x), x_cs, x_c0, _vp(dy), dy_cs, dy_c0,
                                     _vp(gw[l]), _vp(gb[l]), None))

    def _mask(self, V, C, y, y_cs, y_c0, m, m_cs, m_c0, b=None, b_cs=0, b_c0=0, beta=0.0):
        check(lib().agb_axpby_mask(V, C, _vp(y), y_cs, y_c0, _vp(y), y_cs, y_c0, _vp(b), b_cs, b_c0, float(beta),
                                   _vp(m), m_cs, m_c0, None))

    def backward(self, g0, dout):
        """dout: FP32 [V][16], the loss gradient at the output of the last
        forward; returns the FP32 weight and bias gradients of every layer."""
        torch = self.torch
        L = lib()
        G = grids(g0)
        V = [int(np.prod(x)) for x in G]
        a, _ = self.acts(g0)
        gw = [torch.zeros(27, co, ci, device="cuda") for ci, co in zip(self.cin, self.cout)]
        gb = [torch.zeros(co, device="cuda") for co in self.cout]

        def buf(lev, c):
            return torch.empty(V[lev] * c, dtype=torch.bfloat16, device="cuda")

        dy = dout.reshape(-1).to(torch.bfloat16)
        self._wgrad(10, G[0], a[H0], 16, 0, dy, 16, 0, gw, gb)
        g_h0 = buf(0, 16)
        self._dgrad(10, G[0], dy, 16, 0, g_h0, 16, 0)
        self._mask(V[0], 16, g_h0, 16, 0, a[H0], 16, 0)
        self._wgrad(9, G[0], a[F0], 16, 0, g_h0, 16, 0, gw, gb)
        g_f0 = buf(0, 16)
        self._dgrad(9, G[0], g_h0, 16, 0, g_f0, 16, 0)
        self._mask(V[0], 16, g_f0, 16, 0, a[F0], 16, 0)
        self._wgrad(8, G[0], a[CAT0], 48, 0, g_f0, 16, 0, gw, gb)
        g_cat0 = buf(0, 48)
        self._dgrad(8, G[0], g_f0, 16, 0, g_cat0, 48, 0)
        g_e1 = buf(1, 32)
        check(L.agb_grid_prolong_t(_i3(G[0]), _i3(G[1]), 32, _vp(g_cat0), 48, 0, _vp(g_e1), 32, 0, 0.0, 1.0, None))
        self._mask(V[1], 32, g_e1, 32, 0, a[E1], 32, 0)
        self._wgrad(7, G[1], a[D1], 32, 0, g_e1, 32, 0, gw, gb)
        g_d1 = buf(1, 32)
        self._dgrad(7, G[1], g_e1, 32, 0, g_d1, 32, 0)
        self._mask(V[1], 32, g_d1, 32, 0, a[D1], 32, 0)
        self._wgrad(6, G[1], a[CAT1], 96, 0, g_d1, 32, 0, gw, gb)
        g_cat1 = buf(1, 96)
        self._dgrad(6, G[1], g_d1, 32, 0, g_cat1, 96, 0)
        g_c2 = buf(2, 64)
        check(L.agb_grid_prolong_t(_i3(G[1]), _i3(G[2]), 64, _vp(g_cat1), 96, 0, _vp(g_c2), 64, 0, 0.0, 1.0, None))
        self._mask(V[2], 64, g_c2, 64, 0, a[C2], 64, 0)
        self._wgrad(5, G[2], a[C1], 64, 0, g_c2, 64, 0, gw, gb)
        g_c1 = buf(2, 64)
        self._dgrad(5, G[2], g_c2, 64, 0, g_c1, 64, 0)
        self._mask(V[2], 64, g_c1, 64, 0, a[C1], 64, 0)
        self._wgrad(4, G[2], a[P2], 32, 0, g_c1, 64, 0, gw, gb)
        g_p2 = buf(2, 32)
        self._dgrad(4, G[2], g_c1, 64, 0, g_p2, 32, 0)
        # skip 1: its gradient from the concatenation plus (1/8) P of p2's
        g_s1 = buf(1, 32)
        check(L.agb_grid_prolong(_i3(G[1]), _i3(G[2]), 32, _vp(g_p2), 32, 0, _vp(g_s1), 32, 0, 0.0, 0.125, None))
        self._mask(V[1], 32, g_s1, 32, 0, a[CAT1], 96, 64, b=g_cat1, b_cs=96, b_c0=64, beta=1.0)
        self._wgrad(3, G[1], a[B1], 32, 0, g_s1, 32, 0, gw, gb)
        g_b1 = buf(1, 32)
        self._dgrad(3, G[1], g_s1, 32, 0, g_b1, 32, 0)
        self._mask(V[1], 32, g_b1, 32, 0, a[B1], 32, 0)
        self._wgrad(2, G[1], a[P1], 16, 0, g_b1, 32, 0, gw, gb)
        g_p1 = buf(1, 16)
        self._dgrad(2, G[1], g_b1, 32, 0, g_p1, 16, 0)
        g_s0 = buf(0, 16)
        check(L.agb_grid_prolong(_i3(G[0]), _i3(G[1]), 16, _vp(g_p1), 16, 0, _vp(g_s0), 16, 0, 0.0, 0.125, None))
        self._mask(V[0], 16, g_s0, 16, 0, a[CAT0], 48, 32, b=g_cat0, b_cs=48, b_c0=32, beta=1.0)
        self._wgrad(1, G[0], a[A1], 16, 0, g_s0, 16, 0, gw, gb)
        g_a1 = buf(0, 16)
        self._dgrad(1, G[0], g_s0, 16, 0, g_a1, 16, 0)
        self._mask(V[0], 16, g_a1, 16, 0, a[A1], 16, 0)
        self._wgrad(0, G[0], a[FEATS], 16, 0, g_a1, 16, 0, gw, gb)
        return gw, gb

    def adam(self, gw, gb, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        L = lib()
        for l in range(len(self.w)):
            check(L.agb_adam_step(self.w[l].numel(), _vp(self.w[l]), _vp(gw[l]), _vp(self.mw[l]), _vp(self.vw[l]),
                                  _vp(self.wb[l]), lr, b1, b2, eps, self.step, None))
            check(L.agb_adam_step(self.b[l].numel(), _vp(self.b[l]), _vp(gb[l]), _vp(self.mb[l]), _vp(self.vb[l]),
                                  None, lr, b1, b2, eps, self.step, None))
        self.sync()

    # -- use in a solve ------------------------------------------------------------
    def attach(self, solver, min_gain=0.01, max_fail=2):
        """Use the network in `solver` (a mixed-precision Linear with krylov > 0)."""
        check(lib().agb_solver_set_learned(solver.h, self.h, float(min_gain), int(max_fail)))
        solver._learned = self   # keep the network alive while the solver uses it

    @staticmethod
    def detach(solver):
        check(lib().agb_solver_set_learned(solver.h, None, 0.01, 2))
        solver._learned = None


def learned_stats(solver):
    """(directions tried, directions kept, network still in use) of the last solve."""
    t, k, a = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(lib().agb_solver_learned_stats(solver.h, ctypes.byref(t), ctypes.byref(k), ctypes.byref(a)))
    return t.value, k.value, bool(a.value)


def features(op, r):
    """BF16 features [V][16] of a residual r (reference layout, host or
    device) of the operator's finest level, and the residual's RMS."""
    import torch
    V = op.nodes(0)
    feat = torch.empty(V * FEAT, dtype=torch.bfloat16, device="cuda")
    rms = ctypes.c_double()
    pr, mem = _ptr(r)
    check(lib().agb_unet_features(op.h, pr, mem, _vp(feat), ctypes.byref(rms)))
    return feat.view(V, FEAT), rms.value


def _channels_last(v, n):
    """reference layout SoA (3, (n+1)^3) -> [V][3] FP32 (nodes = voxels)."""
    import torch
    t = v if hasattr(v, "data_ptr") else torch.from_numpy(np.ascontiguousarray(v)).cuda()
    return t.reshape(3, -1).t().contiguous().float()


# ---------------------------------------------------------------------------
# training data and training
# ---------------------------------------------------------------------------
def training_samples(count=64, n=64, seed=777, iterates=(1, 2, 3), log=None):
    """Samples from multigrid solves of random cubic polycrystals (8-64
    Voronoi grains of random orientation, the benchmark's moduli) under
    TensionTest uniaxial_stress on n^3-cell boxes: for each problem and each
    k in `iterates`, the residual r_k = b - A x_k of the k-th FP64 F-cycle
    iterate from x = 0 and its error e_k = x - x_k against the converged
    solution (FP32 cycles in FP64 refinement to 1e-10).  Each sample: feat
    (BF16 [V][16] network features of r_k), target (e_k channels-last FP32
    [V][3])."""
    import torch
    from . import microstructure as M
    from .elastic import TensionTest
    rng = np.random.default_rng(seed)
    N = (n + 1) ** 3
    out = []
    for q in range(count):
        ng = int(rng.integers(8, 65))
        ddw, _, _ = M.voronoi_cubic_device(n, ngrains=ng, seed=int(rng.integers(1, 2 ** 31)))
        op = Elastic([n] * 3, None, "majorminor")
        op.SetBC(TensionTest("uniaxial_stress", disp=0.01))
        op.SetModel(ddw)
        del ddw
        zero = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
        b = op.BCInit(torch.zeros(3 * N, dtype=torch.float64, device="cuda"))
        rhs = torch.empty(3 * N, dtype=torch.float64, device="cuda")
        op.NewtonRHS(zero, b, out=rhs)
        xs = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
        full = Linear(op, precision=1, krylov=8)
        full.solve(xs, rhs, 1e-10, 0.0)
        full.Clear()
        for k in iterates:
            s = Linear(op, fixed_iter=k, max_iter=k)
            xk = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
            s.solve(xk, rhs, 1e-30, 0.0, raise_on_fail=False)
            s.Clear()
            rk = torch.empty(3 * N, dtype=torch.float64, device="cuda")
            op.solutionResidual(0, xk, rhs, out=rk)
            feat, _ = features(op, rk)
            out.append({"feat": feat, "target": _channels_last(xs - xk, n)})
        op.close()
        if log and (q + 1) % max(1, count // 4) == 0:
            log("training samples: %d of %d problems" % (q + 1, count))
    return out


def cosine_loss(out, target):
    """1 - cos^2 between the correction out[:, 0:3] and the error, over all
    nodes, and its gradient with respect to out (FP32 [V][16])."""
    import torch
    c = out[:, :3].double()
    e = target.double()
    ce = float((c * e).sum())
    cc = float((c * c).sum())
    ee = float((e * e).sum())
    if cc <= 0 or ee <= 0:
        return 1.0, torch.zeros_like(out)
    loss = 1.0 - ce * ce / (cc * ee)
    g = torch.zeros_like(out)
    g[:, :3] = (-2.0 * ce / (cc * ee) * e + 2.0 * ce * ce / (cc * cc * ee) * c).float()
    return loss, g


def train(net, samples, n, steps=1000, lr=1e-3, warmup=50, log=None):
    """Adam on the cosine loss, one sample per step (cycling), the learning
    rate ramped up over the first `warmup` steps.  Returns the loss history."""
    g0 = (n + 1,) * 3
    hist = []
    for it in range(steps):
        smp = samples[it % len(samples)]
        out = net.forward(g0, smp["feat"])
        loss, dout = cosine_loss(out, smp["target"])
        hist.append(loss)
        gw, gb = net.backward(g0, dout)
        net.adam(gw, gb, lr=lr * min(1.0, (it + 1) / float(warmup)))
        if log and (it + 1) % max(1, steps // 5) == 0:
            log("step %d: mean loss over the last %d steps %.4f" % (it + 1, min(it + 1, 50), float(np.mean(hist[-50:]))))
    return hist


# ---------------------------------------------------------------------------
# training on the GCR gain
# ---------------------------------------------------------------------------
def operator_matrix(op):
    """The FP64 finest-level operator A of `op` (no periodic direction) as a
    torch sparse CSR matrix over the reference layout (3 components of the
    (n+1)^3 nodes), probed with 81 applications of the library's Fapply:
    every row's stencil lies in the 3 x 3 x 3 neighbourhood of its node, so
    a probe that is 1 on component p of the nodes of one colour (i, j, k mod
    3) returns, in each row, the one matrix entry of that row for that
    colour and component."""
    import torch
    nx, ny, nz = [c + 1 for c in op.n]
    N = nx * ny * nz
    k, j, i = torch.meshgrid(torch.arange(nz, device="cuda"), torch.arange(ny, device="cuda"),
                             torch.arange(nx, device="cuda"), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    rows, cols, vals = [], [], []
    f = torch.empty(3 * N, dtype=torch.float64, device="cuda")
    for cz in range(3):
        for cy in range(3):
            for cx in range(3):
                colour = ((i % 3) == cx) & ((j % 3) == cy) & ((k % 3) == cz)
                # the node of this colour in each node's neighbourhood
                mi = i + ((cx - i) % 3 + 1) % 3 - 1
                mj = j + ((cy - j) % 3 + 1) % 3 - 1
                mk = k + ((cz - k) % 3 + 1) % 3 - 1
                inside = (mi >= 0) & (mi < nx) & (mj >= 0) & (mj < ny) & (mk >= 0) & (mk < nz)
                m = mi + nx * (mj + ny * mk)
                for p in range(3):
                    e = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
                    e[p * N:(p + 1) * N] = colour.double()
                    op.Fapply(0, e, out=f)
                    for c in range(3):
                        v = f[c * N:(c + 1) * N]
                        keep = inside & (v != 0)
                        rows.append((c * N + torch.arange(N, device="cuda"))[keep])
                        cols.append((p * N + m)[keep])
                        vals.append(v[keep])
    r = torch.cat(rows)
    c = torch.cat(cols)
    v = torch.cat(vals)
    A = torch.sparse_coo_tensor(torch.stack([r, c]), v, (3 * N, 3 * N)).coalesce()
    return A.to_sparse_csr()


def gain_samples(count=16, n=64, seed=777, iterates=(1, 2, 4, 8), log=None):
    """Residual samples for train_gain: per random polycrystal problem (as in
    training_samples) the residuals r_k of the k-th FP64 F-cycle iterate
    from x = 0, the image w = A M r_k of the multigrid direction on that
    residual (M one F-cycle), the operator A as a sparse matrix and the GCR
    weights 1/diag^2.  Each problem: {A, At, W, h2, items: [(feat, r, rms,
    w)]}."""
    import torch
    from . import microstructure as M
    from .elastic import TensionTest
    rng = np.random.default_rng(seed)
    N = (n + 1) ** 3
    out = []
    for q in range(count):
        ng = int(rng.integers(8, 65))
        ddw, _, _ = M.voronoi_cubic_device(n, ngrains=ng, seed=int(rng.integers(1, 2 ** 31)))
        op = Elastic([n] * 3, None, "majorminor")
        op.SetBC(TensionTest("uniaxial_stress", disp=0.01))
        op.SetModel(ddw)
        del ddw
        zero = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
        b = op.BCInit(torch.zeros(3 * N, dtype=torch.float64, device="cuda"))
        rhs = torch.empty(3 * N, dtype=torch.float64, device="cuda")
        op.NewtonRHS(zero, b, out=rhs)
        A = operator_matrix(op)
        D = op.Diagonal(0, out=torch.empty(3 * N, dtype=torch.float64, device="cuda"))
        items = []
        for k in iterates:
            s = Linear(op, fixed_iter=k, max_iter=k)
            xk = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
            s.solve(xk, rhs, 1e-30, 0.0, raise_on_fail=False)
            s.Clear()
            rk = torch.empty(3 * N, dtype=torch.float64, device="cuda")
            op.solutionResidual(0, xk, rhs, out=rk)
            feat, rms = features(op, rk)
            one = Linear(op, fixed_iter=1, max_iter=1)
            zm = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
            one.solve(zm, rk, 1e-30, 0.0, raise_on_fail=False)
            one.Clear()
            items.append((feat, rk, rms, A @ zm))
        out.append({"A": A, "At": A.t().to_sparse_csr(), "W": 1.0 / D ** 2, "h2": (1.0 / n) ** 2, "items": items})
        op.close()
        if log and (q + 1) % max(1, count // 4) == 0:
            log("gain samples: %d of %d problems" % (q + 1, count))
    return out


def _wproj_out(v, w, W):
    """v minus its weighted projection on w."""
    ww = (w * w * W).sum()
    return v - ((v * w * W).sum() / ww) * w if float(ww) > 0 else v


def gcr_gain(A, W, z, r, w=None):
    """The fraction of ||r||_W^2 one GCR step along z removes,
    <A z, r>_W^2 / (<A z, A z>_W <r, r>_W); with w (the image of the
    multigrid direction on the same residual), the fraction of what the
    multigrid direction leaves that z removes on top of it: r and A z are
    first made W-orthogonal to w, as the solve's GCR makes them."""
    az = A @ z
    if w is not None:
        r = _wproj_out(r, w, W)
        az = _wproj_out(az, w, W)
    return float((az * r * W).sum() ** 2 / ((az * az * W).sum() * (r * r * W).sum()))


def train_gain(net, problems, n, steps=600, lr=1e-3, warmup=50, log=None):
    """Adam on 1 - gain with gain the fraction of the residual the
    multigrid direction leaves that the network's direction removes on top
    of it (gcr_gain with w): z the network's correction of a residual r
    (out[:, 0:3] times rms h^2 in the reference layout), A z and r made
    W-orthogonal to w = A M r; the gradient with respect to z is A^T of the
    gradient with respect to A z (torch autograd through the projection).
    One residual per step, cycling over problems and iterates.  Returns the
    history of the gain."""
    import torch
    g0 = (n + 1,) * 3
    V = (n + 1) ** 3
    items = [(p, it) for p in problems for it in p["items"]]
    hist = []
    for step in range(steps):
        p, (feat, r, rms, w) = items[step % len(items)]
        W = p["W"]
        out = net.forward(g0, feat)
        scale = rms * p["h2"]
        z = out[:, :3].double().t().reshape(-1) * scale   # reference layout
        az = (p["A"] @ z).detach().requires_grad_(True)
        rp = _wproj_out(r, w, W)
        y = _wproj_out(az, w, W)
        a = (y * rp * W).sum()
        gain = a * a / ((y * y * W).sum() * (rp * rp * W).sum())
        (1.0 - gain).backward()
        hist.append(float(gain.detach()))
        gaz = az.grad if az.grad is not None else torch.zeros_like(az)
        gz = p["At"] @ torch.nan_to_num(gaz)
        dout = torch.zeros(V, FEAT, dtype=torch.float32, device="cuda")
        dout[:, :3] = (gz.reshape(3, V).t() * scale).float()
        gw, gb = net.backward(g0, dout)
        net.adam(gw, gb, lr=lr * min(1.0, (step + 1) / float(warmup)))
        if log and (step + 1) % max(1, steps // 10) == 0:
            log("step %d: mean gain over the last 50 steps %.4f" % (step + 1, float(np.mean(hist[-50:]))))
    return hist
