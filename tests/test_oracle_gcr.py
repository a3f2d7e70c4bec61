"""CPU: the Krylov acceleration the mixed solve uses (flexible GCR whose
directions are one multigrid cycle of the residual, inner product weighted by
1/diag^2), restated in numpy over the oracle's F-cycle and operator, on a 16^3
cubic polycrystal under tension: it reaches 1e-8 in well under half the
cycles the cycles alone need (41)."""
import numpy as np

import oracle as O
from helpers import tension_bc_arrays


def test_weighted_gcr_over_oracle_cycles():
    from alamo_gb300 import microstructure as M
    n = 16
    ddw, _, _ = M.voronoi_cubic(n, ngrains=8, seed=7)
    bt, bv = tension_bc_arrays(0.01)
    g = O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bt, bc_val=bv)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, None, np.zeros(3 * N), b)
    _, rep = O.solve(g, ddw, rhs, tol_rel=1e-8, tol_abs=0.0)
    one_cycle = O.default_params(max_iter=1)
    d = O.diagonal(g, ddw)
    wt = np.where(d != 0, 1.0 / d, 0.0) ** 2

    def ip(a, c):
        return float(np.dot(a * wt, c))

    x = np.zeros_like(rhs)
    r = rhs.copy()
    Z, W = [], []
    target = 1e-8 * np.abs(rhs).max()
    cycles = 0
    for it in range(rep.iterations):
        z, _ = O.solve(g, ddw, r, x0=np.zeros_like(r), tol_rel=0.0, tol_abs=0.0, params=one_cycle)
        cycles += 1
        w = O.fapply(g, ddw, z)
        if len(Z) == 8:
            Z, W = [], []
        for Zi, Wi in zip(Z, W):
            beta = ip(w, Wi)
            w = w - beta * Wi
            z = z - beta * Zi
        nw = np.sqrt(ip(w, w))
        w, z = w / nw, z / nw
        a = ip(r, w)
        r_next = r - a * w
        # each step lowers the weighted residual norm
        assert ip(r_next, r_next) <= ip(r, r) * (1 + 1e-12)
        x += a * z
        r = r_next
        Z.append(z)
        W.append(w)
        if np.abs(r).max() <= target:
            break
    assert np.abs(r).max() <= target
    assert np.abs(O.residual(g, ddw, x, rhs)).max() <= 1.0001 * target
    assert cycles < rep.iterations / 2, (cycles, rep.iterations)
