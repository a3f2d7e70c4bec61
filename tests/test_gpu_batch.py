"""GPU: batched periodic RVE solves (agb_batch_*) against the oracle and the
single-box GPU solver on the same problems.  A fully periodic box is singular
(rigid translations): the solve works with the zero-mean parts of the
right-hand side and of the residual, and returns a zero-mean displacement."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def small_rves(sizes, seed=3):
    from alamo_gb300 import microstructure as M
    out = []
    for q, n in enumerate(sizes):
        _, ddw, F0 = M.rve_problem(q, seed=seed, edges=(n,))
        out.append((n, ddw, F0))
    return out


def oracle_solution(n, ddw, F0, tol, vcycle=True):
    g = O.make_grid([n] * 3, sym=O.ISO, periodic=(1, 1, 1))
    N = O.nodes(g)
    F0n = np.tile(np.asarray(F0).reshape(9), N)
    rhs = O.newton_rhs(g, ddw, F0n, np.zeros(3 * N), np.zeros(3 * N))
    p = O.default_params(max_fmg_iter=0) if vcycle else O.default_params()
    x, rep = O.solve(g, ddw, rhs, tol_rel=tol, tol_abs=0.0, params=p)
    return g, rhs, x, rep


def zero_mean(u, n):
    a = u.reshape(3, n + 1, n + 1, n + 1)
    m = a[:, :n, :n, :n].reshape(3, -1).mean(axis=1)
    return (a - m[:, None, None, None]).reshape(-1)


def projected_residual_ratio(g, ddw, u, rhs, n):
    """||P(P b - A u)||_inf / ||P b||_inf, P the zero-mean projection."""
    pb = zero_mean(rhs, n)
    r = zero_mean(O.residual(g, ddw, u, pb), n)
    return np.abs(r).max() / np.abs(pb).max()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_oracle(gpu_lib, precision):
    from alamo_gb300.batch import Batch
    sizes = [8, 12, 16, 8]
    probs = small_rves(sizes)
    bt = Batch([(n, n, n) for n in sizes], precision=precision)
    for q, (n, ddw, F0) in enumerate(probs):
        bt.SetModel(q, ddw)
    bt.SetEigenstrain(np.stack([p[2] for p in probs]))
    tot = bt.solve(1e-8, 0.0)
    assert tot.status == 0
    for q, (n, ddw, F0) in enumerate(probs):
        g, rhs, xo, rep_o = oracle_solution(n, ddw, F0, 1e-8)
        u = bt.solution(q)
        ratio = projected_residual_ratio(g, ddw, u, rhs, n)
        assert ratio <= 1e-8 * 1.00001, (q, ratio)
        assert np.abs(zero_mean(u, n) - u).max() <= 1e-12 * np.abs(u).max()
        err = np.abs(u - xo).max() / np.abs(xo).max()
        assert err < 1e-6, (q, err)
        if precision == 0:
            assert abs(bt.reports[q].iterations - rep_o.iterations) <= 1, (q, bt.reports[q].iterations,
                                                                          rep_o.iterations)
    s = bt.mean_stress()
    assert np.all(np.isfinite(s)) and np.allclose(s, np.transpose(s, (0, 2, 1)), atol=1e-12)
    for l in range(2):
        assert bt.tuning(l) in [(32, 4, 2), (32, 8, 1), (16, 8, 2), (8, 8, 4), (64, 4, 1), (32, 8, 16)]
    bt.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_march_kernel(gpu_lib, monkeypatch, precision):
    """The marching tile kernel (32 x 8 columns through 16 planes, fully
    periodic isotropic batches) forced on every level against the
    node-per-thread kernel: the same solutions, and within the oracle's
    tolerance on partial tiles in every direction (edges 40, 24, 12)."""
    from alamo_gb300.batch import Batch
    sizes = [40, 24, 12]
    probs = small_rves(sizes, seed=5)
    sols, iters = {}, {}
    for shape, dims in ((0, (32, 4, 2)), (5, (32, 8, 16))):
        monkeypatch.setenv("AGB_BATCH_SHAPE", str(shape))
        bt = Batch([(n, n, n) for n in sizes], precision=precision)
        for q, (n, ddw, F0) in enumerate(probs):
            bt.SetModel(q, ddw)
        bt.SetEigenstrain(np.stack([p[2] for p in probs]))
        assert bt.solve(1e-8, 0.0).status == 0
        for l in range(2):
            assert bt.tuning(l) == dims
        sols[shape] = [bt.solution(q) for q in range(len(sizes))]
        iters[shape] = [bt.reports[q].iterations for q in range(len(sizes))]
        bt.close()
    tol = 1e-10 if precision == 0 else 1e-6
    for q, (n, ddw, F0) in enumerate(probs):
        a, b = sols[5][q], sols[0][q]
        assert np.abs(a - b).max() <= tol * np.abs(b).max(), q
        assert abs(iters[5][q] - iters[0][q]) <= 1, (q, iters)
    n, ddw, F0 = probs[0]
    g, rhs, xo, rep_o = oracle_solution(n, ddw, F0, 1e-8)
    assert projected_residual_ratio(g, ddw, sols[5][0], rhs, n) <= 1e-8 * 1.00001
    assert np.abs(sols[5][0] - xo).max() / np.abs(xo).max() < 1e-6


def test_single_box_periodic_matches_oracle(gpu_lib):
    """The single-box path on a fully periodic box: same projection of the null space."""
    from alamo_gb300 import Elastic, Linear
    n, ddw, F0 = small_rves([12], seed=9)[0]
    g, rhs, xo, rep_o = oracle_solution(n, ddw, F0, 1e-9)
    op = Elastic([n] * 3, None, "isotropic", periodic=(1, 1, 1))
    from alamo_gb300 import Constant
    op.SetBC(Constant())
    op.SetModel(ddw)
    x = np.zeros_like(rhs)
    s = Linear(op, max_fmg_iter=0)
    s.solve(x, rhs, 1e-9, 0.0)
    assert abs(s.report.iterations - rep_o.iterations) <= 1
    err = np.abs(x - xo).max() / np.abs(xo).max()
    assert err < 1e-6, err


def test_single_box_periodic_gcr(gpu_lib):
    """The GCR-accelerated mixed solve on a fully periodic box: the GCR
    directions are projected to zero mean like the residuals, and the solve
    reaches the oracle's solution."""
    from alamo_gb300 import Constant, Elastic, Linear
    n, ddw, F0 = small_rves([16], seed=11)[0]
    g, rhs, xo, rep_o = oracle_solution(n, ddw, F0, 1e-9)
    op = Elastic([n] * 3, None, "isotropic", periodic=(1, 1, 1))
    op.SetBC(Constant())
    op.SetModel(ddw)
    x = np.zeros_like(rhs)
    s = Linear(op, precision=1, krylov=8)
    s.solve(x, rhs, 1e-9, 0.0)
    assert s.report.status == 0
    assert projected_residual_ratio(g, ddw, x, rhs, n) <= 1e-9 * 1.00001
    err = np.abs(x - xo).max() / np.abs(xo).max()
    assert err < 1e-6, err


def test_batch_gcr_matches_oracle(gpu_lib):
    """The batched mixed solve with a per-problem GCR over the FP32 V-cycle
    (krylov = 8): every problem converges to the oracle's solution, in no more
    cycles than the FP32 cycles alone need."""
    from alamo_gb300.batch import Batch
    sizes = [8, 12, 16, 24]
    probs = small_rves(sizes, seed=13)
    cyc = {}
    for kr in (0, 8):
        bt = Batch([(n, n, n) for n in sizes], precision=1, krylov=kr)
        for q, (n, ddw, F0) in enumerate(probs):
            bt.SetModel(q, ddw)
        bt.SetEigenstrain(np.stack([p[2] for p in probs]))
        assert bt.solve(1e-8, 0.0).status == 0
        cyc[kr] = [bt.reports[q].iterations for q in range(len(sizes))]
        if kr:
            for q, (n, ddw, F0) in enumerate(probs):
                g, rhs, xo, rep_o = oracle_solution(n, ddw, F0, 1e-8)
                u = bt.solution(q)
                assert projected_residual_ratio(g, ddw, u, rhs, n) <= 1e-8 * 1.00001, q
                assert np.abs(u - xo).max() / np.abs(xo).max() < 1e-6, q
        bt.close()
    print("cycles per problem: alone %s, under GCR %s" % (cyc[0], cyc[8]))
    assert max(cyc[8]) <= max(cyc[0])
