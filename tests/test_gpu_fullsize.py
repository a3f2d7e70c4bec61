"""GPU: parity at the benchmark sizes, through the C ABI, with the oracle as
the checker.

  * C1, 65^3 nodes (sphere inclusion with eigenstrain, zero displacement on
    every face): the plain FP64 solve in F- and V-cycles against the oracle's
    solve (iterations within one, displacement within 1e-6 relative, the
    oracle's residual of the GPU solution at 1e-8), and the mixed solve
    (FP32 F-cycles under GCR(8) in FP64 refinement) against the same.
  * C2, 257^3 nodes (64-grain cubic Voronoi polycrystal, TensionTest
    uniaxial_stress u_x = 0.01): Fapply, the residual, Fsmooth and Diagonal in
    FP64 against the oracle at 1e-12 relative, the FP32 Fapply at 1e-5; the
    benchmark's mixed solve to 1e-8 and C3's mixed solve to 1e-10 checked by
    the oracle's residual; every GPU solution within 1e-6 relative of the
    oracle's complete FP64 solve of the same system (F-cycles, 1e-8).
  * The reference's tests/Eshelby known answer at 256^3 cells on one level
    through agb_newton_solve and agb_stress: the reference script's six
    metrics (relative L2 of u, relative 1-norm of the normal stresses) within
    its tolerance 0.1.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from helpers import eshelby_errors, rel_err

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL_OP64 = 1e-12     # FP64 operator parity (relative to max |oracle|)
TOL_OP32 = 1e-5      # FP32 operator parity
TOL_U = 1e-6         # displacement, relative max norm


def _gpu_op(n, dx, sym, bc, ddw):
    from alamo_gb300 import Elastic
    op = Elastic([n] * 3, dx, sym)
    op.SetBC(bc)
    op.SetModel(ddw)
    return op


def _oracle_res_rel(g, ddw, x, rhs, res0):
    r = O.residual(g, ddw, x, rhs)
    return float(np.abs(r).max() / max(float(np.abs(rhs).max()), res0))


# ---------------------------------------------------------------------------
# C1: 65^3 nodes
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("fcycle", [True, False])
def test_c1_65_solves_match_oracle(gpu_lib, fcycle):
    from alamo_gb300 import Constant, Linear
    from alamo_gb300 import microstructure as M
    n = 64
    ddw, F0 = M.sphere_inclusion(n)
    g = O.make_grid([n] * 3, sym=O.ISO)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, F0, np.zeros(3 * N), b)
    kw = {} if fcycle else {"max_fmg_iter": 0}
    xo, rep_o = O.solve(g, ddw, rhs, tol_rel=1e-8, tol_abs=0.0, params=O.default_params(**kw))
    assert rep_o.status == 0
    op = _gpu_op(n, None, "isotropic", Constant(), ddw)
    # the GPU computes the same right-hand side
    assert rel_err(op.NewtonRHS(np.zeros(3 * N), b, F0=F0), rhs) < TOL_OP64
    plain = Linear(op, **kw)
    x = np.zeros(3 * N)
    plain.solve(x, rhs, 1e-8, 0.0)
    rep = plain.report
    assert rep.status == 0 and abs(rep.iterations - rep_o.iterations) <= 1, (rep.iterations, rep_o.iterations)
    assert _oracle_res_rel(g, ddw, x, rhs, rep.res0) <= 1e-8 * 1.000001
    assert rel_err(x, xo) < TOL_U
    mixed = Linear(op, precision=1, krylov=8, **kw)
    xm = np.zeros(3 * N)
    mixed.solve(xm, rhs, 1e-8, 0.0)
    assert mixed.report.status == 0
    assert _oracle_res_rel(g, ddw, xm, rhs, mixed.report.res0) <= 1e-8 * 1.000001
    assert rel_err(xm, xo) < TOL_U
    plain.Clear()
    mixed.Clear()
    op.close()


# ---------------------------------------------------------------------------
# C2 / C3: 257^3 nodes
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c2():
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import TensionTest
    n = 256
    ddw, _, _ = M.voronoi_cubic(n, ngrains=64, seed=20260)
    bc = TensionTest("uniaxial_stress", disp=0.01)
    g = O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bc.type, bc_val=bc.val)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, None, np.zeros(3 * N), b)
    op = _gpu_op(n, None, "majorminor", bc, ddw)
    state = {"n": n, "ddw": ddw, "bc": bc, "g": g, "N": N, "b": b, "rhs": rhs, "op": op}
    yield state
    op.close()


def _oracle_solution(c2):
    if "xo" not in c2:
        xo, rep = O.solve(c2["g"], c2["ddw"], c2["rhs"], tol_rel=1e-8, tol_abs=0.0)
        assert rep.status == 0
        c2["xo"], c2["rep_o"] = xo, rep
    return c2["xo"], c2["rep_o"]


def test_c2_257_operator_parity(gpu_lib, c2):
    g, ddw, op, N = c2["g"], c2["ddw"], c2["op"], c2["N"]
    rng = np.random.default_rng(257)
    u = rng.uniform(-1, 1, 3 * N)
    f = O.fapply(g, ddw, u)
    assert rel_err(op.Fapply(0, u), f) < TOL_OP64
    bvec = rng.uniform(-1, 1, 3 * N)
    r = O.residual(g, ddw, u, bvec)
    assert rel_err(op.solutionResidual(0, u, bvec), r) < TOL_OP64
    d = O.diagonal(g, ddw)
    assert rel_err(op.Diagonal(0), d) < TOL_OP64
    xs = O.fsmooth(g, ddw, d, u, bvec)
    assert rel_err(op.Fsmooth(0, u.copy(), bvec), xs) < TOL_OP64
    f32 = op.Fapply(0, u.astype(np.float32))
    assert rel_err(f32.astype(np.float64), f) < TOL_OP32
    # the right-hand side of the benchmark solve
    assert rel_err(op.NewtonRHS(np.zeros(3 * N), c2["b"]), c2["rhs"]) < TOL_OP64


def test_c2_257_solutions_match_oracle(gpu_lib, c2):
    """The plain FP64 GPU multigrid, the benchmark's mixed solve (FP32
    F-cycles under GCR(8) in FP64 refinement, 1e-8) and C3's mixed solve
    (FP32 F-cycles in FP64 refinement, 1e-10): residuals checked by the
    oracle, displacements against the oracle's complete FP64 solve."""
    from alamo_gb300 import Linear
    g, ddw, op, N, rhs = c2["g"], c2["ddw"], c2["op"], c2["N"], c2["rhs"]
    plain = Linear(op)
    xp = np.zeros(3 * N)
    plain.solve(xp, rhs, 1e-8, 0.0)
    rp = plain.report
    assert rp.status == 0
    plain.Clear()
    assert _oracle_res_rel(g, ddw, xp, rhs, rp.res0) <= 1e-8 * 1.000001
    bench = Linear(op, precision=1, krylov=8)
    xm = np.zeros(3 * N)
    bench.solve(xm, rhs, 1e-8, 0.0)
    assert bench.report.status == 0
    bench.Clear()
    assert _oracle_res_rel(g, ddw, xm, rhs, bench.report.res0) <= 1e-8 * 1.000001
    assert rel_err(xm, xp) < TOL_U
    c3 = Linear(op, precision=1)
    x3 = np.zeros(3 * N)
    c3.solve(x3, rhs, 1e-10, 0.0)
    assert c3.report.status == 0
    c3.Clear()
    assert _oracle_res_rel(g, ddw, x3, rhs, c3.report.res0) <= 1e-10 * 1.000001
    xo, rep_o = _oracle_solution(c2)
    assert abs(rp.iterations - rep_o.iterations) <= 1, (rp.iterations, rep_o.iterations)
    for name, x in (("plain", xp), ("mixed GCR(8) 1e-8", xm), ("mixed 1e-10", x3)):
        e = rel_err(x, xo)
        print("C2 257^3 %s: displacement error against the oracle %.3e" % (name, e))
        assert e < TOL_U, (name, e)


# ---------------------------------------------------------------------------
# tests/Eshelby at 256^3 cells through the GPU
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("precision", [0, 1])
def test_eshelby_kat_gpu_256(gpu_lib, precision):
    from alamo_gb300 import Constant, Newton
    from alamo_gb300 import microstructure as M
    gd = json.load(open(os.path.join(HERE, "golden", "eshelby_kat.json")))
    n = 256
    L = gd["prob_hi"][0] - gd["prob_lo"][0]
    h = L / n
    ddw, F0 = M.eshelby_problem(n, gd)
    N = (n + 1) ** 3
    op = _gpu_op(n, [h] * 3, "isotropic", Constant(), ddw)
    newton = Newton(op, precision=precision, krylov=8 if precision else 0)
    u = np.zeros(3 * N)
    newton.solve(u, np.zeros(3 * N), F0=F0, tol_rel=1e-8, tol_abs=0.0)
    assert newton.report.status == 0
    sig = op.Stress(u, F0=F0)
    newton.Clear()
    op.close()
    i = int(round((gd["ray"]["x"] - gd["prob_lo"][0]) / h))
    assert abs(gd["prob_lo"][0] + i * h - gd["ray"]["x"]) < 1e-12   # the ray runs along a node line
    z = gd["prob_lo"][2] + np.arange(n + 1) * h
    sel = (z >= gd["ray"]["z"][0] - 1e-12) & (z <= gd["ray"]["z"][1] + 1e-12)
    U = u.reshape(3, n + 1, n + 1, n + 1)[:, :, i, i]
    S = sig.reshape(n + 1, n + 1, n + 1, 9)[:, i, i, :]
    err = eshelby_errors(gd, z[sel], [U[c][sel] for c in range(3)], [S[sel, 0], S[sel, 4], S[sel, 8]])
    print("Eshelby errors at 256^3 on the GPU (precision %d):" % precision, {k: round(v, 4) for k, v in err.items()})
    for k, v in err.items():
        assert v <= gd["tolerance"], (k, v)
