"""GPU: full solves through the C ABI against the oracle and against the
reference's known answers.  Bars: FP64 relative residual <= 1e-8 checked by the
oracle's own residual of the GPU solution; displacement within 1e-6 relative
of the oracle solution."""
import numpy as np
import pytest

import oracle as O
from helpers import golden, rel_err, tension_bc_arrays, uniaxial_tension_bc

pytestmark = pytest.mark.gpu


def c1_problem(n=16):
    """Sphere inclusion with eigenstrain, zero displacement on all faces."""
    from alamo_gb300 import microstructure as M
    ddw, F0 = M.sphere_inclusion(n)
    g = O.make_grid([n] * 3, sym=O.ISO)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, F0, np.zeros(3 * N), b)
    return g, ddw, F0, b, rhs


def c2_problem(n=16, ngrains=8):
    from alamo_gb300 import microstructure as M
    ddw, _, _ = M.voronoi_cubic(n, ngrains=ngrains, seed=7)
    bt, bv = tension_bc_arrays(0.01)
    g = O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bt, bc_val=bv)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, None, np.zeros(3 * N), b)
    return g, ddw, None, b, rhs


def gpu_op(g, ddw):
    from alamo_gb300 import Constant, Elastic
    op = Elastic(list(g.n), list(g.dx), "isotropic" if g.sym == O.ISO else "majorminor", list(g.periodic))
    bc = Constant()
    bc.type[:] = np.array([[g.bc_type[f][c] for c in range(3)] for f in range(26)])
    bc.val[:] = np.array([[g.bc_val[f][c] for c in range(3)] for f in range(26)])
    op.SetBC(bc)
    op.SetModel(ddw)
    return op


@pytest.mark.parametrize("problem,fcycle", [(c1_problem, True), (c1_problem, False), (c2_problem, True)])
def test_plain_solve_matches_oracle(gpu_lib, problem, fcycle):
    from alamo_gb300 import Linear
    g, ddw, F0, b, rhs = problem()
    kw = {} if fcycle else {"max_fmg_iter": 0}
    xo, rep_o = O.solve(g, ddw, rhs, tol_rel=1e-8, tol_abs=0.0, params=O.default_params(**kw))
    op = gpu_op(g, ddw)
    sol = Linear(op, **kw)
    x = np.zeros_like(rhs)
    res = sol.solve(x, rhs, 1e-8, 0.0)
    rep = sol.report
    assert rep.status == 0 and rep_o.status == 0
    assert abs(rep.iterations - rep_o.iterations) <= 1, (rep.iterations, rep_o.iterations)
    r = O.residual(g, ddw, x, rhs)
    assert np.abs(r).max() <= 1e-8 * max(np.abs(rhs).max(), rep.res0) * 1.0000001
    assert abs(res - np.abs(r).max()) <= 1e-12 * np.abs(rhs).max()
    assert rel_err(x, xo) < 1e-6


@pytest.mark.parametrize("problem", [c1_problem, c2_problem])
def test_mixed_precision_solve(gpu_lib, problem):
    """FP32 cycles in FP64 refinement reach 1e-10 relative FP64 residual; the
    error against the FP64 oracle solve is reported."""
    from alamo_gb300 import Linear
    g, ddw, F0, b, rhs = problem(32 if problem is c1_problem else 24)
    xo, rep_o = O.solve(g, ddw, rhs, tol_rel=1e-10, tol_abs=0.0)
    op = gpu_op(g, ddw)
    sol = Linear(op, precision=1)
    x = np.zeros_like(rhs)
    sol.solve(x, rhs, 1e-10, 0.0)
    rep = sol.report
    assert rep.status == 0
    r = O.residual(g, ddw, x, rhs)
    assert np.abs(r).max() <= 1e-10 * max(np.abs(rhs).max(), rep.res0) * 1.0000001
    err = rel_err(x, xo)
    print("mixed: cycles %d refinements %d  error vs FP64 oracle %.3e" % (rep.iterations, rep.refinements, err))
    assert err < 1e-6


def test_uniaxial_tension_kat_gpu(gpu_lib):
    from alamo_gb300 import Newton
    gd = golden()["uniaxial_tension"]
    E, nu, L = gd["E"], gd["nu"], gd["L"]
    lam, mu = E * nu / (1 + nu) / (1 - 2 * nu), E / 2 / (1 + nu)
    n = 16
    bt, bv = uniaxial_tension_bc()
    g = O.make_grid([n] * 3, dx=[L / n] * 3, sym=O.ISO, bc_type=bt, bc_val=bv)
    N = O.nodes(g)
    ddw = np.tile([lam, mu], N)
    op = gpu_op(g, ddw)
    b = op.BCInit(np.zeros(3 * N))
    u = np.zeros(3 * N)
    Newton(op).solve(u, b, None, 1e-10, 0.0)
    x = np.arange(n + 1) * L / n - 8
    ux = u[:N].reshape(n + 1, n + 1, n + 1)[n // 2, n // 2, :]
    exact = (x + 8) * gd["disp"] / 16
    assert np.sum((exact - ux) ** 2) / np.sum(exact ** 2) < gd["tolerance"]


@pytest.mark.parametrize("case", ["linear-cubic", "affine-cubic"])
def test_solid_kat_gpu(gpu_lib, case):
    from alamo_gb300 import Newton
    from alamo_gb300 import microstructure as M
    gd = golden()["solid"]
    ref = gd[case]
    m = gd["moduli"]
    C = M.cubic(m["C11"], m["C12"], m["C44"])
    idx = [0, 1, 50, 99]
    for i in idx:
        t = ref["time"][i]
        bt, bv = tension_bc_arrays(0.01 * t)
        g = O.make_grid(gd["n_cells"], sym=O.MAJORMINOR, bc_type=bt, bc_val=bv)
        N = O.nodes(g)
        ddw = np.tile(C, N)
        F0 = np.tile(np.array(gd["affine_F0"]), N) if case.startswith("affine") else None
        op = gpu_op(g, ddw)
        b = op.BCInit(np.zeros(3 * N))
        u = np.zeros(3 * N)
        Newton(op).solve(u, b, F0, 1e-10, 0.0)
        tr = op.TractionXhi(u, F0)[0]
        r = ref["trac_xhi_x"][i]
        assert abs(tr - r) <= gd["tolerance"] * max(abs(r), 1e-3), (t, tr, r)


def test_status_codes(gpu_lib):
    from alamo_gb300 import AgbError, Elastic, Linear
    g, ddw, F0, b, rhs = c1_problem(8)
    op = Elastic([8, 8, 8])
    with pytest.raises(AgbError) as e:
        Linear(op).solve(np.zeros_like(rhs), rhs)
    assert "AGB_STATE" in str(e.value)
    op = gpu_op(g, ddw)
    s = Linear(op, max_iter=1)
    s.solve(np.zeros_like(rhs), rhs, 1e-12, 0.0, raise_on_fail=False)
    assert s.report.status == 1          # AGB_MAXITER
    bad = rhs.copy()
    bad[len(bad) // 2] = np.nan          # fault injected on the host
    s2 = Linear(op)
    with pytest.raises(AgbError) as e:
        s2.solve(np.zeros_like(rhs), bad, 1e-8, 0.0)
    assert "AGB_NAN" in str(e.value)
    with pytest.raises(AgbError) as e:
        op.Fapply(7, np.zeros(10))
    assert "AGB_BADARG" in str(e.value)


@pytest.mark.parametrize("problem,n", [(c1_problem, 32), (c2_problem, 32), (c2_problem, 24)])
def test_mixed_gcr_solve(gpu_lib, problem, n):
    """FP32 cycles under flexible GCR (krylov = 8 stored directions) inside
    FP64 refinement: reaches 1e-10 relative FP64 residual (checked by the
    oracle's residual of the GPU solution) in fewer cycles than the FP32
    cycles alone, and agrees with the FP64 oracle solve."""
    from alamo_gb300 import Linear
    g, ddw, F0, b, rhs = problem(n)
    xo, rep_o = O.solve(g, ddw, rhs, tol_rel=1e-10, tol_abs=0.0)
    op = gpu_op(g, ddw)
    reps = {}
    for kr in (0, 8):
        sol = Linear(op, precision=1, krylov=kr)
        x = np.zeros_like(rhs)
        sol.solve(x, rhs, 1e-10, 0.0)
        reps[kr] = sol.report
        assert sol.report.status == 0
        r = O.residual(g, ddw, x, rhs)
        assert np.abs(r).max() <= 1e-10 * max(np.abs(rhs).max(), sol.report.res0) * 1.0000001
        assert rel_err(x, xo) < 1e-6
    print("cycles: FP32 cycles alone %d, under GCR %d" % (reps[0].iterations, reps[8].iterations))
    assert reps[8].iterations < reps[0].iterations


@pytest.mark.parametrize("problem", [c1_problem, c2_problem])
def test_mixed_exact_bottom(gpu_lib, monkeypatch, problem):
    """The FP32 cycles' coarsest solve by the dense inverse (made once per
    solve) against MLMG's BiCGStab bottom (AGB_BOTTOM_EXACT=0): both reach
    1e-10 by the oracle's residual and agree with the FP64 oracle solve, and
    the exact bottom takes at most one cycle more (a few cycles of a solve
    that needs tens; each of its coarsest solves costs one product)."""
    from alamo_gb300 import Linear
    g, ddw, F0, b, rhs = problem(32)
    xo, rep_o = O.solve(g, ddw, rhs, tol_rel=1e-10, tol_abs=0.0)
    cycles = {}
    for exact in ("1", "0"):
        monkeypatch.setenv("AGB_BOTTOM_EXACT", exact)
        op = gpu_op(g, ddw)
        sol = Linear(op, precision=1, krylov=8)
        x = np.zeros_like(rhs)
        sol.solve(x, rhs, 1e-10, 0.0)
        assert sol.report.status == 0
        r = O.residual(g, ddw, x, rhs)
        assert np.abs(r).max() <= 1e-10 * max(np.abs(rhs).max(), sol.report.res0) * 1.0000001
        assert rel_err(x, xo) < 1e-6
        cycles[exact] = sol.report.iterations
        sol.Clear()
        op.close()
    print("cycles: exact bottom %d, BiCGStab bottom %d" % (cycles["1"], cycles["0"]))
    assert cycles["1"] <= cycles["0"] + 1


def test_mixed_gcr_rejects_bad_krylov(gpu_lib):
    from alamo_gb300 import AgbError, Linear
    g, ddw, F0, b, rhs = c1_problem(8)
    op = gpu_op(g, ddw)
    for kr in (-1, 17):
        with pytest.raises(AgbError):
            Linear(op, precision=1, krylov=kr)
