"""GPU: the allocation-free bottom solve (agb_bottom_solve_noalloc).

Callers that may not allocate device memory when they need a coarsest-level
solve (a framework that owns every device byte through its own arena, or a
time-stepping code that must not stall on cudaMalloc in the middle of a step)
use this entry point; its work vectors live in a fixed device array of the
library.  These tests call it through the C ABI twice in a row on device
buffers and check each result against the existing entry point that performs
the same computation (agb_solve on a one-level operator with exactly one
iteration, whose single cycle is the bottom solve) and, on a cubic
polycrystal, against the oracle's bottom step.  They also check that a box
above the array's size limit, a periodic BC type and an in-place call
(res == cor) are refused.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12          # against the existing entry point (same kernel, same rounding)
TOL_ORACLE = 1e-7    # against the oracle's converged (1e-12) bottom solve


def problem(n):
    from alamo_gb300 import microstructure as M
    from alamo_gb300.elastic import TensionTest
    ddw, F0 = M.sphere_inclusion(n)
    bc = TensionTest("uniaxial_stress", disp=0.01)
    g = O.make_grid([n] * 3, sym=O.ISO, bc_type=bc.type, bc_val=bc.val)
    N = O.nodes(g)
    b = O.bc_init(g, np.zeros(3 * N))
    rhs = O.newton_rhs(g, ddw, F0, np.zeros(3 * N), b)
    return ddw, bc, rhs


def call_noalloc(n, ddw_soa, diag, rhs, bc, params, out, ret, sym=None):
    from alamo_gb300 import _lib
    L = _lib.lib()
    return L.agb_bottom_solve_noalloc(
        (ctypes.c_int * 3)(n, n, n), (ctypes.c_double * 3)(1.0 / n, 1.0 / n, 1.0 / n),
        _lib.AGB_ISO if sym is None else sym, 0,
        ctypes.byref(bc.to_c()), ctypes.c_void_p(ddw_soa.data_ptr()), ctypes.c_void_p(diag.data_ptr()),
        ctypes.c_void_p(rhs.data_ptr()), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ret.data_ptr()),
        params.bottom_max_iter, params.bottom_tol_rel, params.bottom_tol_abs, params.bottom_smooth,
        params.final_smooth, 2.0 / 3.0, None)


def test_noalloc_bottom_matches_existing_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    from alamo_gb300 import Elastic, Linear, default_params
    from alamo_gb300._lib import AGB_OK, check
    n = 8
    ddw, bc, rhs = problem(n)
    op = Elastic([n] * 3, None, "isotropic", max_coarsening_level=0)
    assert op.NumLevels() == 1
    op.SetBC(bc)
    op.SetModel(ddw)
    # existing entry point: one MLMG iteration of a one-level hierarchy = one bottom solve
    ref = np.zeros_like(rhs)
    s = Linear(op, fixed_iter=1, max_iter=1)
    s.solve(ref, rhs, 1e-30, 0.0)
    assert s.report.iterations == 1
    diag = op.Diagonal(0)
    N = (n + 1) ** 3
    ddw_soa = np.ascontiguousarray(op.GetModel(0).reshape(N, 2).T).reshape(-1)
    d_ddw = torch.from_numpy(ddw_soa).cuda()
    d_diag = torch.from_numpy(diag).cuda()
    d_rhs = torch.from_numpy(rhs).cuda()
    d_ret = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    p = default_params()
    for call in range(2):
        d_out = torch.full((3 * N,), float("nan"), dtype=torch.float64, device="cuda")
        check(call_noalloc(n, d_ddw, d_diag, d_rhs, bc, p, d_out, d_ret))
        torch.cuda.synchronize()
        out = d_out.cpu().numpy()
        assert int(d_ret.item()) in (0, 8)
        err = np.abs(out - ref).max() / np.abs(ref).max()
        assert err < TOL, (call, err)
    s.Clear()
    op.close()


def test_noalloc_rejects_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    from alamo_gb300 import default_params
    from alamo_gb300._lib import AGB_BADARG
    from alamo_gb300.elastic import Constant
    n = 17  # 18^3 nodes > AGB_NOALLOC_MAX_NODES
    N = (n + 1) ** 3
    z = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
    zc = torch.zeros(2 * N, dtype=torch.float64, device="cuda")
    r = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert call_noalloc(n, zc, z, z, Constant(), default_params(), z, r) == AGB_BADARG


def test_noalloc_rejects_periodic_and_in_place(gpu_lib):
    torch = pytest.importorskip("torch")
    from alamo_gb300 import default_params
    from alamo_gb300._lib import AGB_BADARG
    from alamo_gb300.elastic import Constant
    n = 4
    N = (n + 1) ** 3
    z = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
    c = torch.zeros(3 * N, dtype=torch.float64, device="cuda")
    zc = torch.zeros(2 * N, dtype=torch.float64, device="cuda")
    r = torch.zeros(1, dtype=torch.int32, device="cuda")
    bc = Constant()
    bc.type[0, 1] = O.PERIODIC
    assert call_noalloc(n, zc, z, z, bc, default_params(), c, r) == AGB_BADARG
    assert call_noalloc(n, zc, z, z, Constant(), default_params(), z, r) == AGB_BADARG


@pytest.mark.parametrize("tol", [1e-4, 1e-12])
def test_noalloc_bottom_matches_oracle_cubic(gpu_lib, tol):
    """A cubic (MajorMinor) polycrystal box with TensionTest rows, twice in a
    row.  At the default bottom tolerance (1e-4) two BiCGStab runs that sum
    in different orders stop on different iterates, so the check is the
    oracle's residual of the GPU correction (the diagonally scaled residual
    reduced by the tolerance); at 1e-12 both runs converge to the solution of
    the same system and the corrections agree with the oracle's."""
    torch = pytest.importorskip("torch")
    from alamo_gb300 import default_params
    from alamo_gb300 import microstructure as M
    from alamo_gb300._lib import AGB_MAJORMINOR, check
    from alamo_gb300.elastic import TensionTest
    n = 8
    N = (n + 1) ** 3
    ddw, _, _ = M.voronoi_cubic(n, ngrains=6, seed=11)
    bc = TensionTest("uniaxial_stress", disp=0.01)
    g = O.make_grid([n] * 3, sym=O.MAJORMINOR, bc_type=bc.type, bc_val=bc.val)
    diag = O.diagonal(g, ddw)
    res = np.random.default_rng(5).uniform(-1, 1, 3 * N)
    params = default_params(bottom_tol_rel=tol, bottom_max_iter=400)
    ref, ret_o = O.bottom_solve(g, ddw, diag, res, O.default_params(bottom_tol_rel=tol, bottom_max_iter=400))
    ddw_soa = np.ascontiguousarray(ddw.reshape(N, 21).T).reshape(-1)
    d_ddw = torch.from_numpy(ddw_soa).cuda()
    d_diag = torch.from_numpy(diag).cuda()
    d_res = torch.from_numpy(res).cuda()
    d_ret = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    for call in range(2):
        d_out = torch.full((3 * N,), float("nan"), dtype=torch.float64, device="cuda")
        check(call_noalloc(n, d_ddw, d_diag, d_res, bc, params, d_out, d_ret, sym=AGB_MAJORMINOR))
        torch.cuda.synchronize()
        assert int(d_ret.item()) == ret_o == 0, (call, int(d_ret.item()), ret_o)
        cor = d_out.cpu().numpy()
        r = O.residual(g, ddw, cor, res)
        # (the recursively updated BiCGStab residual drifts from the true one
        # near 1e-12, so the true residual is held to 1e-10 there)
        assert np.abs(r / diag).max() <= max(tol, 1e-10) * np.abs(res / diag).max() * 1.001, call
        if tol < 1e-10:
            err = np.abs(cor - ref).max() / np.abs(ref).max()
            assert err < TOL_ORACLE, (call, err)
