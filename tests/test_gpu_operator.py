"""GPU: every operator entry point of the C ABI against the oracle on the same
seeded inputs.  Bar: 1e-12 relative (max-norm) for FP64, 1e-5 for FP32."""
import numpy as np
import pytest

import oracle as O
from helpers import random_bc, random_ddw, random_field, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5

# (cells, dx, periodic): small boxes, a box large enough for the shared-memory
# marching kernel and its boundary-shell kernel (n0 >= 128, n1, n2 >= 16), and
# periodic boxes
CASES = [
    ([8, 6, 10], [0.125, 0.2, 0.1], (0, 0, 0)),
    ([128, 16, 18], [1 / 128, 0.06, 0.05], (0, 0, 0)),
    ([8, 6, 10], [0.125, 0.2, 0.1], (1, 0, 1)),
    ([6, 8, 4], [0.2, 0.1, 0.25], (1, 1, 1)),
]
SYMS = [O.ISO, O.MAJORMINOR]


def make(case, sym, seed, bc_types=("disp", "trac", "neumann")):
    from alamo_gb300 import Constant, Elastic
    n, dx, per = case
    bt, bv = random_bc(seed, bc_types)
    g = O.make_grid(n, dx=dx, sym=sym, periodic=per, bc_type=bt, bc_val=bv)
    op = Elastic(n, dx, "isotropic" if sym == O.ISO else "majorminor", per)
    bc = Constant()
    bc.type[:] = bt
    bc.val[:] = bv
    op.SetBC(bc)
    ddw = random_ddw(n, sym, seed + 100, per)
    op.SetModel(ddw)
    return op, g, ddw


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("sym", SYMS)
def test_fapply_f64(gpu_lib, case, sym):
    op, g, ddw = make(case, sym, 1, ("disp", "trac", "neumann", "periodic"))
    u = random_field(case[0], 2, case[2])
    assert rel_err(op.Fapply(0, u), O.fapply(g, ddw, u)) < TOL64


@pytest.mark.parametrize("case", CASES[:2])
@pytest.mark.parametrize("sym", SYMS)
def test_fapply_uniform_flag(gpu_lib, case, sym):
    op, g, ddw = make(case, sym, 3)
    op.SetUniform(True)
    g.uniform = 1
    u = random_field(case[0], 4, case[2])
    assert rel_err(op.Fapply(0, u), O.fapply(g, ddw, u)) < TOL64


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("sym", SYMS)
def test_fapply_f32(gpu_lib, case, sym):
    op, g, ddw = make(case, sym, 5)
    u32 = random_field(case[0], 6, case[2], dtype=np.float32)
    f32 = op.Fapply(0, u32)
    ref = O.fapply(g, ddw.astype(np.float32).astype(np.float64), u32.astype(np.float64))
    assert rel_err(f32.astype(np.float64), ref) < TOL32


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("sym", SYMS)
def test_diagonal(gpu_lib, case, sym):
    op, g, ddw = make(case, sym, 7)
    assert rel_err(op.Diagonal(0), O.diagonal(g, ddw)) < TOL64


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("sym", SYMS)
def test_fsmooth_and_residual(gpu_lib, case, sym):
    op, g, ddw = make(case, sym, 9)
    x = random_field(case[0], 10, case[2])
    b = random_field(case[0], 11, case[2])
    d = O.diagonal(g, ddw)
    ref = O.fsmooth(g, ddw, d, x, b)
    assert rel_err(op.Fsmooth(0, x.copy(), b), ref) < TOL64
    assert rel_err(op.solutionResidual(0, x, b), O.residual(g, ddw, x, b)) < TOL64
    x32, b32 = x.astype(np.float32), b.astype(np.float32)
    ref32 = O.fsmooth(g, ddw.astype(np.float32).astype(np.float64), d, x32.astype(np.float64),
                      b32.astype(np.float64))
    assert rel_err(op.Fsmooth(0, x32.copy(), b32).astype(np.float64), ref32) < 1e-4


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("sym", SYMS)
def test_coarse_levels(gpu_lib, case, sym):
    """averageDownCoeffs, restriction, interpolation and the coarse-level operator."""
    op, g, ddw = make(case, sym, 13)
    if op.NumLevels() < 2:
        pytest.skip("box does not coarsen")
    op.prepareForSolve()
    gc = O.coarsen(g)
    dd1 = O.average_ddw(g, ddw)
    assert rel_err(op.GetModel(1), dd1) < 1e-14
    fine = random_field(case[0], 14, case[2])
    assert rel_err(op.restriction(1, fine), O.restriction(g, fine)) < 1e-14
    crse = random_field(gc.n, 15, case[2])
    assert rel_err(op.interpolation(0, fine.copy(), crse), O.interpolation(g, fine, crse)) < 1e-14
    u1 = random_field(gc.n, 16, case[2])
    assert rel_err(op.Fapply(1, u1), O.fapply(gc, dd1, u1)) < TOL64
    assert rel_err(op.Diagonal(1), O.diagonal(gc, dd1)) < TOL64


def test_newton_rhs_stress_traction(gpu_lib):
    from alamo_gb300 import microstructure as M
    n = [12, 10, 14]
    case = (n, [1 / 12, 0.1, 1 / 14], (0, 0, 0))
    op, g, ddw = make(case, O.MAJORMINOR, 17)
    u = random_field(n, 18)
    b = O.bc_init(g, np.zeros(3 * O.nodes(g)))
    assert rel_err(op.BCInit(np.zeros_like(b)), b) == 0.0
    F0 = np.tile(np.array([1e-3, 2e-4, 0, 2e-4, -1e-3, 0, 0, 0, 5e-4]), O.nodes(g))
    assert rel_err(op.NewtonRHS(u, b, F0), O.newton_rhs(g, ddw, F0, u, b)) < TOL64
    assert rel_err(op.Stress(u, F0), O.stress(g, ddw, F0, u)) < TOL64
    t = op.TractionXhi(u, F0)
    assert rel_err(t, O.traction_xhi(g, ddw, F0, u)) < 1e-12


@pytest.mark.parametrize("sym", SYMS)
@pytest.mark.parametrize("per", [(0, 0, 0), (1, 0, 1)])
def test_strain_energy(gpu_lib, sym, per):
    n = [12, 10, 14]
    op, g, ddw = make((n, [1 / 12, 0.1, 1 / 14], per), sym, 19)
    u = random_field(n, 20, per)
    e, w = op.StrainEnergy(u)
    eo, wo = O.strain_energy(g, ddw, u)
    assert rel_err(e, eo) < TOL64
    assert rel_err(w, wo) < TOL64
    e2, w2 = op.StrainEnergy(u, energy=False)
    assert w2 is None and np.array_equal(e2, e)


# FP32 interiors of large levels go to the TMA kernel: boxes whose x extent is
# not a multiple of its 32-node tile, whose y interior is not a multiple of
# its 8 rows, and whose k interior splits into several chunks.  The smoothing
# check uses displacement rows only: with random traction and Neumann rows
# some boundary diagonals are ~1/h while the interior ones are ~1/h^2, and two
# sweeps from random data amplify FP32 rounding there by that ratio.
BIG32 = [([100, 37, 45], [0.01, 1 / 37, 0.02], (0, 0, 0)), ([64, 20, 24], [1 / 64, 0.05, 1 / 24], (0, 0, 0))]


@pytest.mark.parametrize("case", BIG32)
@pytest.mark.parametrize("sym", SYMS)
@pytest.mark.parametrize("uniform", [False, True])
def test_fp32_interior_apply_and_smooth(gpu_lib, case, sym, uniform):
    op, g, ddw = make(case, sym, 11)
    if uniform:
        op.SetUniform(True)
        g.uniform = 1
    d32 = ddw.astype(np.float32).astype(np.float64)
    u32 = random_field(case[0], 12, case[2], dtype=np.float32)
    ref = O.fapply(g, d32, u32.astype(np.float64))
    assert rel_err(op.Fapply(0, u32).astype(np.float64), ref) < TOL32
    op.close()
    op, g, ddw = make(case, sym, 11, ("disp",))
    if uniform:
        op.SetUniform(True)
        g.uniform = 1
    d32 = ddw.astype(np.float32).astype(np.float64)
    b32 = random_field(case[0], 13, case[2], dtype=np.float32)
    x = op.Fsmooth(0, u32.copy(), b32)
    xs = O.fsmooth(g, d32, O.diagonal(g, d32), u32.astype(np.float64), b32.astype(np.float64))
    assert rel_err(x.astype(np.float64), xs) < TOL32


@pytest.mark.parametrize("sym", SYMS)
def test_pinned_host_fields(gpu_lib, sym):
    """Pinned host fields are read and written in place by the import and
    export kernels (mapped addresses): SetModel, Fapply (FP64 and FP32) and
    Fsmooth from and into pinned host buffers give the same values, bit for
    bit, as from pageable ones."""
    import torch
    case = CASES[1]
    op, g, ddw = make(case, sym, 31)
    N = O.nodes(g)
    rng = np.random.default_rng(32)
    u = rng.uniform(-1, 1, 3 * N)
    b = rng.uniform(-1, 1, 3 * N)

    def pin(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    f_pageable = op.Fapply(0, u)
    f_pinned = pin(np.zeros(3 * N))
    op.Fapply(0, pin(u), out=f_pinned)
    assert np.array_equal(f_pinned, f_pageable)
    x_pageable = op.Fsmooth(0, u.copy(), b)
    x_pinned = pin(u)
    op.Fsmooth(0, x_pinned, pin(b))
    assert np.array_equal(x_pinned, x_pageable)
    op.SetModel(pin(ddw))
    assert np.array_equal(op.GetModel(0), ddw)
    assert np.array_equal(op.Fapply(0, u), f_pageable)
    u32 = u.astype(np.float32)
    f32 = op.Fapply(0, u32)
    f32_pinned = torch.zeros(3 * N, dtype=torch.float32).pin_memory().numpy()
    op.Fapply(0, torch.from_numpy(u32).pin_memory().numpy(), out=f32_pinned)
    assert np.array_equal(f32_pinned, f32)
    op.close()
