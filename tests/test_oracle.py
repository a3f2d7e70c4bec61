"""CPU: the oracle against the reference's own known answers, plus
self-consistency checks of the restated operator.  No GPU."""
import numpy as np
import pytest

import oracle as O
from helpers import (golden, nodes, random_bc, random_ddw, random_field, rel_err, tension_bc_arrays,
                     uniaxial_tension_bc)


def test_uniaxial_tension_analytic():
    """tests/UniaxialTension: u_x = (x+8) 0.1/16, sigma_xx = E 0.1/16, relative L2 error < 1e-8."""
    g = golden()["uniaxial_tension"]
    E, nu, L = g["E"], g["nu"], g["L"]
    lam, mu = E * nu / (1 + nu) / (1 - 2 * nu), E / 2 / (1 + nu)
    n = 16
    bt, bv = uniaxial_tension_bc()
    grid = O.make_grid([n] * 3, dx=[L / n] * 3, sym=O.ISO, bc_type=bt, bc_val=bv)
    N = O.nodes(grid)
    ddw = np.tile([lam, mu], N)
    b = O.bc_init(grid, np.zeros(3 * N))
    u, rep = O.newton_solve(grid, ddw, None, np.zeros(3 * N), b, 1e-10, 0.0)
    assert rep.status == 0
    x = np.arange(n + 1) * L / n - 8
    ux = u[:N].reshape(n + 1, n + 1, n + 1)[n // 2, n // 2, :]
    exact = (x + 8) * g["disp"] / 16
    assert np.sum((exact - ux) ** 2) / np.sum(exact ** 2) < g["tolerance"]
    s = O.stress(grid, ddw, None, u).reshape(n + 1, n + 1, n + 1, 3, 3)[n // 2, n // 2, :, 0, 0]
    sx = E * g["disp"] / L
    assert np.sum((s - sx) ** 2) / np.sum(np.full_like(s, sx) ** 2) < g["tolerance"]


@pytest.mark.parametrize("case", ["linear-cubic", "affine-cubic"])
def test_solid_kat(case):
    """tests/Solid: trac_xhi_x(t) against the reference's golden file with the
    reference test's own metric (time-integrated relative L2 < 1e-4)."""
    gd = golden()["solid"]
    ref = gd[case]
    m = gd["moduli"]
    C = O.cubic(m["C11"], m["C12"], m["C44"])
    F0v = np.array(gd["affine_F0"]) if case.startswith("affine") else None
    times = np.array(ref["time"])
    trac = []
    for t in times:
        bt, bv = tension_bc_arrays(0.01 * t)
        grid = O.make_grid(gd["n_cells"], sym=O.MAJORMINOR, bc_type=bt, bc_val=bv)
        N = O.nodes(grid)
        ddw = np.tile(C, N)
        F0 = np.tile(F0v, N) if F0v is not None else None
        b = O.bc_init(grid, np.zeros(3 * N))
        u, rep = O.newton_solve(grid, ddw, F0, np.zeros(3 * N), b, 1e-10, 0.0)
        assert rep.status == 0
        trac.append(O.traction_xhi(grid, ddw, F0, u)[0])
    trac = np.array(trac)
    r = np.array(ref["trac_xhi_x"])

    def integrate(x, y):
        return np.sum(0.5 * (y[1:] + y[:-1]) * (x[1:] - x[:-1]))

    err = np.sqrt(integrate(times, (r - trac) ** 2)) / np.sqrt(integrate(times, r * r))
    assert err < gd["tolerance"], err


def test_cubic_builder_identity_and_rotation():
    c = O.cubic(168.3, 1.221, 0.757)
    assert c[0] == 168.3 and c[15] == 168.3 and c[20] == 168.3
    assert c[3] == 1.221 and c[5] == 1.221 and c[17] == 1.221
    assert c[6] == 0.757 and c[11] == 0.757 and c[18] == 0.757
    from alamo_gb300 import microstructure as M
    for seed in range(4):
        r = M.SplitMix64(seed)
        q = [r.normal() for _ in range(4)]
        R = O.quat_to_rot(q)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-14)
        assert rel_err(M.cubic(1.68, 1.21, 0.75, M.quat_to_rot(q)), O.cubic(1.68, 1.21, 0.75, R)) < 1e-13


def test_fapply_linear_field_interior_zero():
    """Uniform C, u linear in x: every interior row vanishes; DISP rows return u."""
    n = [6, 5, 7]
    bt = np.zeros((26, 3), np.int32)
    g = O.make_grid(n, sym=O.MAJORMINOR, bc_type=bt)
    N = O.nodes(g)
    ddw = np.tile(O.cubic(1.68, 1.21, 0.75), N)
    z, y, x = np.meshgrid(*[np.arange(m + 1) / m for m in n[::-1]], indexing="ij")
    u = np.concatenate([(0.1 * x + 0.2 * y - 0.3 * z).ravel(), (0.05 * x - z).ravel(), (y + 0.5).ravel()])
    f = O.fapply(g, ddw, u).reshape(3, n[2] + 1, n[1] + 1, n[0] + 1)
    assert np.abs(f[:, 1:-1, 1:-1, 1:-1]).max() < 1e-12
    uu = u.reshape(3, n[2] + 1, n[1] + 1, n[0] + 1)
    assert np.allclose(f[:, 0], uu[:, 0]) and np.allclose(f[:, :, :, -1], uu[:, :, :, -1])


@pytest.mark.parametrize("sym", [O.ISO, O.MAJORMINOR])
def test_diagonal_equals_probe(sym):
    """Elastic::Diagonal (analytic) equals the diagonal of Fapply probed with unit
    vectors (the generic Operator<Node>::Diagonal, Operator.cpp:31-86)."""
    n = [3, 2, 4]
    bt, bv = random_bc(7)
    g = O.make_grid(n, sym=sym, bc_type=bt, bc_val=bv, dx=[0.3, 0.5, 0.25])
    N = O.nodes(g)
    ddw = random_ddw(n, sym, 3)
    d = O.diagonal(g, ddw)
    probe = np.zeros(3 * N)
    for q in range(3 * N):
        e = np.zeros(3 * N)
        e[q] = 1.0
        probe[q] = O.fapply(g, ddw, e)[q]
    assert rel_err(d, probe) < 1e-13


def test_transfers_constant_fields():
    n = [8, 4, 6]
    g = O.make_grid(n)
    N = O.nodes(g)
    c = O.restriction(g, np.full(3 * N, 2.5))
    assert np.allclose(c, 2.5)
    gc = O.coarsen(g)
    f = O.interpolation(g, np.ones(3 * N), np.full(3 * O.nodes(gc), 0.5))
    assert np.allclose(f, 1.5)
    dd = O.average_ddw(g, np.tile([3.0, 4.0], N))
    assert np.allclose(dd.reshape(-1, 2), [3.0, 4.0])


def test_fsmooth_fixed_point():
    n = [6, 6, 5]
    bt, bv = random_bc(11)
    g = O.make_grid(n, sym=O.MAJORMINOR, bc_type=bt, bc_val=bv)
    ddw = random_ddw(n, O.MAJORMINOR, 5)
    x = random_field(n, 9)
    b = O.fapply(g, ddw, x)
    d = O.diagonal(g, ddw)
    x2 = O.fsmooth(g, ddw, d, x, b)
    assert rel_err(x2, x) < 1e-12


def test_periodic_duplicates_consistent():
    n = [6, 4, 8]
    per = (1, 0, 1)
    bt, bv = random_bc(2)
    g = O.make_grid(n, sym=O.ISO, periodic=per, bc_type=bt, bc_val=bv)
    ddw = random_ddw(n, O.ISO, 4, per)
    u = random_field(n, 8, per)
    f = O.fapply(g, ddw, u).reshape(3, n[2] + 1, n[1] + 1, n[0] + 1)
    assert np.array_equal(f[:, :, :, 0], f[:, :, :, -1])
    assert np.array_equal(f[:, 0], f[:, -1])
