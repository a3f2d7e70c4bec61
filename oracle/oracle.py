"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  The oracle is a
plain-C FP64 restatement of Alamo's Operator::Elastic / Operator<Node> /
MLMG path; see agb_oracle.h for what each routine follows.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

ISO, MAJORMINOR = 0, 1
DISP, TRAC, PERIODIC, NEUMANN, NONE = 0, 1, 2, 3, 4
NFACES = 26
(XLO, YLO, ZLO, XHI, YHI, ZHI,
 YLO_ZLO, YLO_ZHI, YHI_ZLO, YHI_ZHI,
 ZLO_XLO, ZLO_XHI, ZHI_XLO, ZHI_XHI,
 XLO_YLO, XLO_YHI, XHI_YLO, XHI_YHI,
 XLO_YLO_ZLO, XLO_YLO_ZHI, XLO_YHI_ZLO, XLO_YHI_ZHI,
 XHI_YLO_ZLO, XHI_YLO_ZHI, XHI_YHI_ZLO, XHI_YHI_ZHI) = range(26)


class Grid(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int * 3),
        ("dx", ctypes.c_double * 3),
        ("periodic", ctypes.c_int * 3),
        ("sym", ctypes.c_int),
        ("uniform", ctypes.c_int),
        ("bc_type", (ctypes.c_int * 3) * NFACES),
        ("bc_val", (ctypes.c_double * 3) * NFACES),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("max_iter", ctypes.c_int),
        ("fixed_iter", ctypes.c_int),
        ("pre_smooth", ctypes.c_int),
        ("post_smooth", ctypes.c_int),
        ("final_smooth", ctypes.c_int),
        ("bottom_smooth", ctypes.c_int),
        ("max_fmg_iter", ctypes.c_int),
        ("bottom_max_iter", ctypes.c_int),
        ("bottom_tol_rel", ctypes.c_double),
        ("bottom_tol_abs", ctypes.c_double),
        ("omega", ctypes.c_double),
        ("max_coarsening_level", ctypes.c_int),
        ("verbose", ctypes.c_int),
    ]


class Report(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("status", ctypes.c_int),
        ("res0", ctypes.c_double),
        ("res_final", ctypes.c_double),
        ("nlevels", ctypes.c_int),
        ("t_setup", ctypes.c_double),
        ("t_iter", ctypes.c_double),
    ]


_lib = None


def build():
    """Compile liboracle.so from agb_oracle.c (make, gcc)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "agb_oracle.c")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        d = P(ctypes.c_double)
        g = P(Grid)
        L.orc_fapply.argtypes = [g, d, d, d]
        L.orc_diagonal.argtypes = [g, d, d]
        L.orc_fsmooth.argtypes = [g, d, d, d, d, ctypes.c_double]
        L.orc_residual.argtypes = [g, d, d, d, d]
        L.orc_restriction.argtypes = [g, d, d]
        L.orc_interpolation.argtypes = [g, d, d]
        L.orc_average_ddw.argtypes = [g, d, d]
        L.orc_norm_inf.argtypes = [g, d]
        L.orc_norm_inf.restype = ctypes.c_double
        L.orc_bc_init.argtypes = [g, d, ctypes.c_int]
        L.orc_newton_rhs.argtypes = [g, d, d, d, d, d]
        L.orc_stress.argtypes = [g, d, d, d, d]
        L.orc_traction_xhi.argtypes = [g, d, d, d, d]
        L.orc_solve.argtypes = [g, d, P(Params), d, d, ctypes.c_double, ctypes.c_double, P(Report)]
        L.orc_newton_solve.argtypes = [g, d, d, P(Params), d, d, ctypes.c_double, ctypes.c_double,
                                       P(Report)]
        L.orc_solve_begin.argtypes = [g, d, P(Params), d, d, ctypes.c_double, ctypes.c_double]
        L.orc_solve_begin.restype = ctypes.c_void_p
        L.orc_solve_iterate.argtypes = [ctypes.c_void_p, d, ctypes.c_int]
        L.orc_solve_end.argtypes = [ctypes.c_void_p, d, P(Report)]
        L.orc_strain_energy.argtypes = [g, d, d, d, d]
        L.orc_bottom_solve.argtypes = [g, d, d, d, d, P(Params)]
        L.orc_cubic.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, d, d]
        L.orc_quat_to_rot.argtypes = [d, d]
        L.orc_default_params.argtypes = [P(Params)]
        L.orc_num_levels.argtypes = [g, ctypes.c_int]
        L.orc_num_levels.restype = ctypes.c_int
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_grid(n, dx=None, sym=ISO, periodic=(0, 0, 0), bc_type=None, bc_val=None, uniform=False):
    """Grid with n cells per direction; default BC is zero displacement everywhere."""
    g = Grid()
    n = list(n)
    for d in range(3):
        g.n[d] = n[d]
        g.dx[d] = (1.0 / n[d]) if dx is None else dx[d]
        g.periodic[d] = int(periodic[d])
    g.sym = sym
    g.uniform = int(uniform)
    bt = np.zeros((NFACES, 3), np.int32) if bc_type is None else np.asarray(bc_type)
    bv = np.zeros((NFACES, 3)) if bc_val is None else np.asarray(bc_val)
    for f in range(NFACES):
        for c in range(3):
            g.bc_type[f][c] = int(bt[f, c])
            g.bc_val[f][c] = float(bv[f, c])
    return g


def nodes(g):
    return (g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1)


def ncoef(g):
    return 2 if g.sym == ISO else 21


def coarsen(g):
    c = Grid.from_buffer_copy(g)
    for d in range(3):
        c.n[d] = g.n[d] // 2
        c.dx[d] = g.dx[d] * 2.0
    return c


def default_params(**kw):
    p = Params()
    lib().orc_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def fapply(g, ddw, u):
    f = np.zeros(3 * nodes(g))
    lib().orc_fapply(ctypes.byref(g), _p(ddw), _p(u), _p(f))
    return f


def diagonal(g, ddw):
    d = np.zeros(3 * nodes(g))
    lib().orc_diagonal(ctypes.byref(g), _p(ddw), _p(d))
    return d


def fsmooth(g, ddw, diag, x, b, omega=2.0 / 3.0):
    x = np.array(x, dtype=np.float64, copy=True)
    lib().orc_fsmooth(ctypes.byref(g), _p(ddw), _p(diag), _p(x), _p(b), omega)
    return x


def residual(g, ddw, x, b):
    r = np.zeros(3 * nodes(g))
    lib().orc_residual(ctypes.byref(g), _p(ddw), _p(x), _p(b), _p(r))
    return r


def restriction(gf, fine):
    gc = coarsen(gf)
    c = np.zeros(3 * nodes(gc))
    lib().orc_restriction(ctypes.byref(gf), _p(fine), _p(c))
    return c


def interpolation(gf, fine, crse):
    fine = np.array(fine, dtype=np.float64, copy=True)
    lib().orc_interpolation(ctypes.byref(gf), _p(fine), _p(crse))
    return fine


def average_ddw(gf, ddw):
    gc = coarsen(gf)
    c = np.zeros(ncoef(gf) * nodes(gc))
    lib().orc_average_ddw(ctypes.byref(gf), _p(ddw), _p(c))
    return c


def bc_init(g, rhs, homogeneous=False):
    rhs = np.array(rhs, dtype=np.float64, copy=True)
    lib().orc_bc_init(ctypes.byref(g), _p(rhs), int(homogeneous))
    return rhs


def newton_rhs(g, ddw, F0, u, b):
    rhs = np.zeros(3 * nodes(g))
    lib().orc_newton_rhs(ctypes.byref(g), _p(ddw), _p(F0), _p(u), _p(b), _p(rhs))
    return rhs


def strain_energy(g, ddw, u):
    """(eps 9 per node AoS, energy 1 per node)"""
    e = np.zeros(9 * nodes(g))
    w = np.zeros(nodes(g))
    lib().orc_strain_energy(ctypes.byref(g), _p(ddw), _p(u), _p(e), _p(w))
    return e, w


def traction_xhi(g, ddw, F0, u):
    t = np.zeros(3)
    lib().orc_traction_xhi(ctypes.byref(g), _p(ddw), _p(F0), _p(u), _p(t))
    return t


def stress(g, ddw, F0, u):
    s = np.zeros(9 * nodes(g))
    lib().orc_stress(ctypes.byref(g), _p(ddw), _p(F0), _p(u), _p(s))
    return s


def solve(g, ddw, b, x0=None, tol_rel=1e-8, tol_abs=0.0, params=None):
    x = np.zeros(3 * nodes(g)) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    if x.shape != (3 * nodes(g),) or b.shape != (3 * nodes(g),) or ddw.size != ncoef(g) * nodes(g):
        raise ValueError("field sizes do not match the grid")
    p = params or default_params()
    rep = Report()
    lib().orc_solve(ctypes.byref(g), _p(ddw), ctypes.byref(p), _p(x), _p(b), tol_rel, tol_abs,
                    ctypes.byref(rep))
    return x, rep


class Session:
    """orc_solve in pieces: prepareForSolve and the first residual at
    construction, then iterate(k) runs up to k more MLMG iterations (returns
    the status so far: 0 converged, 1 running or out of iterations, 2 NaN),
    finish() returns (x, report).  Holds references to every array the C
    side keeps a pointer to."""

    def __init__(self, g, ddw, b, x0=None, tol_rel=1e-8, tol_abs=0.0, params=None):
        if b.shape != (3 * nodes(g),) or ddw.size != ncoef(g) * nodes(g):
            raise ValueError("field sizes do not match the grid")
        self.g, self.ddw, self.b = g, ddw, b
        self.x = np.zeros(3 * nodes(g)) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
        self.p = params or default_params()
        self.h = lib().orc_solve_begin(ctypes.byref(g), _p(ddw), ctypes.byref(self.p), _p(self.x), _p(b),
                                       tol_rel, tol_abs)

    def iterate(self, k):
        return lib().orc_solve_iterate(self.h, _p(self.x), int(k))

    def finish(self):
        rep = Report()
        lib().orc_solve_end(self.h, _p(self.x), ctypes.byref(rep))
        self.h = None
        return self.x, rep


def bottom_solve(g, ddw, diag, res, params=None):
    """The coarsest-level step of a solve on one level: (cor, BiCGStab code)."""
    cor = np.zeros(3 * nodes(g))
    p = params or default_params()
    ret = lib().orc_bottom_solve(ctypes.byref(g), _p(ddw), _p(diag), _p(res), _p(cor), ctypes.byref(p))
    return cor, ret


def newton_solve(g, ddw, F0, u, b, tol_rel=1e-8, tol_abs=0.0, params=None):
    u = np.array(u, dtype=np.float64, copy=True)
    p = params or default_params()
    rep = Report()
    lib().orc_newton_solve(ctypes.byref(g), _p(ddw), _p(F0), ctypes.byref(p), _p(u), _p(b),
                           tol_rel, tol_abs, ctypes.byref(rep))
    return u, rep


def cubic(C11, C12, C44, R=None):
    R = np.eye(3) if R is None else np.asarray(R, dtype=np.float64)
    R = np.ascontiguousarray(R.reshape(9))
    out = np.zeros(21)
    lib().orc_cubic(C11, C12, C44, _p(R), _p(out))
    return out


def quat_to_rot(q):
    q = np.ascontiguousarray(np.asarray(q, dtype=np.float64))
    R = np.zeros(9)
    lib().orc_quat_to_rot(_p(q), _p(R))
    return R.reshape(3, 3)
