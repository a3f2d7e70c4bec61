"""Python mirror of the reference interface for the nodal elastic solve.

Names and argument meaning follow Alamo's C++ classes so that callers (and
the parity tests) read like the reference:

    BC.Constant / BC.TensionTest   BC/Operator/Elastic/Constant.H, TensionTest.H
    Elastic                        Operator/Elastic.H (Operator::Elastic<SYM>)
    Linear                         Solver/Nonlocal/Linear.H
    Newton                         Solver/Nonlocal/Newton.H (one Newton step = linear solve)

Every call goes through the C ABI of libalamo_gb300.so (include/agb.h); the
arithmetic runs on the GPU only.  Fields are numpy float64 arrays holding the
reference's nodal-MultiFab image (3 components, (n+1)^3 nodes each, i
fastest) or CUDA tensors (anything with data_ptr() on a CUDA device).
Failures raise AgbError carrying the agb_status, the way the reference aborts
through Util::Abort / MLMG exceptions.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib

FACE_NAMES = ["xlo", "ylo", "zlo", "xhi", "yhi", "zhi",
              "ylozlo", "ylozhi", "yhizlo", "yhizhi",
              "zloxlo", "zloxhi", "zhixlo", "zhixhi",
              "xloylo", "xloyhi", "xhiylo", "xhiyhi",
              "xloylozlo", "xloylozhi", "xloyhizlo", "xloyhizhi",
              "xhiylozlo", "xhiylozhi", "xhiyhizlo", "xhiyhizhi"]
FACE = {n: i for i, n in enumerate(FACE_NAMES)}
TYPE = {"displacement": 0, "disp": 0, "traction": 1, "trac": 1, "periodic": 2, "neumann": 3, "none": 4}
DISP, TRAC, PERIODIC, NEUMANN, NONE = 0, 1, 2, 3, 4


def _ptr(a, dtype=np.float64):
    """(pointer, mem) for a numpy array or a CUDA tensor; None -> (None, host)."""
    if a is None:
        return None, _lib.AGB_MEM_HOST
    if isinstance(a, np.ndarray):
        if a.dtype != dtype or not a.flags.c_contiguous:
            raise TypeError("expected a C-contiguous %s array" % np.dtype(dtype).name)
        return a.ctypes.data_as(ctypes.c_void_p), _lib.AGB_MEM_HOST
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise TypeError("expected a contiguous tensor")
        mem = _lib.AGB_MEM_DEVICE if getattr(a, "is_cuda", False) else _lib.AGB_MEM_HOST
        return ctypes.c_void_p(a.data_ptr()), mem
    raise TypeError("unsupported array type %r" % type(a))


# ---------------------------------------------------------------------------
# BC::Operator::Elastic
# ---------------------------------------------------------------------------
class Constant:
    """BC::Operator::Elastic::Constant (Constant.H:31-194): every region
    displacement 0 unless set."""

    def __init__(self):
        self.type = np.zeros((26, 3), np.int32)
        self.val = np.zeros((26, 3))

    def Set(self, face, direction, type_, value=0.0):
        f = FACE[face] if isinstance(face, str) else int(face)
        t = TYPE[type_] if isinstance(type_, str) else int(type_)
        self.type[f, direction] = t
        self.val[f, direction] = value
        return self

    def set_face(self, face, types, vals=None):
        """Reference input style: bc.constant.type.<face> = a b c / val.<face> = x y z."""
        f = FACE[face] if isinstance(face, str) else int(face)
        for d in range(3):
            t = types[d]
            self.type[f, d] = TYPE[t] if isinstance(t, str) else int(t)
            if vals is not None:
                self.val[f, d] = vals[d]
        return self

    def to_c(self):
        c = _lib.AgbBC()
        for f in range(26):
            for d in range(3):
                c.type[f][d] = int(self.type[f, d])
                c.val[f][d] = float(self.val[f, d])
        return c


class TensionTest(Constant):
    """BC::Operator::Elastic::TensionTest::Parse (TensionTest.H:48-306) for a
    load value at the current time (disp or trac, one of the two)."""

    def __init__(self, type="uniaxial_stress_clamp", disp=None, trac=None):
        super().__init__()
        if (disp is None) == (trac is None):
            raise ValueError("specify exactly one of disp or trac")
        mode_disp = disp is not None
        load = disp if mode_disp else trac
        T, D = TRAC, DISP
        ty, va = self.type, self.val
        xhi_all = ["xhi", "xhiylo", "xhiyhi", "zloxhi", "zhixhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo", "xhiyhizhi"]
        xlo_all = ["xlo", "xloylo", "xloyhi", "zloxlo", "zhixlo", "xloylozlo", "xloylozhi", "xloyhizlo", "xloyhizhi"]
        if type == "uniaxial_stress_clamp":
            for f in xhi_all:
                va[FACE[f], 0] = load
            for f in ["ylo", "yhi", "zlo", "zhi", "ylozlo", "yhizlo", "ylozhi", "yhizhi"]:
                ty[FACE[f], :] = T
        elif type == "uniaxial_kolsky":
            for f in ["xlo", "xloylo", "xloyhi"]:
                va[FACE[f], 0] = load
            for f in ["ylo", "yhi"]:
                ty[FACE[f], :] = T
        elif type in ("uniaxial_stress", "uniaxial_strain"):
            ty[:, :] = T
            for f in xlo_all:
                ty[FACE[f], 0] = D
            if type == "uniaxial_stress":
                for f in ["xhi", "xhiylo", "xhiyhi", "zloxhi", "zhixhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo",
                          "xhiyhizhi"]:
                    ty[FACE[f], 0] = D if mode_disp else T
                    va[FACE[f], 0] = load
                for f in ["ylo", "xloylo", "xhiylo", "ylozlo", "ylozhi", "xloylozlo", "xloylozhi", "xhiylozlo",
                          "xhiylozhi"]:
                    ty[FACE[f], 1] = D
                for f in ["zlo", "ylozlo", "yhizlo", "zloxlo", "zloxhi", "xloylozlo", "xloyhizlo", "xhiylozlo",
                          "xhiyhizlo"]:
                    ty[FACE[f], 2] = D
            else:
                for f in xhi_all:
                    ty[FACE[f], 0] = D
                    va[FACE[f], 0] = load
                for f in ["ylo", "xloylo", "xhiylo", "yhi", "xloyhi", "xhiyhi", "ylozlo", "ylozhi", "yhizlo",
                          "yhizhi", "xloylozlo", "xloylozhi", "xhiylozlo", "xhiylozhi", "xloyhizlo", "xloyhizhi",
                          "xhiyhizlo", "xhiyhizhi"]:
                    ty[FACE[f], 1] = D
                for f in ["zlo", "zhi", "ylozlo", "yhizlo", "zloxlo", "zloxhi", "ylozhi", "yhizhi", "zhixlo",
                          "zhixhi", "xloylozlo", "xloyhizlo", "xhiylozlo", "xhiyhizlo", "xloylozhi", "xloyhizhi",
                          "xhiylozhi", "xhiyhizhi"]:
                    ty[FACE[f], 2] = D
        else:
            raise ValueError("Unknown BC type " + str(type))


# ---------------------------------------------------------------------------
# Operator::Elastic
# ---------------------------------------------------------------------------
class Elastic:
    """Operator::Elastic<SYM> on one box, single AMR level (amrlev = 0).

    sym: "isotropic" (Matrix4<3,Isotropic>: lambda, mu per node) or
    "majorminor" (Matrix4<3,MajorMinor>: 21 coefficients per node).
    """

    def __init__(self, n_cells, dx=None, sym="isotropic", periodic=(0, 0, 0), max_coarsening_level=30):
        self.n = [int(v) for v in n_cells]
        self.dx = [1.0 / v for v in self.n] if dx is None else [float(v) for v in dx]
        self.sym = _lib.AGB_ISO if sym in ("isotropic", "iso", 0) else _lib.AGB_MAJORMINOR
        self.ncoef = 2 if self.sym == _lib.AGB_ISO else 21
        self.periodic = [int(bool(p)) for p in periodic]
        h = ctypes.c_void_p()
        check(lib().agb_op_create((ctypes.c_int * 3)(*self.n), (ctypes.c_double * 3)(*self.dx),
                                  (ctypes.c_int * 3)(*self.periodic), self.sym, int(max_coarsening_level),
                                  ctypes.byref(h)))
        self.h = h
        self.bc = None

    def close(self):
        if getattr(self, "h", None):
            lib().agb_op_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # geometry
    def NumLevels(self):
        v = ctypes.c_int()
        check(lib().agb_op_num_levels(self.h, ctypes.byref(v)))
        return v.value

    def LevelCells(self, mglev):
        v = (ctypes.c_int * 3)()
        check(lib().agb_op_level_cells(self.h, mglev, v))
        return list(v)

    def nodes(self, mglev=0):
        n = self.LevelCells(mglev)
        return (n[0] + 1) * (n[1] + 1) * (n[2] + 1)

    # setup, Elastic.H:49-105
    def SetBC(self, bc):
        self.bc = bc
        check(lib().agb_op_set_bc(self.h, ctypes.byref(bc.to_c())))

    def SetModel(self, ddw, layout="aos"):
        p, mem = _ptr(ddw)
        check(lib().agb_op_set_model(self.h, p, _lib.AGB_LAYOUT_AOS if layout == "aos" else _lib.AGB_LAYOUT_SOA,
                                     mem))

    def SetUniform(self, uniform):
        check(lib().agb_op_set_uniform(self.h, int(bool(uniform))))

    def SetOmega(self, omega):
        check(lib().agb_op_set_omega(self.h, float(omega)))

    def prepareForSolve(self):
        check(lib().agb_op_prepare(self.h))

    def GetModel(self, mglev=0):
        out = np.zeros(self.ncoef * self.nodes(mglev))
        p, mem = _ptr(out)
        check(lib().agb_op_get_model(self.h, mglev, p, _lib.AGB_LAYOUT_AOS, mem))
        return out

    # MLNodeLinOp virtuals
    def _vec(self, mglev, out, dtype=np.float64):
        return np.zeros(3 * self.nodes(mglev), dtype) if out is None else out

    def Fapply(self, mglev, u, out=None):
        if isinstance(u, np.ndarray) and u.dtype == np.float32:
            out = self._vec(mglev, out, np.float32)
            pf, mem = _ptr(out, np.float32)
            pu, _ = _ptr(u, np.float32)
            check(lib().agb_op_fapply_f32(self.h, mglev, pf, pu, mem))
            return out
        out = self._vec(mglev, out)
        pf, mem = _ptr(out)
        pu, _ = _ptr(u)
        check(lib().agb_op_fapply(self.h, mglev, pf, pu, mem))
        return out

    def Diagonal(self, mglev, out=None):
        out = self._vec(mglev, out)
        p, mem = _ptr(out)
        check(lib().agb_op_diagonal(self.h, mglev, p, mem))
        return out

    def Fsmooth(self, mglev, x, b):
        """Two damped-Jacobi sweeps in place (Operator.cpp:88-154)."""
        if isinstance(x, np.ndarray) and x.dtype == np.float32:
            px, mem = _ptr(x, np.float32)
            pb, _ = _ptr(b, np.float32)
            check(lib().agb_op_fsmooth_f32(self.h, mglev, px, pb, mem))
            return x
        px, mem = _ptr(x)
        pb, _ = _ptr(b)
        check(lib().agb_op_fsmooth(self.h, mglev, px, pb, mem))
        return x

    def solutionResidual(self, mglev, x, b, out=None):
        out = self._vec(mglev, out)
        pr, mem = _ptr(out)
        px, _ = _ptr(x)
        pb, _ = _ptr(b)
        check(lib().agb_op_residual(self.h, mglev, pr, px, pb, mem))
        return out

    def restriction(self, cmglev, fine, out=None):
        out = self._vec(cmglev, out)
        pc, mem = _ptr(out)
        pf, _ = _ptr(fine)
        check(lib().agb_op_restriction(self.h, cmglev, pc, pf, mem))
        return out

    def interpolation(self, fmglev, fine, crse):
        """fine += P crse, in place (Operator.cpp:365-434)."""
        pf, mem = _ptr(fine)
        pc, _ = _ptr(crse)
        check(lib().agb_op_interpolation(self.h, fmglev, pf, pc, mem))
        return fine

    # around the solve
    def BCInit(self, rhs, homogeneous=False):
        p, mem = _ptr(rhs)
        check(lib().agb_bc_init(self.h, p, int(bool(homogeneous)), mem))
        return rhs

    def NewtonRHS(self, u, b, F0=None, out=None):
        out = self._vec(0, out)
        po, mem = _ptr(out)
        check(lib().agb_newton_rhs(self.h, _ptr(F0)[0], _ptr(u)[0], _ptr(b)[0], po, mem))
        return out

    def Stress(self, u, F0=None):
        out = np.zeros(9 * self.nodes(0))
        po, mem = _ptr(out)
        check(lib().agb_stress(self.h, _ptr(F0)[0], _ptr(u)[0], po, mem))
        return out

    def StrainEnergy(self, u, strain=True, energy=True):
        """Elastic::Strain (9 per node, row-major, AoS) and Elastic::Energy (1
        per node) of u; returns (eps or None, energy or None)."""
        eps = np.zeros(9 * self.nodes(0)) if strain else None
        w = np.zeros(self.nodes(0)) if energy else None
        pu, mem = _ptr(u)
        check(lib().agb_strain_energy(self.h, pu, _ptr(eps)[0], _ptr(w)[0], mem))
        return eps, w

    def TractionXhi(self, u, F0=None):
        t = (ctypes.c_double * 3)()
        pu, mem = _ptr(u)
        check(lib().agb_traction_xhi(self.h, _ptr(F0)[0], pu, t, mem))
        return np.array(list(t))

    def time_sweep(self, mglev=0, precision="f32", mode=2, reps=10):
        ms = ctypes.c_double()
        prec = _lib.AGB_PREC_MIXED if precision == "f32" else _lib.AGB_PREC_F64
        check(lib().agb_op_time_sweep(self.h, mglev, prec, mode, reps, ctypes.byref(ms)))
        return ms.value


def fp64_fma_peak(iters=600):
    """Measured FP64 FMA throughput of the current device (TFLOP/s, launch ms)."""
    tf, ms = ctypes.c_double(), ctypes.c_float()
    check(lib().agb_fp64_fma_peak(int(iters), ctypes.byref(tf), ctypes.byref(ms)))
    return tf.value, ms.value


# ---------------------------------------------------------------------------
# Solver::Nonlocal::Linear / Newton
# ---------------------------------------------------------------------------
def default_params(**kw):
    p = _lib.AgbSolverParams()
    lib().agb_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError("unknown solver parameter %s" % k)
        setattr(p, k, v)
    return p


class Linear:
    """Solver::Nonlocal::Linear (Linear.H:18-392) over the GPU MLMG driver.
    params: agb_solver_params fields (Linear::Parse's keys, Linear.H:296-382),
    plus precision=1 (FP32 cycles in FP64 refinement) and krylov=k (flexible
    GCR over the FP32 cycle with k stored directions; no reference key)."""

    def __init__(self, op=None, **params):
        self.params = default_params(**params)
        self.h = None
        self.op = None
        self.report = None
        if op is not None:
            self.Define(op)

    def Define(self, op):
        if self.h is not None:
            raise RuntimeError("Solver cannot be re-defined")
        self.op = op
        h = ctypes.c_void_p()
        check(lib().agb_solver_create(op.h, ctypes.byref(self.params), ctypes.byref(h)))
        self.h = h

    def Clear(self):
        if self.h is not None:
            lib().agb_solver_destroy(self.h)
            self.h = None
            self.op = None

    def __del__(self):
        try:
            self.Clear()
        except Exception:
            pass

    # setters, Linear.H:178-184 (take effect at the next Define)
    def setMaxIter(self, v): self.params.max_iter = v
    def setBottomMaxIter(self, v): self.params.bottom_max_iter = v
    def setMaxFmgIter(self, v): self.params.max_fmg_iter = v
    def setFixedIter(self, v): self.params.fixed_iter = v
    def setVerbose(self, v): self.params.verbose = v
    def setPreSmooth(self, v): self.params.pre_smooth = v
    def setPostSmooth(self, v): self.params.post_smooth = v

    def solve(self, sol, rhs, tol_rel=1e-8, tol_abs=1e-8, raise_on_fail=True):
        """MLMG solve; updates sol in place and returns ||b - A x||_inf."""
        rep = _lib.AgbSolveReport()
        ps, mem = _ptr(sol)
        pr, _ = _ptr(rhs)
        st = lib().agb_solve(self.h, ps, pr, float(tol_rel), float(tol_abs), mem, ctypes.byref(rep))
        self.report = rep
        if st != _lib.AGB_OK and (raise_on_fail or st not in (_lib.AGB_MAXITER, _lib.AGB_STALL)):
            check(st)
        return rep.res_final

    def apply(self, out, inp):
        po, mem = _ptr(out)
        pi, _ = _ptr(inp)
        check(lib().agb_apply(self.h, po, pi, mem))
        return out


class Newton(Linear):
    """Solver::Nonlocal::Newton with one Newton iteration (linear models):
    rhs = b - div DW(u) / BC rows, solve for dsol, u += dsol."""

    def solve(self, u, b, F0=None, tol_rel=1e-8, tol_abs=1e-8, raise_on_fail=True):
        rep = _lib.AgbSolveReport()
        pu, mem = _ptr(u)
        st = lib().agb_newton_solve(self.h, _ptr(F0)[0], pu, _ptr(b)[0], float(tol_rel), float(tol_abs), mem,
                                    ctypes.byref(rep))
        self.report = rep
        if st != _lib.AGB_OK and (raise_on_fail or st not in (_lib.AGB_MAXITER, _lib.AGB_STALL)):
            check(st)
        return rep.res_final
