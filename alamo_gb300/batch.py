"""Batched RVE homogenization through the C ABI (agb_batch_*): many
independent periodic boxes of different sizes solved together on the GPU."""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .elastic import _ptr, default_params


class Batch:
    def __init__(self, sizes, dx=None, sym="isotropic", periodic=(1, 1, 1), **params):
        """sizes: list of (nx, ny, nz) cells per problem; dx: list of cell sizes
        (default 1/n: unit cubes); params: agb_solver_params fields, e.g.
        precision=1 (FP32 cycles in FP64 refinement) and krylov=8 (each
        problem's GCR over the batched FP32 cycle)."""
        self.sizes = [tuple(int(v) for v in s) for s in sizes]
        self.np = len(self.sizes)
        if dx is None:
            dx = [(1.0 / s[0], 1.0 / s[1], 1.0 / s[2]) for s in self.sizes]
        self.dx = [tuple(float(v) for v in d) for d in dx]
        self.sym = _lib.AGB_ISO if sym in ("isotropic", "iso", 0) else _lib.AGB_MAJORMINOR
        self.ncoef = 2 if self.sym == _lib.AGB_ISO else 21
        self.params = default_params(**params)
        n = (ctypes.c_int * (3 * self.np))(*[v for s in self.sizes for v in s])
        d = (ctypes.c_double * (3 * self.np))(*[v for s in self.dx for v in s])
        h = ctypes.c_void_p()
        check(lib().agb_batch_create(self.np, n, d, (ctypes.c_int * 3)(*periodic), self.sym,
                                     ctypes.byref(self.params), ctypes.byref(h)))
        self.h = h
        self.reports = None
        self.total = None

    def close(self):
        if getattr(self, "h", None):
            lib().agb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nodes(self, q):
        s = self.sizes[q]
        return (s[0] + 1) * (s[1] + 1) * (s[2] + 1)

    def SetBC(self, bc):
        check(lib().agb_batch_set_bc(self.h, ctypes.byref(bc.to_c())))

    def SetModel(self, q, ddw, layout="aos"):
        p, mem = _ptr(ddw)
        check(lib().agb_batch_set_model(self.h, q, p, _lib.AGB_LAYOUT_AOS if layout == "aos" else _lib.AGB_LAYOUT_SOA,
                                        mem))

    def SetEigenstrain(self, F0):
        F0 = np.ascontiguousarray(np.asarray(F0, dtype=np.float64).reshape(self.np * 9))
        check(lib().agb_batch_set_eigenstrain(self.h, F0.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def solve(self, tol_rel=1e-8, tol_abs=0.0, raise_on_fail=True):
        reps = (_lib.AgbSolveReport * self.np)()
        tot = _lib.AgbSolveReport()
        st = lib().agb_batch_solve(self.h, float(tol_rel), float(tol_abs), reps, ctypes.byref(tot))
        self.reports, self.total = reps, tot
        if st != _lib.AGB_OK and raise_on_fail:
            check(st)
        return tot

    def solution(self, q):
        u = np.zeros(3 * self.nodes(q))
        p, mem = _ptr(u)
        check(lib().agb_batch_get_solution(self.h, q, p, mem))
        return u

    def mean_stress(self):
        s = np.zeros(9 * self.np)
        check(lib().agb_batch_mean_stress(self.h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return s.reshape(self.np, 3, 3)

    def tuning(self, level):
        d = (ctypes.c_int * 3)()
        check(lib().agb_batch_tuning(self.h, level, d))
        return tuple(d)
