"""ctypes binding of libalamo_gb300.so (the C ABI of include/agb.h).

The shared library is built in-tree by alamo_gb300.build (nvcc, sm_103a).  If
it is missing this module raises at import time: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libalamo_gb300.so")

AGB_OK, AGB_MAXITER, AGB_STALL, AGB_NAN, AGB_BADARG, AGB_CUDA, AGB_NOMEM, AGB_STATE = range(8)
STATUS_NAMES = {0: "AGB_OK", 1: "AGB_MAXITER", 2: "AGB_STALL", 3: "AGB_NAN", 4: "AGB_BADARG", 5: "AGB_CUDA",
                6: "AGB_NOMEM", 7: "AGB_STATE"}
AGB_ISO, AGB_MAJORMINOR = 0, 1
AGB_MEM_HOST, AGB_MEM_DEVICE = 0, 1
AGB_LAYOUT_AOS, AGB_LAYOUT_SOA = 0, 1
AGB_PREC_F64, AGB_PREC_MIXED = 0, 1
NFACES = 26


class AgbBC(ctypes.Structure):
    _fields_ = [("type", (ctypes.c_int * 3) * NFACES), ("val", (ctypes.c_double * 3) * NFACES)]


class AgbSolverParams(ctypes.Structure):
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
        ("precision", ctypes.c_int),
        ("inner_tol_rel", ctypes.c_double),
        ("inner_max_iter", ctypes.c_int),
        ("max_refine", ctypes.c_int),
        ("use_graph", ctypes.c_int),
        ("krylov", ctypes.c_int),
    ]


class AgbSolveReport(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("status", ctypes.c_int),
        ("res0", ctypes.c_double),
        ("res_final", ctypes.c_double),
        ("rhs_norm", ctypes.c_double),
        ("nlevels", ctypes.c_int),
        ("refinements", ctypes.c_int),
        ("solve_ms", ctypes.c_double),
        ("kernels", ctypes.c_longlong),
    ]


class AgbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


_lib = None


def lib():
    """Load libalamo_gb300.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libalamo_gb300.so not built: run `python -m alamo_gb300.build` "
                          "(the CUDA library is required; there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, dp, fp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
    st = ctypes.c_int
    sig = {
        "agb_default_params": (None, [ctypes.POINTER(AgbSolverParams)]),
        "agb_last_error": (ctypes.c_char_p, []),
        "agb_version": (ctypes.c_char_p, []),
        "agb_op_create": (st, [ip, dp, ip, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]),
        "agb_op_destroy": (st, [vp]),
        "agb_op_set_bc": (st, [vp, ctypes.POINTER(AgbBC)]),
        "agb_op_set_model": (st, [vp, vp, ctypes.c_int, ctypes.c_int]),
        "agb_op_set_uniform": (st, [vp, ctypes.c_int]),
        "agb_op_set_omega": (st, [vp, ctypes.c_double]),
        "agb_op_num_levels": (st, [vp, ip]),
        "agb_op_level_cells": (st, [vp, ctypes.c_int, ip]),
        "agb_op_prepare": (st, [vp]),
        "agb_op_get_model": (st, [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int]),
        "agb_op_fapply": (st, [vp, ctypes.c_int, vp, vp, ctypes.c_int]),
        "agb_op_fapply_f32": (st, [vp, ctypes.c_int, vp, vp, ctypes.c_int]),
        "agb_op_diagonal": (st, [vp, ctypes.c_int, vp, ctypes.c_int]),
        "agb_op_fsmooth": (st, [vp, ctypes.c_int, vp, vp, ctypes.c_int]),
        "agb_op_fsmooth_f32": (st, [vp, ctypes.c_int, vp, vp, ctypes.c_int]),
        "agb_op_residual": (st, [vp, ctypes.c_int, vp, vp, vp, ctypes.c_int]),
        "agb_op_restriction": (st, [vp, ctypes.c_int, vp, vp, ctypes.c_int]),
        "agb_op_interpolation": (st, [vp, ctypes.c_int, vp, vp, ctypes.c_int]),
        "agb_solver_create": (st, [vp, ctypes.POINTER(AgbSolverParams), ctypes.POINTER(vp)]),
        "agb_solver_destroy": (st, [vp]),
        "agb_solve": (st, [vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                           ctypes.POINTER(AgbSolveReport)]),
        "agb_apply": (st, [vp, vp, vp, ctypes.c_int]),
        "agb_bc_init": (st, [vp, vp, ctypes.c_int, ctypes.c_int]),
        "agb_newton_rhs": (st, [vp, vp, vp, vp, vp, ctypes.c_int]),
        "agb_newton_solve": (st, [vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.POINTER(AgbSolveReport)]),
        "agb_stress": (st, [vp, vp, vp, vp, ctypes.c_int]),
        "agb_traction_xhi": (st, [vp, vp, vp, dp, ctypes.c_int]),
        "agb_strain_energy": (st, [vp, vp, vp, vp, ctypes.c_int]),
        "agb_conv3_tc_pack": (st, [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, vp]),
        "agb_conv3_tc": (st, [ip, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, vp, vp,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]),
        "agb_conv3_tc_error": (st, [ctypes.POINTER(ctypes.c_int)]),
        "agb_op_time_sweep": (st, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]),
        "agb_fp64_fma_peak": (st, [ctypes.c_int, dp, ctypes.POINTER(ctypes.c_float)]),
        "agb_host_alloc": (st, [ctypes.c_size_t, ctypes.POINTER(vp)]),
        "agb_host_free": (st, [vp]),
        "agb_conv3_flip": (st, [ctypes.c_int, ctypes.c_int, vp, vp, vp]),
        "agb_adam_step": (st, [ctypes.c_longlong, vp, vp, vp, vp, vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                               ctypes.c_float, ctypes.c_int, vp]),
        "agb_conv3_wgrad0": (st, [ip, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                  ctypes.c_int, vp, vp, vp]),
        "agb_grid_prolong": (st, [ip, ip, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_float, ctypes.c_float, vp]),
        "agb_grid_prolong_t": (st, [ip, ip, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_float, ctypes.c_float, vp]),
        "agb_axpby_mask": (st, [ctypes.c_longlong, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, vp, ctypes.c_int,
                                ctypes.c_int, vp]),
        "agb_unet_layers": (st, [ip, ip, ip]),
        "agb_unet_acts": (st, [ip, ip]),
        "agb_unet_create": (st, [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.POINTER(vp)]),
        "agb_unet_set_weights": (st, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]),
        "agb_unet_forward": (st, [vp, ip, ctypes.POINTER(vp), vp, vp]),
        "agb_unet_features": (st, [vp, vp, ctypes.c_int, vp, dp]),
        "agb_learned_destroy": (st, [vp]),
        "agb_solver_set_learned": (st, [vp, vp, ctypes.c_double, ctypes.c_int]),
        "agb_solver_learned_stats": (st, [vp, ip, ip, ip]),
        "agb_write_node_plotfile": (st, [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ip, dp, dp, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_char_p), ip, ctypes.POINTER(vp), ctypes.c_int]),
        "agb_gen_voronoi_cubic": (st, [ip, ctypes.c_int, dp, dp, vp, vp, ctypes.c_int, vp]),
        "agb_gen_ellipsoids": (st, [ip, ctypes.c_int, dp, ctypes.c_double, vp, ctypes.c_int, vp]),
        "agb_gen_sphere": (st, [ip, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, vp, vp, ctypes.c_int, vp]),
        "agb_batch_create": (st, [ctypes.c_int, ip, dp, ip, ctypes.c_int, ctypes.POINTER(AgbSolverParams),
                                  ctypes.POINTER(vp)]),
        "agb_batch_destroy": (st, [vp]),
        "agb_batch_set_bc": (st, [vp, ctypes.POINTER(AgbBC)]),
        "agb_batch_set_model": (st, [vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int]),
        "agb_batch_set_eigenstrain": (st, [vp, dp]),
        "agb_batch_solve": (st, [vp, ctypes.c_double, ctypes.c_double, ctypes.POINTER(AgbSolveReport),
                                 ctypes.POINTER(AgbSolveReport)]),
        "agb_batch_get_solution": (st, [vp, ctypes.c_int, vp, ctypes.c_int]),
        "agb_batch_mean_stress": (st, [vp, dp]),
        "agb_batch_tuning": (st, [vp, ctypes.c_int, ip]),
        "agb_bottom_solve_noalloc": (st, [ip, dp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(AgbBC), vp, vp, vp, vp,
                                          vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status):
    if status != AGB_OK:
        msg = lib().agb_last_error()
        raise AgbError(status, msg.decode() if msg else "")
    return status


def exported_symbols():
    """Names the C ABI declares (parsed from include/agb.h)."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "agb.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(agb_[a-z0-9_]+)\s*\(", text)))
