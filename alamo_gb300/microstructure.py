"""Seeded synthetic microstructures for the benchmark workloads.

No public dataset is involved; every field is generated from a SplitMix64
stream so that runs are reproducible on any host.

    sphere_inclusion   isotropic matrix with a smoothed spherical inclusion and
                       an eigenstrain inside it (65^3-node workload)
    voronoi_cubic      cubic-anisotropic polycrystal: Voronoi grains with
                       uniformly random orientations (257^3-node workload)
    rve_problem        periodic RVE with diffuse ellipsoidal inclusions
                       (batched-RVE workload)
    *_device           the same fields evaluated on the GPU from the same
                       random draws (agb_gen_* in the C ABI)
    cubic              Matrix4<3,MajorMinor>::Cubic(C11, C12, C44, R)
                       (Set/Matrix4_MajorMinor.H:518-547), including its slot
                       aliasing: the stored value of each of the 21 slots is the
                       rotated non-minor-symmetric tensor at the last (p,q,s,t)
                       of the reference's loop that maps to the slot.
"""
import ctypes
import itertools

import numpy as np

_MASK = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = int(seed) & _MASK

    def next_u64(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self, n=None):
        if n is None:
            return (self.next_u64() >> 11) * (1.0 / (1 << 53))
        return np.array([(self.next_u64() >> 11) * (1.0 / (1 << 53)) for _ in range(n)])

    def normal(self):
        u1 = max(self.uniform(), 1e-300)
        u2 = self.uniform()
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def _mm_slot_table():
    groups = [[0], [27, 9, 3, 1], [54, 18, 6, 2], [36, 4], [63, 45, 7, 5], [72, 8], [30, 12, 28, 10],
              [57, 21, 33, 15, 55, 19, 29, 11], [39, 37, 31, 13], [66, 48, 64, 46, 34, 16, 32, 14],
              [75, 73, 35, 17], [60, 24, 56, 20], [42, 58, 22, 38], [69, 51, 61, 25, 65, 47, 59, 23],
              [78, 74, 62, 26], [40], [67, 49, 43, 41], [76, 44], [70, 52, 68, 50], [79, 77, 71, 53], [80]]
    t = {}
    for slot, uids in enumerate(groups):
        for u in uids:
            t[u] = slot
    return t


_SLOT = _mm_slot_table()


def quat_to_rot(q):
    """Rotation matrix of the normalised quaternion (w, x, y, z)."""
    w, x, y, z = np.asarray(q, dtype=np.float64) / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def cubic(C11, C12, C44, R=None):
    R = np.eye(3) if R is None else np.asarray(R, dtype=np.float64)
    Ct = np.zeros((3, 3, 3, 3))
    for i, j, k, l in itertools.product(range(3), repeat=4):
        if i == j == k == l:
            Ct[i, j, k, l] = C11
        elif i == k and j == l:
            Ct[i, j, k, l] = C44
        elif i == j and k == l:
            Ct[i, j, k, l] = C12
    full = np.einsum("pi,sk,ijkl,qj,tl->pqst", R, R, Ct, R, R)
    out = np.zeros(21)
    for p, q, s, t in itertools.product(range(3), repeat=4):
        out[_SLOT[p + 3 * q + 9 * s + 27 * t]] = full[p, q, s, t]
    return out


def node_coords(n, lo=0.0, hi=1.0):
    return lo + (hi - lo) * np.arange(n + 1) / n


def sphere_inclusion(n=64, radius=0.25, lam_m=1.0, mu_m=1.0, lam_i=10.0, mu_i=10.0, eig=1e-3):
    """Isotropic matrix + smoothed sphere (eta = (1 - tanh((r-R)/(2 dx)))/2).
    Returns (ddw AoS (lambda, mu) per node, F0 AoS 9 per node) on (n+1)^3 nodes."""
    x = node_coords(n)
    dx = 1.0 / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    eta = 0.5 * (1.0 - np.tanh((r - radius) / (2.0 * dx)))
    eta = eta.reshape(-1)
    ddw = np.empty((eta.size, 2))
    ddw[:, 0] = eta * lam_i + (1.0 - eta) * lam_m
    ddw[:, 1] = eta * mu_i + (1.0 - eta) * mu_m
    F0 = np.zeros((eta.size, 9))
    F0[:, 0] = F0[:, 4] = F0[:, 8] = eta * eig
    return ddw.reshape(-1), F0.reshape(-1)


def ellipse_eta(n, prob_lo, prob_hi, a, x0=(0.0, 0.0, 0.0), eps=0.1):
    """IC::Ellipse (IC/Ellipse.H:58-59) at the nodes of an n^3-cell box:
    eta = 1/2 - 1/2 erf(((x-x0)^T A (x-x0) - 1) / eps / |A (x-x0)|), A =
    diag(1/a^2).  (n+1)^3 values, i fastest; at x = x0 (0/0) eta = 1."""
    from math import erf
    ax = [prob_lo[d] + (prob_hi[d] - prob_lo[d]) * np.arange(n + 1) / n for d in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    d = [X - x0[0], Y - x0[1], Z - x0[2]]
    A = [1.0 / (a[k] * a[k]) for k in range(3)]
    q = sum(A[k] * d[k] * d[k] for k in range(3))
    norm = np.sqrt(sum((A[k] * d[k]) ** 2 for k in range(3)))
    with np.errstate(divide="ignore", invalid="ignore"):
        arg = (q - 1.0) / eps / norm
    arg = np.where(norm > 0, arg, -np.inf)
    try:
        from scipy.special import erf as verf   # vectorised; erf(+-inf) = +-1
    except ImportError:
        verf = np.vectorize(lambda v: erf(v) if np.isfinite(v) else np.sign(v))
    return (0.5 - 0.5 * verf(arg)).reshape(-1)


def eshelby_problem(n, gd):
    """The reference's tests/Eshelby configuration on one uniform level of n^3
    cells (gd: tests/golden/eshelby_kat.json): affine isotropic moduli from E,
    nu everywhere and the eigenstrain F0_inside weighted by the ellipse eta
    (Integrator/Mechanics.H:249-253 mixing, both models share E and nu).
    Returns (ddw AoS (lambda, mu) per node, F0 AoS 9 per node)."""
    E, nu = gd["E"], gd["nu"]
    lam = E * nu / (1 + nu) / (1 - 2 * nu)
    mu = E / 2 / (1 + nu)
    el = gd["ellipse"]
    eta = ellipse_eta(n, gd["prob_lo"], gd["prob_hi"], el["a"], el["x0"], el["eps"])
    ddw = np.tile([lam, mu], eta.size)
    F0 = (eta[:, None] * np.asarray(gd["F0_inside"], float)[None, :]).reshape(-1)
    return ddw, F0


def voronoi_seeds(ngrains=64, seed=20260, C11=1.68, C12=1.21, C44=0.75):
    rng = SplitMix64(seed)
    pts = np.array([[rng.uniform() for _ in range(3)] for _ in range(ngrains)])
    table = np.zeros((ngrains, 21))
    for g in range(ngrains):
        q = [rng.normal() for _ in range(4)]
        table[g] = cubic(C11, C12, C44, quat_to_rot(q))
    return pts, table


def voronoi_grain_ids(n, pts):
    """Nearest seed (Euclidean, non-periodic) of every node, int32, (n+1)^3."""
    x = node_coords(n)
    ids = np.empty((n + 1, n + 1, n + 1), np.int32)
    YY, XX = np.meshgrid(x, x, indexing="ij")
    for k in range(n + 1):
        d2 = ((XX[..., None] - pts[:, 0]) ** 2 + (YY[..., None] - pts[:, 1]) ** 2 + (x[k] - pts[:, 2]) ** 2)
        ids[k] = np.argmin(d2, axis=-1)
    return ids.reshape(-1)


RVE_EDGES = (32, 48, 64, 80, 96)


def rve_params(q, seed=4242, edges=RVE_EDGES, contrast_max=100.0):
    """The random draws of periodic RVE number q of a batch: edge uniform in
    `edges` cells, 1-8 ellipsoidal isotropic inclusions (centre uniform in the
    cube, semi-axes 0.05-0.2 of the edge, uniformly random orientation,
    stiffness contrast log-uniform in [1, contrast_max]) in a matrix with
    lambda = mu = 1, and a macroscopic strain with symmetric entries
    U(+-1e-3) applied as the uniform eigenstrain F0 = -strain.
    Returns (n, inclusion table (ninc, 16): centre[3], semi-axes[3], R[9]
    row-major, log(contrast); F0 (3x3))."""
    rng = SplitMix64(seed * 1000003 + q)
    n = int(edges[min(int(rng.uniform() * len(edges)), len(edges) - 1)])
    ninc = 1 + min(int(rng.uniform() * 8), 7)
    table = np.zeros((ninc, 16))
    for t in range(ninc):
        table[t, 0:3] = [rng.uniform() for _ in range(3)]
        table[t, 3:6] = [0.05 + 0.15 * rng.uniform() for _ in range(3)]
        table[t, 6:15] = quat_to_rot([rng.normal() for _ in range(4)]).reshape(9)
        table[t, 15] = np.log(contrast_max) * rng.uniform()
    e = np.zeros((3, 3))
    for a, b in ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)):
        e[a, b] = e[b, a] = (2.0 * rng.uniform() - 1.0) * 1e-3
    return n, table, -e


def ellipsoid_field(n, table, width=2.0):
    """Host evaluation of the inclusion field: lambda = mu = exp(max_t phi_t *
    log(contrast_t)), phi = (1 - tanh(s n / w_t))/2 with s = (|y/axes| - 1) *
    mean(axes) the approximate distance to the surface, y = d R, d the
    nearest periodic image of node - centre, and w_t = width * max(1,
    log10(contrast_t)) cells, so that log(stiffness) changes by at most about
    0.6 per cell.  AoS (lambda, mu) on (n+1)^3 nodes."""
    x = np.arange(n + 1) / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    P = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    logc = np.zeros(P.shape[0])
    for t in range(table.shape[0]):
        c, axes, R, lk = table[t, 0:3], table[t, 3:6], table[t, 6:15].reshape(3, 3), table[t, 15]
        d = P - c
        d -= np.round(d)              # nearest periodic image
        y = d @ R                     # components in the inclusion frame
        r = np.sqrt(np.sum((y / axes) ** 2, axis=1))
        s = (r - 1.0) * axes.mean()
        wq = width * max(1.0, lk / np.log(10.0))   # wider for contrasts above 10
        phi = 0.5 * (1.0 - np.tanh(s * n / wq))
        logc = np.maximum(logc, phi * lk)
    contrast = np.exp(logc)
    ddw = np.empty((P.shape[0], 2))
    ddw[:, 0] = contrast
    ddw[:, 1] = contrast
    return ddw.reshape(-1)


def rve_problem(q, seed=4242, edges=RVE_EDGES, contrast_max=100.0, width=2.0):
    """Periodic RVE number q of a batch (rve_params), its field evaluated on the host.

    The inclusion boundary is diffuse: log(contrast) follows a tanh profile of
    `width` cells across the approximate distance to the ellipsoid surface
    (the 2-cell profile of the sphere-inclusion workload), as a phase-field
    microstructure would give.  The operator's grad(C) term is a central
    difference, and a stiffness jump of tens across one cell makes it lose
    diagonal dominance: the damped-Jacobi multigrid then diverges on the same
    material with any boundary condition, so sharp inclusions are not a
    usable workload for this solver.
    Returns (n, ddw AoS (lambda, mu) on the (n+1)^3 nodal box, F0 (3x3))."""
    n, table, F0 = rve_params(q, seed, edges, contrast_max)
    return n, ellipsoid_field(n, table, width), F0


def rve_problem_device(q, seed=4242, edges=RVE_EDGES, contrast_max=100.0, width=2.0, out=None):
    """rve_problem with the field evaluated on the GPU (agb_gen_ellipsoids).
    Returns (n, ddw as a CUDA float64 tensor, F0)."""
    import torch
    n, table, F0 = rve_params(q, seed, edges, contrast_max)
    ddw = out if out is not None else torch.empty(2 * (n + 1) ** 3, dtype=torch.float64, device="cuda")
    _check(_gen().agb_gen_ellipsoids(_cells(n), table.shape[0], _dptr(np.ascontiguousarray(table.reshape(-1))),
                                     float(width), ctypes.c_void_p(ddw.data_ptr()), 1, None))
    return n, ddw, F0


def voronoi_cubic(n=256, ngrains=64, seed=20260, C11=1.68, C12=1.21, C44=0.75):
    """Returns (ddw AoS 21 per node, grain ids, table)."""
    pts, table = voronoi_seeds(ngrains, seed, C11, C12, C44)
    ids = voronoi_grain_ids(n, pts)
    return table[ids].reshape(-1), ids, table


def voronoi_cubic_device(n=256, ngrains=64, seed=20260, C11=1.68, C12=1.21, C44=0.75):
    """voronoi_cubic with the per-node field built on the GPU
    (agb_gen_voronoi_cubic).  Returns (ddw CUDA float64 tensor, ids CUDA
    int32 tensor, table)."""
    import torch
    pts, table = voronoi_seeds(ngrains, seed, C11, C12, C44)
    N = (n + 1) ** 3
    ddw = torch.empty(21 * N, dtype=torch.float64, device="cuda")
    ids = torch.empty(N, dtype=torch.int32, device="cuda")
    _check(_gen().agb_gen_voronoi_cubic(_cells(n), ngrains, _dptr(np.ascontiguousarray(pts.reshape(-1))),
                                        _dptr(np.ascontiguousarray(table.reshape(-1))),
                                        ctypes.c_void_p(ddw.data_ptr()), ctypes.c_void_p(ids.data_ptr()), 1, None))
    return ddw, ids, table


def sphere_inclusion_device(n=64, radius=0.25, lam_m=1.0, mu_m=1.0, lam_i=10.0, mu_i=10.0, eig=1e-3):
    """sphere_inclusion evaluated on the GPU (agb_gen_sphere): (ddw, F0) CUDA tensors."""
    import torch
    N = (n + 1) ** 3
    ddw = torch.empty(2 * N, dtype=torch.float64, device="cuda")
    F0 = torch.empty(9 * N, dtype=torch.float64, device="cuda")
    _check(_gen().agb_gen_sphere(_cells(n), radius, lam_m, mu_m, lam_i, mu_i, eig, ctypes.c_void_p(ddw.data_ptr()),
                                 ctypes.c_void_p(F0.data_ptr()), 1, None))
    return ddw, F0


def _gen():
    from ._lib import lib
    return lib()


def _check(st):
    from ._lib import check
    check(st)


def _cells(n):
    return (ctypes.c_int * 3)(n, n, n)


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
