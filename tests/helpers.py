"""Shared fixtures-by-function for the parity tests: seeded fields, BC sets and
reference-KAT problem builders.  The oracle is the checker."""
import json
import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "solid_kat.json")
TYPES = {"disp": O.DISP, "trac": O.TRAC, "neumann": O.NEUMANN, "periodic": O.PERIODIC}
FACES = ["xlo", "ylo", "zlo", "xhi", "yhi", "zhi", "ylozlo", "ylozhi", "yhizlo", "yhizhi", "zloxlo", "zloxhi",
         "zhixlo", "zhixhi", "xloylo", "xloyhi", "xhiylo", "xhiyhi", "xloylozlo", "xloylozhi", "xloyhizlo",
         "xloyhizhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo", "xhiyhizhi"]


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def rng(seed):
    return np.random.default_rng(seed)


def nodes(n):
    return (n[0] + 1) * (n[1] + 1) * (n[2] + 1)


def sync_periodic(v, n, periodic, ncomp):
    """Make periodic duplicate nodes equal to node 0 (full-box SoA/AoS-agnostic per component)."""
    a = v.reshape(ncomp, n[2] + 1, n[1] + 1, n[0] + 1)
    if periodic[0]:
        a[:, :, :, n[0]] = a[:, :, :, 0]
    if periodic[1]:
        a[:, :, n[1], :] = a[:, :, 0, :]
    if periodic[2]:
        a[:, n[2], :, :] = a[:, 0, :, :]
    return v


def random_ddw(n, sym, seed, periodic=(0, 0, 0)):
    r = rng(seed)
    nc = 2 if sym == O.ISO else 21
    d = r.uniform(0.5, 1.5, size=(nodes(n), nc))
    # AoS -> make periodic duplicates consistent
    a = d.reshape(n[2] + 1, n[1] + 1, n[0] + 1, nc)
    if periodic[0]:
        a[:, :, n[0]] = a[:, :, 0]
    if periodic[1]:
        a[:, n[1]] = a[:, 0]
    if periodic[2]:
        a[n[2]] = a[0]
    return np.ascontiguousarray(d.reshape(-1))


def random_field(n, seed, periodic=(0, 0, 0), ncomp=3, dtype=np.float64):
    v = rng(seed).uniform(-1, 1, size=ncomp * nodes(n))
    return sync_periodic(v, n, periodic, ncomp).astype(dtype)


def random_bc(seed, types=("disp", "trac", "neumann")):
    r = rng(seed)
    bt = np.zeros((26, 3), np.int32)
    bv = r.uniform(-0.1, 0.1, size=(26, 3))
    for f in range(26):
        for c in range(3):
            bt[f, c] = TYPES[types[r.integers(len(types))]]
    return bt, bv


def tension_bc_arrays(disp):
    """TensionTest uniaxial_stress (DISP mode) as (type, val) arrays, TensionTest.H:115-214."""
    from alamo_gb300.elastic import TensionTest
    t = TensionTest("uniaxial_stress", disp=disp)
    return t.type.copy(), t.val.copy()


def uniaxial_tension_bc():
    g = golden()["uniaxial_tension"]["bc_constant"]
    bt = np.full((26, 3), O.DISP, np.int32)
    bv = np.zeros((26, 3))
    for k, v in g.items():
        if k.startswith("val."):
            bv[FACES.index(k[4:])] = v
        else:
            bt[FACES.index(k)] = [TYPES[t] for t in v]
    return bt, bv


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def eshelby_errors(gd, z, u, sig):
    """The metrics of the reference's tests/Eshelby/test along its ray: for
    the displacement the relative L2 error sqrt(int (ref - u)^2 / int ref^2),
    for the normal stresses the relative 1-norm error int |ref - sig| /
    int |ref|, the reference tables scaled as the script scales them and
    interpolated at the sample points z (trapezoidal integrals)."""
    import numpy as np

    def integrate(x, y):
        return float(np.sum(0.5 * (y[1:] + y[:-1]) * np.diff(x)))

    dref = gd["displacement"]
    sref = gd["sigma_normal"]
    xd = np.asarray(dref["x"])
    xs = np.asarray(sref["x"])
    out = {}
    for c, key in enumerate(("disp1", "disp2", "disp3")):
        r = np.asarray(dref[key]) * gd["disp_scale"]
        out["u%d" % (c + 1)] = np.sqrt(integrate(z, (np.interp(z, xd, r) - u[c]) ** 2) / integrate(xd, r ** 2))
    for c, key in enumerate(("sigma11", "sigma22", "sigma33")):
        r = np.asarray(sref[key]) * gd["sigma_scale"]
        out["sig%d%d" % (c + 1, c + 1)] = integrate(z, np.abs(np.interp(z, xs, r) - sig[c])) / integrate(xs, np.abs(r))
    return out
