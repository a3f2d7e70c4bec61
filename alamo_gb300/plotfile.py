"""Nodal plotfiles in the AMReX plotfile format (agb_write_node_plotfile), and
a reader for them.

The writer is the library's: the directory <plot_file>/<step:05d>node that
Alamo's Integrator::WritePlotFile (Integrator/Integrator.cpp:795-1055) writes
for its nodal fields, one level and one box.  The reader parses what the
writer produces (the plotfile Header, the FabArray header Level_0/Cell_H and
the FAB Level_0/Cell_D_00000) into numpy arrays, the way yt's AMReX frontend
reads a single-level, single-grid plotfile.
"""
import ctypes
import os
import re

import numpy as np

from ._lib import check, lib
from .elastic import _ptr


def write_node_plotfile(plot_file, step, time, n_cells, fields, prob_lo=(0.0, 0.0, 0.0), prob_hi=(1.0, 1.0, 1.0)):
    """fields: list of (name, array) with 1, 3 or 9 components, each SoA over
    the (n+1)^3 nodes (numpy float64 or CUDA tensors, all on the same side).
    Returns the plotfile directory."""
    N = (n_cells[0] + 1) * (n_cells[1] + 1) * (n_cells[2] + 1)
    names = (ctypes.c_char_p * len(fields))(*[f[0].encode() for f in fields])
    ncomp, ptrs, mem = [], [], None
    for name, a in fields:
        size = a.numel() if hasattr(a, "numel") else a.size
        if size % N:
            raise ValueError("field %s: size %d is not a multiple of %d nodes" % (name, size, N))
        ncomp.append(size // N)
        p, m = _ptr(a)
        if mem is not None and m != mem:
            raise ValueError("all fields must be on the host or all on the device")
        mem = m
        ptrs.append(p)
    check(lib().agb_write_node_plotfile(str(plot_file).encode(), int(step), float(time),
                                        (ctypes.c_int * 3)(*n_cells), (ctypes.c_double * 3)(*prob_lo),
                                        (ctypes.c_double * 3)(*prob_hi), len(fields), names,
                                        (ctypes.c_int * len(fields))(*ncomp),
                                        (ctypes.c_void_p * len(fields))(*[p.value for p in ptrs]), mem))
    return os.path.join(str(plot_file), "%05dnode" % step)


def _box(s):
    m = re.match(r"\(\((-?\d+),(-?\d+),(-?\d+)\) \((-?\d+),(-?\d+),(-?\d+)\) \((\d+),(\d+),(\d+)\)\)", s.strip())
    if not m:
        raise ValueError("not a box: %r" % s)
    v = [int(x) for x in m.groups()]
    return v[0:3], v[3:6], v[6:9]


def read_node_plotfile(path):
    """Returns a dict: names, time, step, prob_lo, prob_hi, dx, domain (cell
    box), box (the FAB's nodal box), min, max (from Cell_H) and fields
    {component name: array of shape (nz+1, ny+1, nx+1)}."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    if lines[0] != "HyperCLaw-V1.1":
        raise ValueError("not a plotfile header: %r" % lines[0])
    nc = int(lines[1])
    names = lines[2:2 + nc]
    k = 2 + nc
    dim = int(lines[k])
    time = float(lines[k + 1])
    finest = int(lines[k + 2])
    lo = [float(v) for v in lines[k + 3].split()]
    hi = [float(v) for v in lines[k + 4].split()]
    # lines[k + 5] holds the refinement ratios (none for one level)
    domain = _box(lines[k + 6])
    step = int(lines[k + 7].split()[0])
    dx = [float(v) for v in lines[k + 8].split()]
    level_line = lines[k + 11].split()
    ngrids = int(level_line[1])
    mf_prefix = lines[k + 13 + dim * ngrids]
    with open(os.path.join(path, mf_prefix + "_H")) as f:
        h = f.read().split("\n")
    ncomp_h = int(h[2])
    fab_box = _box(h[5])
    m = re.match(r"FabOnDisk: (\S+) (\d+)", h[8])
    fab_file, fab_off = m.group(1), int(m.group(2))
    # two blocks "nfabs,ncomp" + one line of values each: minima, then maxima
    blocks = [i for i in range(9, len(h)) if re.match(r"^\d+,\d+$", h[i])]
    mins = [float(v) for v in h[blocks[0] + 1].rstrip(",").split(",")]
    maxs = [float(v) for v in h[blocks[1] + 1].rstrip(",").split(",")]
    with open(os.path.join(path, os.path.dirname(mf_prefix), fab_file), "rb") as f:
        f.seek(fab_off)
        head = f.readline().decode()
        m = re.match(r"FAB \(\(8, \(64 11 52 0 1 12 0 1023\)\),\(8, \((8 7 6 5 4 3 2 1|1 2 3 4 5 6 7 8)\)\)\)"
                     r"(\(\(.*\)\)) (\d+)", head)
        if not m:
            raise ValueError("unsupported FAB header: %r" % head)
        order = "<" if m.group(1).startswith("8") else ">"
        blo, bhi, _ = _box(m.group(2))
        ncf = int(m.group(3))
        shape = tuple(bhi[d] - blo[d] + 1 for d in (2, 1, 0))
        data = np.fromfile(f, dtype=order + "f8", count=ncf * shape[0] * shape[1] * shape[2])
    data = data.reshape(ncf, *shape)
    return {"names": names, "time": time, "step": step, "finest_level": finest, "prob_lo": lo, "prob_hi": hi,
            "dx": dx, "domain": domain, "box": fab_box, "ncomp": ncomp_h, "min": mins, "max": maxs,
            "fields": {names[c]: data[c] for c in range(nc)}}
