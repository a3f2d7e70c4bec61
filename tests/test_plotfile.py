"""The nodal plotfile writer (agb_write_node_plotfile, host memory, no GPU
needed) against the reader: component names as Alamo's Set::Field gives them,
geometry, per-component minima and maxima, the data bit for bit, and the
nodeoutput.visit index across steps."""
import os

import numpy as np


def test_node_plotfile_round_trip(tmp_path):
    from alamo_gb300 import build
    build.build()
    from alamo_gb300.plotfile import read_node_plotfile, write_node_plotfile
    n = (6, 5, 4)
    N = (n[0] + 1) * (n[1] + 1) * (n[2] + 1)
    rng = np.random.default_rng(3)
    u = rng.standard_normal(3 * N)
    sig = rng.standard_normal(9 * N)
    eta = rng.random(N)
    lo, hi = (-1.0, 0.0, 2.0), (2.0, 0.5, 3.0)
    root = tmp_path / "output"
    d0 = write_node_plotfile(root, 0, 0.0, n, [("disp", u), ("stress", sig), ("eta", eta)], lo, hi)
    d7 = write_node_plotfile(root, 7, 0.35, n, [("disp", 2 * u)], lo, hi)
    assert os.path.basename(d0) == "00000node" and os.path.basename(d7) == "00007node"
    p = read_node_plotfile(d0)
    assert p["names"] == (["disp_x", "disp_y", "disp_z"] +
                          ["stress_" + a + b for a in "xyz" for b in "xyz"] + ["eta"])
    assert p["time"] == 0.0 and p["step"] == 0 and p["finest_level"] == 0
    assert p["prob_lo"] == list(lo) and p["prob_hi"] == list(hi)
    assert np.allclose(p["dx"], [(hi[d] - lo[d]) / n[d] for d in range(3)], rtol=0, atol=1e-15)
    assert p["domain"] == ([0, 0, 0], [n[0] - 1, n[1] - 1, n[2] - 1], [0, 0, 0])
    assert p["box"] == ([0, 0, 0], list(n), [1, 1, 1])
    shape = (n[2] + 1, n[1] + 1, n[0] + 1)
    for c, name in enumerate(["disp_x", "disp_y", "disp_z"]):
        assert np.array_equal(p["fields"][name], u[c * N:(c + 1) * N].reshape(shape))
    for c in range(9):
        name = p["names"][3 + c]
        assert np.array_equal(p["fields"][name], sig[c * N:(c + 1) * N].reshape(shape))
    assert np.array_equal(p["fields"]["eta"], eta.reshape(shape))
    allc = np.concatenate([u, sig, eta]).reshape(13, N)
    assert np.array_equal(p["min"], allc.min(axis=1)) and np.array_equal(p["max"], allc.max(axis=1))
    q = read_node_plotfile(d7)
    assert q["time"] == 0.35 and q["step"] == 7
    assert np.array_equal(q["fields"]["disp_y"], 2 * u[N:2 * N].reshape(shape))
    with open(root / "nodeoutput.visit") as f:
        assert f.read().split() == ["00000node/Header", "00007node/Header"]
    assert (root / "00000node" / "Checkpoint").read_text() == "(1 0\n((0,0,0) (5,4,3) (0,0,0))\n)"


def test_node_plotfile_rejects_bad_fields(tmp_path):
    import pytest
    from alamo_gb300 import AgbError, build
    build.build()
    from alamo_gb300.plotfile import write_node_plotfile
    n = (2, 2, 2)
    with pytest.raises((AgbError, ValueError)):
        write_node_plotfile(tmp_path, 0, 0.0, n, [("bad", np.zeros(2 * 27))])
    with pytest.raises(ValueError):
        write_node_plotfile(tmp_path, 0, 0.0, n, [("short", np.zeros(26))])


# The files AMReX's WriteMultiLevelPlotfile writes for a one-level, one-box
# nodal MultiFab (what Integrator::WritePlotFile calls, Integrator.cpp:1022),
# restated by hand from AMReX's plotfile layout (WriteGenericPlotfileHeader;
# VisMF header version 1 written "NFiles", minima and maxima in scientific
# notation with 16 digits after the point; the FAB header of a little-endian
# IEEE double FAB): a 2 x 1 x 1-cell box on [0,1] x [0,0.5] x [0,0.5] at time
# 0.25, step 3, one 3-component field "disp".
GOLDEN_HEADER = """HyperCLaw-V1.1
3
disp_x
disp_y
disp_z
3
0.25
0
0 0 0 
1 0.5 0.5 

((0,0,0) (1,0,0) (0,0,0)) 
3 
0.5 0.5 0.5 
0
0
0 1 0.25
3
0 1
0 0.5
0 0.5
Level_0/Cell
"""
GOLDEN_CELL_H = """1
1
3
0
(1 0
((0,0,0) (2,1,1) (1,1,1))
)
1
FabOnDisk: Cell_D_00000 0

1,3
0.0000000000000000e+00,-2.7500000000000000e+00,1.0000000000000000e+00,

1,3
5.5000000000000000e+00,0.0000000000000000e+00,1.0000000000000000e+00,

"""
GOLDEN_FAB_HEAD = b"FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))((0,0,0) (2,1,1) (1,1,1)) 3\n"


def test_node_plotfile_matches_amrex_layout(tmp_path):
    from alamo_gb300 import build
    build.build()
    from alamo_gb300.plotfile import write_node_plotfile
    n = (2, 1, 1)
    N = 12
    ux = 0.5 * np.arange(N)
    uy = 0.0 - 0.25 * np.arange(N)   # (+0.0 at node 0)
    uz = np.ones(N)
    d = write_node_plotfile(tmp_path, 3, 0.25, n, [("disp", np.concatenate([ux, uy, uz]))], (0.0, 0.0, 0.0),
                            (1.0, 0.5, 0.5))
    assert open(os.path.join(d, "Header")).read() == GOLDEN_HEADER
    assert open(os.path.join(d, "Level_0", "Cell_H")).read() == GOLDEN_CELL_H
    raw = open(os.path.join(d, "Level_0", "Cell_D_00000"), "rb").read()
    assert raw[:len(GOLDEN_FAB_HEAD)] == GOLDEN_FAB_HEAD
    body = np.frombuffer(raw[len(GOLDEN_FAB_HEAD):], dtype="<f8")
    assert np.array_equal(body, np.concatenate([ux, uy, uz]))
