"""Extract the reference's known-answer data for the elastic path into
tests/golden/solid_kat.json and tests/golden/eshelby_kat.json.

Run where the reference tree is available, giving its root as the only
argument or in ALAMO_REFERENCE (there is no default path); the JSON travels
with the repository:

    python tests/golden/make_golden.py <alamo source tree>
  Sources (paths relative to the alamo tree):
  tests/Solid/input, tests/Solid/test                 4^3 cells, tensiontest
                                                      uniaxial_stress, disp (0,1:0,0.01),
                                                      tolerance 1e-4
  tests/Solid/reference/linear-cubic.dat, affine-cubic.dat   trac_xhi_x vs time
  tests/UniaxialTension/input, tests/UniaxialTension/test    analytic u_x, sigma_xx,
                                                      tolerance 1e-8
  tests/Eshelby/input, tests/Eshelby/test             ellipsoidal inclusion (affine.isotropic,
                                                      eigenstrain 1e-3 I inside), box [-8,8]^3,
                                                      zero displacement on the faces
  tests/Eshelby/reference/Eshelby_displacement.csv, Eshelby_sigma_normal.csv
                                                      analytic profiles along the ray
                                                      x = y = 0.25, z in [-2, 2]; tolerance 0.1
"""
import json
import os
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ALAMO_REFERENCE")
if not REF:
    sys.exit("usage: make_golden.py <alamo source tree>  (or set ALAMO_REFERENCE)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solid_kat.json")
OUT_ESHELBY = os.path.join(os.path.dirname(os.path.abspath(__file__)), "eshelby_kat.json")


def load_csv(path):
    with open(path) as f:
        head = f.readline().strip().split(",")
        rows = [list(map(float, line.split(","))) for line in f if line.strip()]
    return {h: [r[i] for r in rows] for i, h in enumerate(head)}


def load_dat(path):
    with open(path) as f:
        head = f.readline().split()
        rows = [list(map(float, line.split())) for line in f if line.strip()]
    return {h: [r[i] for r in rows] for i, h in enumerate(head)}


def parse_bc(path):
    """bc.constant.type.<region> / bc.constant.val.<region> lines of a reference input file."""
    out = {}
    for line in open(path):
        line = line.split("#")[0].strip()
        if not line.startswith("bc.constant."):
            continue
        key, val = [t.strip() for t in line.split("=", 1)]
        kind, region = key.split(".")[2], key.split(".")[3]
        toks = val.split()
        out[("val." if kind == "val" else "") + region] = [float(t) for t in toks] if kind == "val" else toks
    return out


def main():
    solid = os.path.join(REF, "tests", "Solid")
    out = {
        "source": "alamo tests/Solid/reference/*.dat and tests/UniaxialTension (analytic)",
        "solid": {
            "n_cells": [4, 4, 4], "prob_lo": [0, 0, 0], "prob_hi": [1, 1, 1],
            "bc": {"type": "uniaxial_stress", "disp_of_t": [[0.0, 0.0], [1.0, 0.01]]},
            "moduli": {"C11": 168.3, "C12": 1.221, "C44": 0.757},
            "tolerance": 1e-4,
            "linear-cubic": load_dat(os.path.join(solid, "reference", "linear-cubic.dat")),
            "affine-cubic": load_dat(os.path.join(solid, "reference", "affine-cubic.dat")),
            "affine_F0": [0.001, 0, 0, 0, 0.001, 0, 0, 0, 0.001],
        },
        "uniaxial_tension": {
            "E": 210.0, "nu": 0.3, "disp": 0.1, "L": 16.0, "prob_lo": [-8, -8, -8], "prob_hi": [8, 8, 8],
            "tolerance": 1e-8,
            "bc_constant": parse_bc(os.path.join(REF, "tests", "UniaxialTension", "input")),
        },
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)
    esh = os.path.join(REF, "tests", "Eshelby")
    eshelby = {
        "source": "alamo tests/Eshelby (input, test, reference/*.csv)",
        "prob_lo": [-8.0, -8.0, -8.0], "prob_hi": [8.0, 8.0, 8.0],
        "E": 210.0, "nu": 0.3,
        "F0_inside": [0.001, 0, 0, 0, 0.001, 0, 0, 0, 0.001],
        "ellipse": {"a": [1.0, 0.75, 0.5], "x0": [0.0, 0.0, 0.0], "eps": 0.1},
        "ray": {"x": 0.25, "y": 0.25, "z": [-2.0, 2.0]},
        "tolerance": 0.1,
        # the reference script scales the tables: displacement / 10000, stress * 210 / 1000
        "disp_scale": 1.0 / 10000.0, "sigma_scale": 210.0 / 1000.0,
        "displacement": load_csv(os.path.join(esh, "reference", "Eshelby_displacement.csv")),
        "sigma_normal": load_csv(os.path.join(esh, "reference", "Eshelby_sigma_normal.csv")),
    }
    with open(OUT_ESHELBY, "w") as f:
        json.dump(eshelby, f, indent=0)
    print("wrote", OUT_ESHELBY)


if __name__ == "__main__":
    main()
