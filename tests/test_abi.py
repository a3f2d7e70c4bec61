"""CPU: the C ABI library loads, exports every symbol include/agb.h declares,
and refuses to run without a GPU (no CPU fallback).  No compute calls."""
import ctypes
import subprocess

import pytest


def _built():
    from alamo_gb300 import build
    return build.build()


def test_exports_every_declared_symbol():
    path = _built()
    from alamo_gb300 import _lib
    L = ctypes.CDLL(path)
    declared = _lib.exported_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    for s in declared:
        assert (" T " + s) in out, s


def test_no_gpu_fails_loudly():
    _built()
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from alamo_gb300 import AgbError, Elastic
    with pytest.raises(AgbError) as e:
        Elastic([8, 8, 8])
    assert "AGB_CUDA" in str(e.value)


def test_default_params_match_reference_defaults():
    _built()
    from alamo_gb300 import default_params
    p = default_params()
    assert (p.pre_smooth, p.post_smooth, p.final_smooth, p.bottom_smooth) == (2, 2, 8, 0)
    assert p.max_fmg_iter == 100000000 and p.bottom_max_iter == 200 and p.max_iter == 200
    assert p.bottom_tol_rel == 1e-4 and p.omega < 0
    assert p.krylov == 0   # the FP32 cycles alone unless a caller asks for the GCR acceleration


def test_params_struct_matches_header():
    """The ctypes mirror of agb_solver_params lists the header's fields in the
    header's order with the header's types (the struct crosses the ABI by
    pointer)."""
    import os
    import re
    from alamo_gb300 import _lib
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = open(os.path.join(root, "include", "agb.h")).read()
    body = re.search(r"typedef struct \{([^}]*)\} agb_solver_params;", src).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"\b(int|double)\s+(\w+)\s*;", body)
    ctype = {"int": ctypes.c_int, "double": ctypes.c_double}
    assert [(n, ctype[t]) for t, n in fields] == list(_lib.AgbSolverParams._fields_)
