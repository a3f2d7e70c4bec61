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
