"""alamo_gb300: GB300 (sm_103a) implementation of Alamo's nodal linear-elastic
multigrid solve (Operator::Elastic / Solver::Nonlocal::Linear), behind the C
ABI of include/agb.h.

The compute path is libalamo_gb300.so (built by alamo_gb300.build); importing
the operator classes loads it and fails loudly when it is missing.
"""
from ._lib import AgbError, exported_symbols  # noqa: F401
from .elastic import (Constant, Elastic, Linear, Newton, TensionTest,  # noqa: F401
                      default_params, FACE, FACE_NAMES)

__all__ = ["AgbError", "Constant", "TensionTest", "Elastic", "Linear", "Newton", "default_params",
           "exported_symbols", "FACE", "FACE_NAMES"]
