"""GB300 (sm_103a) engine for wholeCellFE's per-step cell mechanics.

The compute path is ``libwcfe.so`` (CUDA kernels + C ABI, include/wcfe.h);
this package holds its build recipe, the ctypes mirror of the ABI, the
reference constants and the synthetic cell generator.
"""
from .params import Params, default_params  # noqa: F401
