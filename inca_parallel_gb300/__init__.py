"""GB300 (sm_103a) engine for the intracule hot path of INCA.

The product is the C ABI library ``libinca_gpu.so`` (include/inca_gpu.h) and the ``inca_gpu``
driver built next to this file; ``_lib.Context`` is a thin ctypes binding of the library.
"""
from ._lib import INCA_FP64, INCA_FP64_SCREENED, INCA_MIXED, Context, IncaError, centercalc, load, read_dm2p  # noqa: F401,E501

__all__ = ["Context", "IncaError", "centercalc", "load", "read_dm2p", "INCA_FP64", "INCA_MIXED", "INCA_FP64_SCREENED"]
