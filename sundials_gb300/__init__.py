"""sundials_gb300 -- GB300-native N_Vector, block-diagonal matrix / linear
solvers, fused SPGMR and a batched BDF integrator for SUNDIALS' CVODE/ARKODE
hot path.  The product is the C-ABI library ``lib/libsundials_gb300.so``
(headers in ``include/``); this package only builds and loads it."""
from ._lib import LIB_PATH, load  # noqa: F401

__all__ = ["load", "LIB_PATH"]
