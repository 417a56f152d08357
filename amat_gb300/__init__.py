"""GB300-native assembly-free (AFM) finite-element operator.

A drop-in, single-rank replacement for the stored-element-matrix matvec of
paralab/aMat (par::aMatFree, MATFREE_TYPE::QUASI_FREE) and the solver calls
around it, running on hand-written sm_103a kernels behind the C ABI of
include/afm.h.
"""
from .afm import BC_METH, CG_NORM, MATFREE_TYPE, PRECISION, Maps, aMatFree  # noqa: F401
from ._native import AfmError, libafm, libproblems  # noqa: F401

__all__ = ["BC_METH", "CG_NORM", "MATFREE_TYPE", "PRECISION", "Maps", "aMatFree", "AfmError", "libafm",
           "libproblems"]
