"""GB300-native TreeTime ancestral-reconstruction hot path.

Public API mirrors TreeTime's: ``TreeAnc``, ``GTR``, ``GTR_site_specific``
and the TreeTime exception types.  Compute runs in hand-written sm_103a CUDA
kernels (``treetime_gb300/csrc``) behind a C-ABI shared library.
"""

from .errors import TreeTimeError, MissingDataError, UnknownMethodError, NotReadyError, TreeTimeUnknownError
from .gtr import GTR, GTR_site_specific

version = "0.1.0"

__all__ = ["TreeAnc", "GTR", "GTR_site_specific", "TreeTimeError", "MissingDataError", "UnknownMethodError",
           "NotReadyError", "TreeTimeUnknownError"]


def __getattr__(name):
    if name == "TreeAnc":
        from .treeanc import TreeAnc
        return TreeAnc
    raise AttributeError(name)
