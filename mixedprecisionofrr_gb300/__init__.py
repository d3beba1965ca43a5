"""GB300-native orthogonalization-free projection eigen/SVD solvers (MixedPrecisionOFRR path).

The compute lives in ``libofrr_gb300.so`` (CUDA, sm_103a), whose C ABI is ``include/ofrr.h``.
``api`` mirrors the reference's MATLAB interface on top of that ABI.
"""
from . import _lib  # noqa: F401

__all__ = ["api", "build", "lib"]


def lib():
    """The loaded shared library (raises if it was not built)."""
    return _lib.load()
