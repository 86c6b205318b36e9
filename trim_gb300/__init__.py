"""trim_gb300: GB300 (sm_103a) symmetric block-tensor permute + sector-GEMM
path of the Uni10 tensor-network library, behind a C ABI (include/trim_gb300.h)
and its C++ drop-in API (include/uni10.hpp).

Python access goes through ``trim_gb300.capi`` (ctypes over the in-tree
libtrim_gb300.so) and ``trim_gb300.uni10`` (UniTensor / Network mirror).
"""
from . import capi  # noqa: F401

__all__ = ["capi", "build"]


def build(verbose: bool = False) -> str:
    from .buildlib import build as _b

    return _b(verbose=verbose)
