"""GB300-native Feynman-Kac hot path of SpAc.

The compute path is libspac_fk.so (CUDA sm_103a kernels behind the C ABI in
include/spac_fk.h).  This package builds it in-tree and exposes a thin ctypes
binding (spac_gb300.fk) used by the tests and the benchmark.  There is no CPU
fallback: without the built library or a CUDA device every entry point raises.
"""
import os

from . import _build_lib

LIB_PATH = _build_lib.LIB


def build(verbose=False):
    """Compile libspac_fk.so for sm_103a into spac_gb300/_build/."""
    return _build_lib.build(verbose=verbose)


def lib_path():
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libspac_fk.so is not built: run spac_gb300.build() (nvcc, sm_103a)")
    return LIB_PATH
