"""Tests of the boundary: libnbkdt.so builds for sm_103a, loads, and exports every entry
point include/nbkdt.h declares (CPU, no compute calls); on a GPU, the runtime runs its
kernels from sm_103a code."""
import ctypes
import os
import re

import pytest

from nbodylib_gb300 import _build, _capi

HEADER = os.path.join(os.path.dirname(__file__), "..", "include", "nbkdt.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nbk_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_hot_path():
    names = declared_functions()
    for must in ["nbk_create", "nbk_knn", "nbk_density", "nbk_veldensity", "nbk_fof",
                 "nbk_ball_tagged", "nbk_ball_mark", "nbk_density_adjoint", "nbk_batch_density"]:
        assert must in names


def test_library_builds_loads_and_exports_every_symbol(lib_built):
    lib = ctypes.CDLL(_build.LIB)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers every declared entry point
    assert set(declared_functions()) <= set(_capi.SIGNATURES)


@pytest.mark.gpu
def test_library_kernels_run_as_sm103a(gpu):
    # what the CUDA runtime selected for a product kernel on this GPU: SASS for sm_103a
    # and PTX of the same target (cudaFuncGetAttributes through the library itself)
    lib = _capi.load()
    b, p = ctypes.c_int(), ctypes.c_int()
    _capi.check(lib.nbk_kernel_binary_version(ctypes.byref(b), ctypes.byref(p)))
    assert (b.value, p.value) == (103, 103)
