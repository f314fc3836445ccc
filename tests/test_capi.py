"""CPU tests of the boundary: libnbkdt.so builds for sm_103a, loads, and exports every
entry point include/nbkdt.h declares (no compute calls: there may be no GPU)."""
import ctypes
import os
import re

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


def test_library_is_sm103a():
    # the build passes exactly one target, compute_103a -> sm_103a
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
