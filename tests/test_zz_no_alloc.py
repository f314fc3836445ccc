"""nbk_density_noalloc: the SPH density for callers that cannot allocate device memory
while they run (codes that own all HBM through their own pool; work inside a stream
capture). It must give what nbk_density gives, call after call, with its scratch in a
static device array, and must refuse trees larger than that array.

Collected last on purpose: it leaves the shared static scratch holding the last call's
contents, and a failure here should not stop the rest of a run that halts at the first
failure."""
import ctypes

import numpy as np
import pytest

from nbodylib_gb300 import KDTree, _capi
from nbodylib_gb300 import synthetic as syn
from tests.helpers import assert_density_close

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 22  # the scratch size stated in include/nbkdt.h


def _density_noalloc(tree, k, out):
    lib = _capi.load()
    return lib.nbk_density_noalloc(tree._h, k, ctypes.c_void_p(out.data_ptr()))


def test_noalloc_density_matches_nbk_density_twice(gpu):
    import torch
    pos, mass = syn.clustered_box(200000, 100.0, seed=71)
    t = KDTree(pos, None, mass, 16, kerntype=0)
    want = t.CalcDensity(32)  # the existing entry point (host output)
    for call in range(2):
        out = torch.full((len(mass),), -1.0, dtype=torch.float64, device="cuda")
        _capi.check(_density_noalloc(t, 32, out))
        torch.cuda.synchronize()
        assert_density_close(out.cpu().numpy(), want, f"no-alloc call {call}")
    # a different, smaller tree next: the scratch is cleared per call, not carried over
    pos2, mass2 = syn.uniform_box(5000, 1.0, seed=72)
    t2 = KDTree(pos2, None, mass2, 16, kerntype=0)
    out2 = torch.empty(len(mass2), dtype=torch.float64, device="cuda")
    _capi.check(_density_noalloc(t2, 16, out2))
    assert_density_close(out2.cpu().numpy(), t2.CalcDensity(16), "no-alloc second tree")


def test_noalloc_density_rejects_trees_beyond_the_scratch(gpu):
    import torch
    n = MAX_PARTICLES + 1
    pos = np.random.default_rng(73).random((n, 3))
    t = KDTree(pos, None, None, 16, kerntype=0)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    st = _density_noalloc(t, 8, out)
    assert st == 1  # NBK_ERR_INVALID
    assert "scratch holds at most" in _capi.load().nbk_last_error().decode()
