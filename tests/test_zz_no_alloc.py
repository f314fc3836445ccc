"""nbk_density_noalloc: the SPH density for callers that cannot allocate device memory
while they run (simulation codes and in-situ halo finders that reserve the GPU's memory
for their own pool at start-up and allow no allocation afterwards). It must give what
nbk_density gives, and what the oracle gives, call after call, with its scratch in a
static device array; it must allocate nothing; and it must refuse what it cannot do
(trees larger than that array, phase-space trees, k above the other particles).

Collected last on purpose: it leaves the shared static scratch holding the last call's
contents, and a failure here should not stop the rest of a run that halts at the first
failure."""
import ctypes

import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree, _capi
from nbodylib_gb300 import synthetic as syn
from nbodylib_gb300.kdtree import TPHS
from tests.helpers import assert_density_close

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 1 << 22  # the scratch size stated in include/nbkdt.h
NBK_ERR_INVALID, NBK_ERR_UNSUPPORTED, NBK_ERR_TOO_FEW = 1, 2, 5


def _density_noalloc(tree, k, out):
    lib = _capi.load()
    return lib.nbk_density_noalloc(tree._h, k, ctypes.c_void_p(out.data_ptr()))


def test_noalloc_density_matches_nbk_density_and_oracle_twice(gpu, port_built):
    import torch
    pos, mass = syn.clustered_box(200000, 100.0, seed=71)
    t = KDTree(pos, None, mass, 16, kerntype=0)
    want = t.CalcDensity(32)  # the existing entry point (host output)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, None, backend="port", nthreads=16)
    ref = o.density(32)
    o.close()
    for call in range(2):
        out = torch.full((len(mass),), -1.0, dtype=torch.float64, device="cuda")
        _capi.check(_density_noalloc(t, 32, out))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert_density_close(got, want, f"no-alloc call {call} vs nbk_density")
        assert_density_close(got, ref, f"no-alloc call {call} vs the oracle")
    # a different, smaller tree next: the scratch is cleared per call, not carried over
    pos2, mass2 = syn.uniform_box(5000, 1.0, seed=72)
    t2 = KDTree(pos2, None, mass2, 16, kerntype=0)
    out2 = torch.empty(len(mass2), dtype=torch.float64, device="cuda")
    _capi.check(_density_noalloc(t2, 16, out2))
    assert_density_close(out2.cpu().numpy(), t2.CalcDensity(16), "no-alloc second tree")


def test_noalloc_density_allocates_nothing(gpu):
    import torch
    lib = _capi.load()
    pos, mass = syn.clustered_box(100000, 100.0, seed=74)
    t = KDTree(pos, None, mass, 16, kerntype=0)
    out = torch.empty(len(mass), dtype=torch.float64, device="cuda")
    _capi.check(_density_noalloc(t, 32, out))  # first call: set-up, modules loaded
    torch.cuda.synchronize()
    live = lib.nbk_debug_live_allocations()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _capi.check(_density_noalloc(t, 32, out))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert lib.nbk_debug_live_allocations() == live
    assert free1 == free0


def test_noalloc_density_refusals(gpu):
    import torch
    lib = _capi.load()
    # phase-space trees are not supported by this entry point
    pos, mass, vel = syn.clustered_box(3000, 20.0, seed=75, velocities=True)
    tp = KDTree(pos, vel, mass, 16, treetype=TPHS, kerntype=0)
    out = torch.empty(len(mass), dtype=torch.float64, device="cuda")
    assert _density_noalloc(tp, 8, out) == NBK_ERR_UNSUPPORTED
    # k above the other particles: the reference exits here
    t = KDTree(pos[:20], None, mass[:20], 16, kerntype=0)
    out20 = torch.empty(20, dtype=torch.float64, device="cuda")
    assert _density_noalloc(t, 20, out20) == NBK_ERR_TOO_FEW
    assert "exceeds" in lib.nbk_last_error().decode()
    _capi.check(_density_noalloc(t, 19, out20))


def test_noalloc_density_rejects_trees_beyond_the_scratch(gpu):
    import torch
    n = MAX_PARTICLES + 1
    pos = np.random.default_rng(73).random((n, 3))
    t = KDTree(pos, None, None, 16, kerntype=0)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    st = _density_noalloc(t, 8, out)
    assert st == NBK_ERR_INVALID
    assert "scratch holds at most" in _capi.load().nbk_last_error().decode()
