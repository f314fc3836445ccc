"""Failure paths on the GPU, made without faulting, trapping or hanging the device.

The reference has two failure modes on this path, both `exit`: fewer than k neighbours in
CalcDensity (src/KDTree/KDCalcSmoothQuantities.cxx:273-276) and a full priority queue
(src/KDTree/PriorityQueue.h:49-53). The drop-in returns status codes instead, so these
tests check that a device-side limit that runs out, and a device allocation that fails,
come back as a clean status and leave the library usable and leak-free:

* the union-find loops of FOF stop at an iteration cap and set the call's error word;
  with the cap lowered to 1 (a test hook) the limit runs out on an ordinary input, the
  call returns NBK_ERR_DEVICE, and with the cap restored the same context gives the
  oracle's groups;
* a device allocation made to fail at each point of a tree's life in turn (creation,
  FOF, density; a batch's creation and search) returns NBK_ERR_NOMEM, and the library's
  count of live device allocations is back where it started afterwards.
"""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import BatchedDensity, KDTree, _capi
from nbodylib_gb300 import synthetic as syn
from nbodylib_gb300._capi import NbkError
from tests.helpers import assert_density_close, assert_same_partition

pytestmark = pytest.mark.gpu

NBK_ERR_NOMEM = 4
NBK_ERR_DEVICE = 6


def _fof_case(n=20000):
    box = 100.0 * (n / (1 << 20)) ** (1.0 / 3.0)
    pos, mass = syn.clustered_box(n, box, seed=81)
    return pos, mass, box, syn.linking_length(n, box)


def test_union_find_iteration_cap_runs_out_and_reports(gpu, port_built):
    lib = _capi.load()
    pos, mass, box, ll = _fof_case()
    t = KDTree(pos, None, mass, 16, kerntype=0, period=[box] * 3)
    try:
        _capi.check(lib.nbk_debug_set_iteration_cap(1))
        with pytest.raises(NbkError) as ei:
            t.FOF(ll, 20)
        assert ei.value.status == NBK_ERR_DEVICE
        assert "code 1" in str(ei.value)  # kErrIterCap
    finally:
        _capi.check(lib.nbk_debug_set_iteration_cap(0))
    # the context is still usable: the same tree, default cap, the oracle's partition
    g, ng = t.FOF(ll, 20)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, [box] * 3, backend="port")
    go, ngo = o.fof(ll, 20)
    o.close()
    t.close()
    assert ng == ngo
    assert_same_partition(g, go)


def _run_tree_life(pos, mass, box, ll):
    t = KDTree(pos, None, mass, 16, kerntype=0, period=[box] * 3)
    try:
        g, ng = t.FOF(ll, 20)
        rho = t.CalcDensity(16)
    finally:
        t.close()
    return g, ng, rho


def test_allocation_failure_at_every_point_is_clean(gpu, port_built):
    lib = _capi.load()
    pos, mass, box, ll = _fof_case(5000)
    g_ok, ng_ok, rho_ok = _run_tree_life(pos, mass, box, ll)  # warm-up: caches, modules
    base = lib.nbk_debug_live_allocations()
    failures = 0
    for countdown in range(200):
        _capi.check(lib.nbk_debug_fail_allocation(countdown))
        try:
            g, ng, rho = _run_tree_life(pos, mass, box, ll)
        except NbkError as e:
            assert e.status == NBK_ERR_NOMEM, e
            assert "injected failure" in str(e)
            failures += 1
            assert lib.nbk_debug_live_allocations() == base, f"leak after failure {countdown}"
            continue
        finally:
            _capi.check(lib.nbk_debug_fail_allocation(-1))
        # the countdown outlasted every allocation of the sequence: it ran to the end
        assert ng == ng_ok and np.array_equal(g, g_ok)
        assert_density_close(rho, rho_ok, "density after the injected failures")
        break
    else:
        raise AssertionError("the sequence never completed")
    assert failures >= 4  # creation, FOF and density allocate (kept scratch blocks do not)
    assert lib.nbk_debug_live_allocations() == base


def test_batch_allocation_failure_is_clean(gpu, port_built):
    lib = _capi.load()
    sizes = syn.group_sizes(200, 20, 2000, seed=82)
    gp, gv, gm, off = syn.plummer_groups(sizes, seed=82)

    def life():
        B = BatchedDensity(gp, gm, off, bucket_size=16)
        try:
            return B.density(32, use_graph=True)
        finally:
            B.close()

    want = life()
    base = lib.nbk_debug_live_allocations()
    for countdown in range(200):
        _capi.check(lib.nbk_debug_fail_allocation(countdown))
        try:
            rho = life()
        except NbkError as e:
            assert e.status == NBK_ERR_NOMEM, e
            assert lib.nbk_debug_live_allocations() == base, f"leak after failure {countdown}"
            continue
        finally:
            _capi.check(lib.nbk_debug_fail_allocation(-1))
        assert_density_close(rho, want, "batched density after the injected failures")
        break
    else:
        raise AssertionError("the sequence never completed")
    assert lib.nbk_debug_live_allocations() == base


def test_tree_gives_back_every_allocation(gpu):
    # a tree holds its arrays while it lives and gives every one back when destroyed (a
    # first build keeps this thread's build scratch block, so the count is taken after it)
    lib = _capi.load()
    pos, mass = syn.uniform_box(4096, 1.0, seed=83)
    KDTree(pos, None, mass, 16, kerntype=0).close()
    base = lib.nbk_debug_live_allocations()
    t = KDTree(pos, None, mass, 16, kerntype=0)
    assert lib.nbk_debug_live_allocations() > base
    t.close()
    assert lib.nbk_debug_live_allocations() == base
