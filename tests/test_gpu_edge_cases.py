"""Edge cases of the boundary on the GPU: empty and non-finite inputs are refused with a
status (the reference would build on garbage or exit), a one-particle tree, the largest
supported neighbour count with and without periods, and batches whose groups hold one
particle."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import BatchedDensity, KDTree
from nbodylib_gb300 import synthetic as syn
from nbodylib_gb300._capi import NbkError
from nbodylib_gb300.kdtree import KSPH
from tests.helpers import assert_density_close, assert_knn_equal, rows_by_id, to_ids

pytestmark = pytest.mark.gpu


def test_create_refuses_empty_and_non_finite(gpu):
    with pytest.raises(NbkError):
        KDTree(np.zeros((0, 3)), None, None, 16)
    for bad in (np.nan, np.inf, -np.inf):
        pos = np.random.default_rng(1).random((100, 3))
        pos[37, 1] = bad
        with pytest.raises(NbkError):
            KDTree(pos, None, None, 16)


def test_one_particle_tree(gpu, port_built):
    pos = np.array([[0.5, 0.25, 0.75]])
    t = KDTree(pos, None, None, 16, kerntype=KSPH, period=[1.0] * 3)
    assert t.GetNumNodes() == 1 and t.GetNumLeafNodes() == 1
    g, ng = t.FOF(0.1, 2)
    assert ng == 0 and np.asarray(g).tolist() == [0]
    nn, d2 = t.FindNearest(1)  # no neighbour exists: the reference's empty heap slot
    o = oracle.OracleTree(pos, None, None, 16, 0, 0, 1000, [1.0] * 3, backend="port")
    onn, od2 = o.knn(1)
    np.testing.assert_array_equal(np.asarray(nn), onn)
    np.testing.assert_array_equal(np.asarray(d2), od2)
    with pytest.raises(NbkError):
        t.CalcDensity(1)  # the reference exits: fewer than k neighbours
    t.close()


@pytest.mark.parametrize("periodic", [False, True])
def test_largest_k(gpu, port_built, periodic):
    """k = 127 (a heap of 128 when periodic), the largest the kernels take; one more with
    a period is refused."""
    pos, mass = syn.uniform_box(3000, 1.0, seed=9)
    per = [1.0] * 3 if periodic else None
    t = KDTree(pos, None, mass, 16, kerntype=KSPH, period=per)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, per, backend="port", nthreads=8)
    nn, d2 = t.FindNearest(127)
    perm = np.asarray(t.GetPerm())
    want_nn, want_d2 = o.knn(127)
    assert_knn_equal(rows_by_id(to_ids(np.asarray(nn), perm), perm), rows_by_id(np.asarray(d2), perm),
                     want_nn, want_d2, f"FindNearest(127) periodic={periodic}")
    if periodic:
        with pytest.raises(NbkError):
            t.FindNearest(128)
    t.close()


def test_batch_with_one_particle_groups(gpu, port_built):
    """Groups of one particle have no neighbour: their density stays 0 (CalcDensity(0) has
    no defined result in the reference); every other group is checked as usual."""
    sizes = np.array([1, 40, 1, 2, 300, 1, 25])
    pos, vel, mass, off = syn.plummer_groups(sizes, seed=5)
    B = BatchedDensity(pos, mass, off, bucket_size=16)
    rho = np.asarray(B.density(32, use_graph=False))
    B.close()
    for g in range(len(sizes)):
        s, e = off[g], off[g + 1]
        if e - s == 1:
            assert rho[s] == 0.0
            continue
        t = oracle.OracleTree(pos[s:e], None, mass[s:e], 16, 0, 0, 1000, None, backend="port")
        assert_density_close(rho[s:e], t.density(min(32, e - s - 1)), f"group {g}")


def test_degenerate_parameters(gpu, port_built):
    """ll = 0 links nothing (the test is strict), minnum above n leaves no group, a ball of
    radius 0 is empty, and k = n - 1 (every other particle of a 100-particle tree) matches
    the restatement."""
    pos, mass = syn.uniform_box(600, 1.0, seed=12)
    t = KDTree(pos, None, mass, 8, kerntype=KSPH)
    o = oracle.OracleTree(pos, None, mass, 8, 0, 0, 1000, None, backend="port")
    g, ng = t.FOF(0.0, 2)
    assert ng == 0 and not np.any(np.asarray(g))
    g, ng = t.FOF(0.3, 601)
    assert ng == 0 and not np.any(np.asarray(g))
    off, out = t.SearchBallPosTagged(np.arange(600, dtype=np.int32), 0.0)
    assert int(np.asarray(off)[-1]) == 0
    t.close()
    small, ms = syn.uniform_box(100, 1.0, seed=14)
    t = KDTree(small, None, ms, 8, kerntype=KSPH)
    o = oracle.OracleTree(small, None, ms, 8, 0, 0, 1000, None, backend="port")
    assert_density_close(t.CalcDensity(99), o.density(99), "k = n - 1")
    t.close()


def test_exact_duplicates(gpu, port_built):
    """Coincident particles: the non-periodic target search skips zero distances (the
    reference's FindNearest(tt), KDLeafNode.cxx:19-21), so a duplicate is never its twin's
    neighbour; FOF links duplicates (distance 0 < ll)."""
    base, _ = syn.uniform_box(500, 1.0, seed=13)
    pos = np.concatenate([base, base[:100]])
    mass = np.full(len(pos), 1.0 / len(pos))
    t = KDTree(pos, None, mass, 16, kerntype=KSPH)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, None, backend="port")
    nn, d2 = t.FindNearest(8)
    perm = np.asarray(t.GetPerm())
    want_nn, want_d2 = o.knn(8)
    assert_knn_equal(rows_by_id(to_ids(np.asarray(nn), perm), perm), rows_by_id(np.asarray(d2), perm),
                     want_nn, want_d2, "duplicates")
    assert np.all(np.asarray(d2) > 0)
    g, ng = t.FOF(1e-6, 2)
    go, no = o.fof(1e-6, 2)
    assert ng == no == 100
    t.close()
