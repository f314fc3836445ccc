"""GPU parity: kNN (FindNearest / FindNearestPos, periodic and not) against the
reference's golden outputs, the oracle restatement and brute force."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import PERIODIC_MIN_IMAGE, KDTree
from nbodylib_gb300 import synthetic as syn
from tests.helpers import (assert_knn_equal, brute_min_image_knn, golden, rows_by_id, to_ids)

pytestmark = pytest.mark.gpu


def gpu_knn_ids(t, k, method=0, mode=0):
    nn, d2 = (t.FindNearest if method == 0 else t.FindNearestPos)(k, periodic_mode=mode)
    perm = t.GetPerm()
    return rows_by_id(to_ids(nn, perm), perm), rows_by_id(d2, perm)


def test_golden_nonperiodic(gpu):
    g = golden("nonperiodic")
    t = KDTree(g["pos"], None, g["mass"], int(g["b"]), kerntype=int(g["kerntype"]))
    ids, d2 = gpu_knn_ids(t, int(g["k"]))
    assert assert_knn_equal(ids, d2, g["nn_findnearest"], g["d2_findnearest"]) == 0
    nn, dd = t.FindNearestPosPoints(g["points"], 12)
    assert_knn_equal(to_ids(nn, t.GetPerm()), dd, g["knn_points_nn"], g["knn_points_d2"])


@pytest.mark.parametrize("method,key", [(0, "findnearest"), (1, "findnearestpos")])
def test_golden_uniform_periodic_reference_gates(gpu, method, key):
    g = golden("uniform_periodic")
    t = KDTree(g["pos"], None, g["mass"], int(g["b"]), kerntype=0, period=g["period"])
    ids, d2 = gpu_knn_ids(t, int(g["k"]), method)
    assert_knn_equal(ids, d2, g["nn_" + key], g["d2_" + key], key)


@pytest.mark.parametrize("method,key", [(0, "findnearest"), (1, "findnearestpos")])
def test_golden_tiny_periodic_single_leaf(gpu, method, key):
    g = golden("tiny_periodic")
    t = KDTree(g["pos"], None, g["mass"], 16, kerntype=0, period=g["period"])
    ids, d2 = gpu_knn_ids(t, int(g["k"]), method)
    assert_knn_equal(ids, d2, g["nn_" + key], g["d2_" + key], key)


def test_uniform_32768_periodic_k32_vs_oracle(gpu, port_built):
    """The plain-method workload: 32768 uniform particles, periodic unit box, b=16, k=32."""
    pos, mass = syn.uniform_box(32768, 1.0, seed=1)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, [1, 1, 1], backend="port", nthreads=8)
    t = KDTree(pos, None, mass, 16, kerntype=0, period=[1, 1, 1])
    for m in (0, 1):
        ids, d2 = gpu_knn_ids(t, 32, m)
        oi, od = o.knn(32, m)
        assert_knn_equal(ids, d2, oi, od, f"method {m}")


def test_min_image_mode_vs_brute_force(gpu):
    pos, mass = syn.uniform_box(4096, 1.0, seed=21)
    t = KDTree(pos, None, mass, 16, kerntype=0, period=[1, 1, 1])
    ids, d2 = gpu_knn_ids(t, 32, 0, PERIODIC_MIN_IMAGE)
    bid, bd2 = brute_min_image_knn(pos, [1, 1, 1], 32)
    assert_knn_equal(ids, d2, bid, bd2, "min image")


@pytest.mark.parametrize("b", [1, 5, 16, 40])
def test_clustered_nonperiodic_vs_oracle(gpu, port_built, b):
    pos, mass = syn.clustered_box(1 << 15, 100.0, seed=31)
    o = oracle.OracleTree(pos, None, mass, b, 0, 0, 1000, None, backend="port", nthreads=8)
    t = KDTree(pos, None, mass, b, kerntype=0)
    ids, d2 = gpu_knn_ids(t, 64)
    oi, od = o.knn(64, 0)
    assert_knn_equal(ids, d2, oi, od, f"b={b}")


def test_points_periodic_vs_oracle(gpu, port_built):
    pos, mass = syn.clustered_box(50000, 100.0, seed=32)
    x = np.random.default_rng(33).random((5000, 3)) * 100.0
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, [100.0] * 3, backend="port", nthreads=8)
    t = KDTree(pos, None, mass, 16, kerntype=0, period=[100.0] * 3)
    nn, d2 = t.FindNearestPosPoints(x, 20)
    oi, od = o.knn_pos(x, 20)
    assert_knn_equal(to_ids(nn, t.GetPerm()), d2, oi, od, "points")


def test_duplicates_and_too_few(gpu):
    """Coincident particles are excluded by the target search (KDLeafNode.cxx:19-21); a
    k larger than the other particles leaves -1 slots (the reference prints a warning)."""
    pos = np.repeat(np.random.default_rng(3).random((50, 3)), 2, axis=0)
    t = KDTree(pos, None, None, 4, kerntype=0)
    o = oracle.OracleTree(pos, None, None, 4, 0, 0, 1000, None, backend="port")
    ids, d2 = gpu_knn_ids(t, 8)
    oi, od = o.knn(8, 0)
    assert_knn_equal(ids, d2, oi, od, "duplicates")
    small = KDTree(pos[:6], None, None, 16, kerntype=0)
    nn, dd = small.FindNearest(8)
    assert (nn == -1).sum() > 0 and np.all(dd[nn == -1] == 1e32)
