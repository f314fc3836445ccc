"""Periodic boxes with a different period per dimension (the reference takes period[3]):
FindNearest and FindNearestPos with the reference's image gates, the minimum-image mode
against brute force, CalcDensity (which ignores the period), FOF and
SearchBallPosTagged, on the GPU against the restatement. Particles crowd the faces so
that every image pass has work."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import PERIODIC_MIN_IMAGE, KDTree
from tests.helpers import (assert_density_close, assert_knn_equal, assert_same_partition,
                           brute_min_image_knn, rows_by_id, to_ids)

pytestmark = pytest.mark.gpu

PERIOD = [100.0, 60.0, 35.0]


def box_particles(n, seed):
    rng = np.random.default_rng(seed)
    per = np.asarray(PERIOD)
    pos = rng.random((n, 3)) * per
    # a third of the particles within 2% of a face
    m = n // 3
    face = rng.integers(0, 3, m)
    side = rng.integers(0, 2, m)
    depth = rng.random(m) * 0.02
    pos[np.arange(m), face] = np.where(side == 1, per[face] * (1 - depth), per[face] * depth)
    return pos, np.full(n, 1.0 / n)


def test_noncubic_knn_density_fof_ball(gpu, port_built):
    n = 30000
    pos, mass = box_particles(n, 41)
    t = KDTree(pos, None, mass, 16, kerntype=0, period=PERIOD)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, PERIOD, backend="port", nthreads=8)
    perm = np.asarray(t.GetPerm())
    for m in (0, 1):
        nn, d2 = (t.FindNearest if m == 0 else t.FindNearestPos)(16)
        oi, od = o.knn(16, m)
        assert_knn_equal(rows_by_id(to_ids(nn, perm), perm), rows_by_id(d2, perm), oi, od,
                         f"non-cubic method {m}", dropped_nearest=(m == 0))
    assert_density_close(t.CalcDensity(24), o.density(24), "non-cubic CalcDensity")
    ll = 0.2 * (np.prod(PERIOD) / n) ** (1.0 / 3.0)
    g, ng = t.FOF(ll, 5)
    go, no = o.fof(ll, 5)
    assert ng == no
    assert_same_partition(np.asarray(g), go, "non-cubic FOF")
    inv = np.argsort(perm)
    ids = np.random.default_rng(42).choice(n, 300, replace=False)
    r2 = 9.0
    off, out = t.SearchBallPosTagged(inv[ids], r2)
    for j, i in enumerate(ids):
        np.testing.assert_array_equal(np.sort(perm[out[off[j]:off[j + 1]]]),
                                      o.ball_tagged(int(i), r2))
    t.close()


def test_noncubic_min_image_vs_brute_force(gpu):
    pos, mass = box_particles(3000, 43)
    t = KDTree(pos, None, mass, 16, kerntype=0, period=PERIOD)
    nn, d2 = t.FindNearest(24, periodic_mode=PERIODIC_MIN_IMAGE)
    perm = np.asarray(t.GetPerm())
    bid, bd2 = brute_min_image_knn(pos, PERIOD, 24)
    assert_knn_equal(rows_by_id(to_ids(nn, perm), perm), rows_by_id(d2, perm), bid, bd2,
                     "non-cubic minimum image")
    t.close()
