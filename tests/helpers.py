"""Shared checks for the parity tests."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DENSITY_RTOL = 1e-12  # relative density tolerance stated by the benchmark spec


def golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def to_ids(nn_tree, perm):
    """Tree-index neighbour lists -> input-order IDs (-1 kept)."""
    nn_tree = np.asarray(nn_tree)
    out = np.where(nn_tree >= 0, perm[np.clip(nn_tree, 0, None)], -1)
    return out


def rows_by_id(arr_rows_tree, perm):
    """Reorder rows indexed by tree index into rows indexed by ID."""
    out = np.empty_like(arr_rows_tree)
    out[perm] = arr_rows_tree
    return out


def assert_knn_equal(ids_a, d2_a, ids_b, d2_b, what="", dropped_nearest=False):
    """Neighbour lists must agree bit-exactly: per row, the sorted squared distances are
    identical and the ID sets are identical. Where two candidates tie exactly in d2 at
    the k-th place the reference's pick depends on traversal order; such rows are only
    required to agree on d2 and are counted (expected: none on continuous data). With
    dropped_nearest (periodic FindNearest, whose heap of k+1 drops its nearest entry),
    ties at the row's smallest distance are allowed as well: which of two exact
    duplicates is dropped depends on the heap's order of equal keys."""
    ids_a, ids_b = np.asarray(ids_a), np.asarray(ids_b)
    d2_a, d2_b = np.asarray(d2_a), np.asarray(d2_b)
    assert ids_a.shape == ids_b.shape, (ids_a.shape, ids_b.shape)
    sa = np.sort(d2_a, axis=1)
    sb = np.sort(d2_b, axis=1)
    bad_d2 = np.nonzero(np.any(sa != sb, axis=1))[0]
    assert bad_d2.size == 0, f"{what}: {bad_d2.size} rows differ in d2, e.g. row {bad_d2[:5]}"
    ia = np.sort(ids_a, axis=1)
    ib = np.sort(ids_b, axis=1)
    diff = np.nonzero(np.any(ia != ib, axis=1))[0]
    ties = 0
    for r in diff:
        # allowed only for candidates tied exactly at the k-th (largest) distance
        da = dict(zip(ids_a[r].tolist(), d2_a[r].tolist()))
        db = dict(zip(ids_b[r].tolist(), d2_b[r].tolist()))
        only = set(da) ^ set(db)
        kth = sa[r, -1]
        ok = (kth,) + ((sa[r, 0],) if dropped_nearest else ())
        if all(da.get(i, db.get(i)) in ok for i in only):
            ties += 1
            continue
        raise AssertionError(f"{what}: row {r} neighbour sets differ: {sorted(only)}")
    return ties


def canonical_groups(group, ids=None):
    """Relabel each group by its minimum member ID (0 stays 0)."""
    group = np.asarray(group)
    n = group.size
    ids = np.arange(n) if ids is None else ids
    out = np.zeros(n, np.int64)
    lab = group > 0
    if lab.any():
        g = group[lab]
        order = np.argsort(g, kind="stable")
        gs = g[order]
        idx = ids[lab][order]
        starts = np.r_[0, np.nonzero(np.diff(gs))[0] + 1]
        mins = np.minimum.reduceat(idx, starts)
        lut = dict(zip(gs[starts], mins + 1))
        out[lab] = np.array([lut[v] for v in g])
    return out


def assert_same_partition(ga, gb, what=""):
    ca, cb = canonical_groups(ga), canonical_groups(gb)
    bad = np.nonzero(ca != cb)[0]
    assert bad.size == 0, f"{what}: {bad.size} particles in different groups, e.g. {bad[:10]}"


def assert_density_close(a, b, what="", rtol=DENSITY_RTOL):
    a, b = np.asarray(a), np.asarray(b)
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    worst = float(rel.max()) if rel.size else 0.0
    assert worst <= rtol, f"{what}: max relative error {worst:.3e} > {rtol:.0e}"
    return worst


def reflect_images(x, period):
    """The reference's 8 query positions: direct + one-sided mirrors (DistFunc.h:326-355),
    in the search order x, y, z, xy, xz, yz, xyz. Returns (8, nq, 3)."""
    x = np.asarray(x, np.float64)
    p = np.asarray(period, np.float64)
    masks = [0, 1, 2, 4, 3, 5, 6, 7]
    out = np.empty((8,) + x.shape)
    for m_i, m in enumerate(masks):
        xp = x.copy()
        for k in range(3):
            if m >> k & 1:
                low = x[:, k] < p[k] / 2.0
                xp[:, k] = np.where(low, x[:, k] + p[k], x[:, k] - p[k])
        out[m_i] = xp
    return out


def d2_ref(a, b):
    """((dx*dx + dy*dy) + dz*dz) with separately rounded numpy ops."""
    dx = a[..., 0] - b[..., 0]
    dy = a[..., 1] - b[..., 1]
    dz = a[..., 2] - b[..., 2]
    return (dx * dx + dy * dy) + dz * dz


def brute_min_image_knn(pos, period, k, drop_self=True, chunk=256):
    """Exact minimum-image kNN by brute force: per pair the minimum over the reference's
    image positions. Returns IDs and d2 (ascending)."""
    n = pos.shape[0]
    imgs = reflect_images(pos, period)
    ids = np.empty((n, k), np.int64)
    dd = np.empty((n, k))
    for s in range(0, n, chunk):
        q = imgs[:, s:s + chunk]  # (8, c, 3)
        d = np.min(d2_ref(q[:, :, None, :], pos[None, None, :, :]), axis=0)  # (c, n)
        if drop_self:
            d[np.arange(d.shape[0]), np.arange(s, s + d.shape[0])] = np.inf
        part = np.argpartition(d, k - 1, axis=1)[:, :k]
        pd = np.take_along_axis(d, part, axis=1)
        o = np.argsort(pd, axis=1, kind="stable")
        ids[s:s + chunk] = np.take_along_axis(part, o, axis=1)
        dd[s:s + chunk] = np.take_along_axis(pd, o, axis=1)
    return ids, dd
