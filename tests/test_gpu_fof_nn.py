"""GPU FOFNNCriterion / FOFNNDistCriterion (KDFOF.cxx:380-640): friends-of-friends over the
tree's own FindNearest lists, against the C restatement (pinned to the reference on the
CPU). Partitions must be identical after relabelling by minimum member ID; groups are
numbered by decreasing size (among equal sizes the reference's order follows its heap,
so only the size order is asserted)."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree
from nbodylib_gb300 import synthetic as syn
from nbodylib_gb300.kdtree import KSPH
from tests.helpers import assert_same_partition

pytestmark = pytest.mark.gpu

PARAMS = {0: [0, 0, 0, 0, 0, 0, 0.35, 0],      # FOF3d: linked when |dx|^2 < params[6]
          1: [0, 0, 0, 0, 0, 0, 0.02, 0],      # FOFVel: |dv|^2 < params[6]
          2: [0, 0, 0, 0, 0, 0, 0.6, 0.05]}    # FOF6d: |dx|^2/p6 + |dv|^2/p7 < 1


def sizes_non_increasing(g):
    s = np.bincount(g)[1:]
    return s.size == 0 or bool(np.all(np.diff(s) <= 0))


@pytest.mark.parametrize("cmp", [0, 1, 2])
@pytest.mark.parametrize("dist_form", [False, True])
def test_fof_nn_vs_restatement(gpu, port_built, cmp, dist_form):
    pos, mass, vel = syn.clustered_box(30000, 100.0, seed=60 + cmp, velocities=True)
    t = KDTree(pos, vel, mass, 16, kerntype=KSPH)
    nn, d2 = t.FindNearest(16)  # tree indices, rows by tree index
    P = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port", nthreads=8)
    pn, pd = P.tree_knn(16)
    params = PARAMS[cmp]
    if dist_form:
        # params[6] per target from its lists, as a distfunc(numNN, dist2) would give it
        g, ng = t.FOFNNDistCriterion(cmp, params, nn, np.max(d2, 1) * 0.05, [6], 5)
        gp, ngp = P.fof_nn(cmp, params, pn, 5, values=np.max(pd, 1) * 0.05, pidx=[6])
    else:
        g, ng = t.FOFNNCriterion(cmp, params, nn, 5)
        gp, ngp = P.fof_nn(cmp, params, pn, 5)
    assert ng == ngp and ng >= (1 if dist_form else 4), (ng, ngp)
    assert_same_partition(np.asarray(g), gp, f"FOFNN cmp={cmp} dist={dist_form}")
    assert sizes_non_increasing(np.asarray(g))
    t.close()


def test_fof_nn_device_lists_and_bad_index(gpu):
    import torch
    pos, mass, vel = syn.clustered_box(5000, 40.0, seed=66, velocities=True)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    t = KDTree(dev(pos), dev(vel), dev(mass), 16, kerntype=KSPH, device=True)
    nn, d2 = t.FindNearest(8)
    g, ng = t.FOFNNCriterion(0, PARAMS[0], nn, 3)
    th = KDTree(pos, vel, mass, 16, kerntype=KSPH)
    nnh, _ = th.FindNearest(8)
    gh, ngh = th.FOFNNCriterion(0, PARAMS[0], nnh, 3)
    assert ng == ngh
    assert_same_partition(g.cpu().numpy(), gh, "device vs host lists")
    bad = nnh.copy()
    bad[3, 2] = len(mass) + 7  # an index outside the tree is reported, not read
    from nbodylib_gb300._capi import NbkError
    with pytest.raises(NbkError):
        th.FOFNNCriterion(0, PARAMS[0], bad, 3)
    t.close()
    th.close()
