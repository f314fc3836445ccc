"""GPU phase-space (TreeType TPHS) and velocity (TVEL) trees against the reference's outputs
in the phase_space golden fixture and against the C restatement on larger clustered sets.

Phase-space neighbour searches run the reference's own depth-first walk (the local-metric
search prunes with unscaled offsets, so its result depends on the walk), so neighbour IDs
and squared distances must match bit-exactly. Densities: 1e-12 relative (FP64 atomics and
a one-FMA kernel interpolation change the rounding of the sums). FOF partitions: identical
after relabelling by minimum member ID."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree
from nbodylib_gb300 import synthetic as syn
from nbodylib_gb300.kdtree import KSPH, TPHS, TVEL
from nbodylib_gb300._capi import NbkError
from tests.helpers import (assert_density_close, assert_knn_equal, assert_same_partition, golden,
                           rows_by_id, to_ids)

pytestmark = pytest.mark.gpu


def _gpu_tree(g, treetype, aniso, periodic, **kw):
    per = [float(g["box"])] * 3 if periodic else None
    return KDTree(g["pos"], g["vel"], g["mass"], int(g["b"]), treetype=treetype, kerntype=KSPH,
                  aniso=aniso, period=per, **kw)


def _ids_rows(t, nn, d2):
    perm = np.asarray(t.GetPerm())
    return rows_by_id(to_ids(nn, perm), perm), rows_by_id(np.asarray(d2), perm)


@pytest.mark.parametrize("aniso", [-1, 0])
@pytest.mark.parametrize("periodic", [False, True])
def test_phase_findnearest_vs_reference_golden(gpu, aniso, periodic):
    g = golden("phase_space")
    tag = ("plain" if aniso == -1 else "metric") + ("_per" if periodic else "")
    t = _gpu_tree(g, TPHS, aniso, periodic)
    assert t.GetNumNodes() == int(g["phs_num_nodes"])
    want_nn, want_d2 = g[f"phs_{tag}_nn"], g[f"phs_{tag}_d2"]
    k = want_nn.shape[1]
    nn, d2 = t.FindNearest(k)
    ids, dd = _ids_rows(t, nn, d2)
    assert_knn_equal(ids, dd, want_nn, want_d2, f"FindNearest TPHS aniso={aniso} {tag}")
    np.testing.assert_array_equal(dd, want_d2)  # ascending rows, as LoadNN fills them
    nn, d2 = t.FindNearestPoints(g["points6"], k)
    perm = np.asarray(t.GetPerm())
    assert_knn_equal(to_ids(nn, perm), d2, g[f"phs_{tag}_pt_nn"], g[f"phs_{tag}_pt_d2"],
                     f"FindNearest(x) TPHS aniso={aniso} {tag}")
    t.close()


@pytest.mark.parametrize("periodic", [False, True])
def test_phase_density_vs_reference_golden(gpu, periodic):
    g = golden("phase_space")
    tag = "metric" + ("_per" if periodic else "")
    t = _gpu_tree(g, TPHS, 0, periodic)
    assert_density_close(t.CalcDensity(16), g[f"phs_{tag}_rho"], "CalcDensity TPHS")
    perm = np.asarray(t.GetPerm())
    tree_of = np.empty_like(perm)
    tree_of[perm] = np.arange(len(perm))
    got = t.CalcDensityParticle(tree_of[g["ids"]].astype(np.int32), 16)
    assert_density_close(got, g[f"phs_{tag}_rho_id"], "CalcDensityParticle TPHS")
    t.close()


def test_velocity_tree_vs_reference_golden(gpu):
    g = golden("phase_space")
    t = _gpu_tree(g, TVEL, 0, False)
    assert t.GetNumNodes() == int(g["vel_num_nodes"])
    k = g["vel_nn"].shape[1]
    nn, d2 = t.FindNearest(k)
    ids, dd = _ids_rows(t, nn, d2)
    assert_knn_equal(ids, dd, g["vel_nn"], g["vel_d2"], "FindNearest TVEL")
    nn, d2 = t.FindNearestPoints(g["points3"], k)
    perm = np.asarray(t.GetPerm())
    assert_knn_equal(to_ids(nn, perm), d2, g["vel_pt_nn"], g["vel_pt_d2"], "FindNearest(x) TVEL")
    assert_density_close(t.CalcDensity(16), g["vel_rho"], "CalcDensity TVEL")
    t.close()


@pytest.mark.parametrize("cmp", [0, 1, 2])
@pytest.mark.parametrize("periodic", [False, True])
def test_phase_fof_criterion_vs_reference_golden(gpu, cmp, periodic):
    g = golden("phase_space")
    tag = "_per" if periodic else ""
    t = _gpu_tree(g, TPHS, 0, periodic)
    grp, ng = t.FOFCriterion(cmp, g[f"fof_params_{cmp}"], 8)
    assert ng == int(g[f"fof{tag}_{cmp}_ng"])
    assert_same_partition(grp, g[f"fof{tag}_{cmp}"], f"FOFCriterion TPHS cmp={cmp} {tag}")
    t.close()


@pytest.mark.parametrize("aniso", [-1, 0])
@pytest.mark.parametrize("periodic", [False, True])
def test_phase_vs_restatement_clustered(gpu, port_built, aniso, periodic):
    """20000 clustered particles, k = 32 (periodic: a heap of 33), against the C
    restatement; densities with the local metric."""
    box = 60.0
    pos, mass, vel = syn.clustered_box(20000, box, seed=53, velocities=True)
    per = [box] * 3 if periodic else None
    P = oracle.OracleTree(pos, vel, mass, 16, 3, 0, 1000, per, backend="port", nthreads=8,
                          aniso=aniso)
    t = KDTree(pos, vel, mass, 16, treetype=TPHS, kerntype=KSPH, aniso=aniso, period=per)
    k = 32
    want_nn, want_d2 = P.knn(k)
    nn, d2 = t.FindNearest(k)
    ids, dd = _ids_rows(t, nn, d2)
    assert_knn_equal(ids, dd, want_nn, want_d2, f"FindNearest TPHS aniso={aniso}")
    x = np.concatenate([pos[::97], vel[::97]], 1) + 0.01
    want_nn, want_d2 = P.knn_coord(x, k)
    nn, d2 = t.FindNearestPoints(x, k)
    assert_knn_equal(to_ids(nn, np.asarray(t.GetPerm())), d2, want_nn, want_d2,
                     f"FindNearest(x) TPHS aniso={aniso}")
    if aniso == 0:
        assert_density_close(t.CalcDensity(k), P.density(k), "CalcDensity TPHS")
    t.close()


def test_phase_device_arrays_and_targets(gpu, port_built):
    """Device-resident inputs and outputs; FindNearest for a target subset equals the
    corresponding rows of the all-particle call."""
    import torch
    pos, mass, vel = syn.clustered_box(5000, 30.0, seed=61, velocities=True)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    t = KDTree(dev(pos), dev(vel), dev(mass), 16, treetype=TPHS, kerntype=KSPH, device=True)
    nn, d2 = t.FindNearest(16)
    nn, d2 = nn.cpu().numpy(), d2.cpu().numpy()
    tgt = np.arange(0, 5000, 37).astype(np.int32)
    nt, dt = t.FindNearestTargets(dev(tgt), 16)
    np.testing.assert_array_equal(nt.cpu().numpy(), nn[tgt])
    np.testing.assert_array_equal(dt.cpu().numpy(), d2[tgt])
    P = oracle.OracleTree(pos, vel, mass, 16, 3, 0, 1000, None, backend="port", nthreads=8)
    assert_density_close(t.CalcDensity(24).cpu().numpy(), P.density(24), "CalcDensity TPHS dev")
    t.close()


def test_phase_and_velocity_trees_refuse_other_calls(gpu):
    pos, mass, vel = syn.clustered_box(600, 10.0, seed=7, velocities=True)
    t = KDTree(pos, vel, mass, 16, treetype=TPHS)
    with pytest.raises(NbkError):
        t.FOF(0.2, 5)
    with pytest.raises(NbkError):
        t.FindNearestPos(8)
    with pytest.raises(NbkError):
        t.CalcSmoothVel(16)
    t.close()
    t = KDTree(pos, vel, mass, 16, treetype=TPHS, aniso=-1)
    with pytest.raises(NbkError):
        t.CalcDensity(16)  # the reference reads uninitialised metric arrays here
    t.close()
    t = KDTree(pos, vel, mass, 16, treetype=TVEL)
    with pytest.raises(NbkError):
        t.FOFCriterion(1, [2, 1, 1, 0, 0, 0, 0.01], 5)
    t.close()
    with pytest.raises(NbkError):
        KDTree(pos, None, mass, 16, treetype=TPHS)  # velocities required
    with pytest.raises(NbkError):
        KDTree(pos, vel, mass, 16, treetype=TVEL, period=[10.0] * 3)
    with pytest.raises(NbkError):
        KDTree(pos, vel, mass, 16, treetype=TPHS, aniso=1)


@pytest.mark.parametrize("n,dup,per,k", [(12, 0, 5.0, 4), (12, 0, None, 4), (9, 0, 3.0, 3),
                                         (300, 40, 10.0, 8), (300, 40, None, 8)])
@pytest.mark.parametrize("aniso", [-1, 0])
def test_phase_edge_cases_vs_restatement(gpu, port_built, n, dup, per, k, aniso):
    """One-leaf trees (periodic ones search without images), fewer than 16 particles, exact
    duplicates (zero distances skipped by the target searches, zero metric offsets)."""
    from tests.test_oracle import _phase_edge_inputs
    pos, vel, m = _phase_edge_inputs(n, dup, per or 10.0)
    P = oracle.OracleTree(pos, vel, m, 16, 3, 0, 1000, per, backend="port", nthreads=2,
                          aniso=aniso)
    t = KDTree(pos, vel, m, 16, treetype=TPHS, kerntype=KSPH, aniso=aniso, period=per)
    want_nn, want_d2 = P.knn(k)
    nn, d2 = t.FindNearest(k)
    ids, dd = _ids_rows(t, nn, d2)
    assert_knn_equal(ids, dd, want_nn, want_d2, f"FindNearest n={n} dup={dup} per={per}",
                     dropped_nearest=per is not None)
    x = np.hstack([pos[:5], vel[:5]]) + 0.01
    want_nn, want_d2 = P.knn_coord(x, k)
    nn, d2 = t.FindNearestPoints(x, k)
    assert_knn_equal(to_ids(nn, np.asarray(t.GetPerm())), d2, want_nn, want_d2,
                     f"FindNearest(x) n={n}")
    if aniso == 0:
        assert_density_close(t.CalcDensity(k), P.density(k), f"CalcDensity n={n}")
    t.close()


def test_phase_too_few_particles_for_the_metric(gpu):
    rng = np.random.default_rng(1)
    pos, vel, m = rng.random((7, 3)), rng.random((7, 3)), np.ones(7)
    t = KDTree(pos, vel, m, 16, treetype=TPHS)
    with pytest.raises(NbkError):
        t.FindNearest(3)  # the metric spacing needs 8 particles (the reference exits)
    t.close()


@pytest.mark.parametrize("periodic", [False, True])
def test_findnearestphase_and_vel_variants_vs_reference_golden(gpu, periodic):
    """KDTree::FindNearestPhase on a tree built with the local metric (Aniso 0) searches
    with the plain phase distance, so it returns the reference's plain results; and
    FindNearestVel on a velocity tree is its FindNearest."""
    g = golden("phase_space")
    tag = "plain" + ("_per" if periodic else "")
    t = _gpu_tree(g, TPHS, 0, periodic)
    k = g[f"phs_{tag}_nn"].shape[1]
    nn, d2 = t.FindNearestPhase(k)
    ids, dd = _ids_rows(t, nn, d2)
    assert_knn_equal(ids, dd, g[f"phs_{tag}_nn"], g[f"phs_{tag}_d2"], f"FindNearestPhase {tag}")
    nn, d2 = t.FindNearestPhasePoints(g["points6"], k)
    assert_knn_equal(to_ids(nn, np.asarray(t.GetPerm())), d2, g[f"phs_{tag}_pt_nn"],
                     g[f"phs_{tag}_pt_d2"], f"FindNearestPhase(x, v) {tag}")
    with pytest.raises(NbkError):
        t.FindNearestVel(k)
    t.close()
    if not periodic:
        tv = _gpu_tree(g, TVEL, 0, False)
        nn, d2 = tv.FindNearestVel(int(g["vel_nn"].shape[1]))
        ids, dd = _ids_rows(tv, nn, d2)
        assert_knn_equal(ids, dd, g["vel_nn"], g["vel_d2"], "FindNearestVel")
        with pytest.raises(NbkError):
            tv.FindNearestPhase(4)
        tv.close()
