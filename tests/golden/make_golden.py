"""Generate the golden fixtures from the reference NBodylib KDTree itself.

Runs only where the reference checkout exists (it compiles oracle/_ref/libnbref.so from
the reference's own sources). Each fixture stores the seeded inputs together with the
reference's outputs, so the tests never need the reference at run time:

    python tests/golden/make_golden.py

Outputs are in input order ("ID"); neighbour lists hold IDs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

import oracle  # noqa: E402
from nbodylib_gb300 import synthetic as syn  # noqa: E402


def ref_tree(pos, vel, mass, b, kerntype, period):
    return oracle.OracleTree(pos, vel, mass, b, 0, kerntype, 1000, period, backend="ref",
                             nthreads=4)


def uniform_periodic():
    n = 1500
    pos, mass = syn.uniform_box(n, 1.0, seed=11)
    t = ref_tree(pos, None, mass, 16, 0, [1.0, 1.0, 1.0])
    nn_fn, d2_fn = t.knn(16, method=0)
    nn_fp, d2_fp = t.knn(16, method=1)
    rho = t.density(32)
    t2 = ref_tree(pos, None, mass, 16, 0, [1.0, 1.0, 1.0])
    ll = syn.linking_length(n, 1.0, 0.5)
    grp, ng = t2.fof(ll, 5, 0)
    return dict(pos=pos, mass=mass, period=np.ones(3), b=16, kerntype=0, k=16,
                nn_findnearest=nn_fn, d2_findnearest=d2_fn, nn_findnearestpos=nn_fp,
                d2_findnearestpos=d2_fp, k_density=32, rho=rho, ll=ll, fof_minnum=5,
                fof_group=grp, fof_ngroup=ng, num_nodes=t.num_nodes, num_leaves=t.num_leaves,
                leaf_start_ids=_leaf_sets(t))


def _leaf_sets(t):
    """Leaf membership as a label per ID: the smallest ID in the same leaf."""
    ids = t.ids()
    ls = t.leaf_start()
    lab = np.empty(len(ids), np.int64)
    for s in np.unique(ls):
        members = ids[ls == s]
        lab[members] = members.min()
    return lab


def clustered():
    n = 6000
    box = 100.0
    pos, mass, vel = syn.clustered_box(n, box, seed=12, velocities=True)
    per = [box] * 3
    rng = np.random.default_rng(13)
    ids = rng.choice(n, 40, replace=False).astype(np.int32)
    out = dict(pos=pos, mass=mass, vel=vel, period=np.full(3, box), b=16, kerntype=0)
    t = ref_tree(pos, vel, mass, 16, 0, per)
    out["num_nodes"] = t.num_nodes
    out["num_leaves"] = t.num_leaves
    out["leaf_start_ids"] = _leaf_sets(t)
    out["k"] = 32
    out["rho"] = t.density(32)
    out["veldens_32_32"] = ref_tree(pos, vel, mass, 16, 0, per).veldensity(32, 32)
    out["veldens_16_32"] = ref_tree(pos, vel, mass, 16, 0, per).veldensity(16, 32)
    t3 = ref_tree(pos, vel, mass, 16, 0, per)
    out["query_ids"] = ids
    out["dens_particle"] = np.array([t3.density_particle(i, 32) for i in ids])
    out["veldens_particle"] = np.array([t3.veldensity_particle(i, 16, 32) for i in ids])
    ll = syn.linking_length(n, box)
    out["ll"] = ll
    g, ng = ref_tree(pos, vel, mass, 16, 0, per).fof(ll, 10, 0)
    out["fof_group"], out["fof_ngroup"] = g, ng
    g, ng = ref_tree(pos, vel, mass, 16, 0, per).fof(ll, 10, 1)
    out["fof_group_ordered"], out["fof_ngroup_ordered"] = g, ng
    r2 = (3 * ll) ** 2
    out["ball_r2"] = r2
    tb = ref_tree(pos, vel, mass, 16, 0, per)
    lists = [tb.ball_tagged(int(i), r2) for i in ids]
    out["ball_offsets"] = np.concatenate([[0], np.cumsum([len(x) for x in lists])]).astype(np.int64)
    out["ball_ids"] = np.concatenate(lists).astype(np.int32)
    return out


def nonperiodic():
    n = 700
    pos, mass = syn.uniform_box(n, 2.0, seed=14)
    rng = np.random.default_rng(15)
    t = ref_tree(pos, None, mass, 8, 2, None)  # Epanechnikov, the constructor default
    nn, d2 = t.knn(20, method=0)
    rho = ref_tree(pos, None, mass, 8, 2, None).density(20)
    ids = rng.choice(n, 25, replace=False).astype(np.int32)
    r2 = 0.35 ** 2
    tb = ref_tree(pos, None, mass, 8, 2, None)
    lists = [tb.ball_tagged(int(i), r2) for i in ids]
    marks = []
    for i in ids[:10]:
        m, d = tb.ball_mark(int(i), r2, imark=7)
        marks.append(np.where(m == 7, d, -1.0))
    x = rng.random((30, 3)) * 2.0
    nnx, d2x = tb.knn_pos(x, 12)
    return dict(pos=pos, mass=mass, b=8, kerntype=2, k=20, nn_findnearest=nn, d2_findnearest=d2,
                rho=rho, num_nodes=t.num_nodes, num_leaves=t.num_leaves,
                leaf_start_ids=_leaf_sets(t), query_ids=ids, ball_r2=r2,
                ball_offsets=np.concatenate([[0], np.cumsum([len(v) for v in lists])]).astype(np.int64),
                ball_ids=np.concatenate(lists).astype(np.int32),
                mark_d2=np.array(marks), points=x, knn_points_nn=nnx, knn_points_d2=d2x)


def tiny_periodic():
    """n <= b: the reference's periodic searches fall back to the non-periodic target
    search (KDLeafNode.cxx:658-661)."""
    n = 10
    pos, mass = syn.uniform_box(n, 1.0, seed=16)
    t = ref_tree(pos, None, mass, 16, 0, [1.0, 1.0, 1.0])
    nn, d2 = t.knn(5, method=0)
    nnp, d2p = t.knn(5, method=1)
    return dict(pos=pos, mass=mass, period=np.ones(3), b=16, k=5, nn_findnearest=nn,
                d2_findnearest=d2, nn_findnearestpos=nnp, d2_findnearestpos=d2p)


def smoothing():
    """The SPH smoothing family (KDCalcSmoothQuantities.cxx) on clustered particles with
    velocities, densities computed by the reference (densityset != 1), k = 24; the
    Particle forms for a few particles (stored by ID) and the Position forms at a few
    points; CalcVelDensityWithPhysDensity on widely spaced particles (every neighbour
    distance above 1, where the reference stays inside its kernel table)."""
    pos, mass, vel = syn.clustered_box(2500, 50.0, seed=21, velocities=True)
    t = ref_tree(pos, vel, mass, 16, 0, None)
    k = 24
    rho = t.density(k)
    sv = t.smooth_vel_moments(0, k, None)
    dp = t.smooth_vel_moments(1, k, None, sv).reshape(-1, 9)
    skew = t.smooth_vel_moments(2, k, None, sv, dp)
    kurt = t.smooth_vel_moments(3, k, None, sv, dp)
    rng = np.random.default_rng(22)
    weight = rng.random(len(mass))
    ids = np.array([0, 5, 911, 1700, len(mass) - 1], np.int32)
    pts = pos[ids] + rng.normal(scale=0.05, size=(len(ids), 3))
    one = {}
    for tag, kw in (("id", [dict(pid=int(i)) for i in ids]), ("pt", [dict(x=x) for x in pts])):
        one[f"vel_{tag}"] = np.array([t.smooth_one(0, k, rho=None, **a) for a in kw])
        one[f"veldisp_{tag}"] = np.array([t.smooth_one(1, k, rho=None, smvel=sv[j], **a)
                                          for j, a in zip(ids, kw)])
        one[f"mean_{tag}"] = np.array([t.smooth_one(4, k, rho=None, weight=weight, **a)
                                       for a in kw])
        one[f"disp_{tag}"] = np.array([t.smooth_one(5, k, rho=None, weight=weight, mean=0.4, **a)
                                       for a in kw])
    prng = np.random.default_rng(23)
    ppos = prng.random((3000, 3)) * 200.0
    pvel = prng.normal(size=(3000, 3))
    pmass = prng.random(3000) + 0.5
    tp = ref_tree(ppos, pvel, pmass, 16, 0, None)
    vphys = tp.veldensity_phys(16, 32, None)
    vphys_id = np.array([tp.veldensity_phys_particle(int(i), 16, 32, None) for i in ids])
    return dict(pos=pos, vel=vel, mass=mass, b=16, k=k, rho=rho, smvel=sv, veldisp=dp,
                velskew=skew, velkurt=kurt, weight=weight, ids=ids, points=pts, mean_ref=0.4,
                phys_pos=ppos, phys_vel=pvel, phys_mass=pmass, phys_nsmooth=16,
                phys_nsearch=32, veldensity_phys=vphys, veldensity_phys_id=vphys_id, **one)


def position_density():
    """CalcDensityPosition and CalcVelDensityPosition (KDCalcSmoothQuantities.cxx:
    1092-1207) on a periodic physical tree of clustered particles (both forms ignore the
    period): at particle positions, random points in the box and points outside it, with
    random velocities."""
    pos, mass, vel = syn.clustered_box(3000, 40.0, seed=31, velocities=True)
    per = [40.0] * 3
    t = ref_tree(pos, vel, mass, 16, 0, per)
    rng = np.random.default_rng(32)
    pts = np.concatenate([pos[:10], rng.random((30, 3)) * 40.0,
                          rng.random((5, 3)) * 10.0 + 45.0])
    pv = rng.normal(size=(len(pts), 3))
    return dict(pos=pos, vel=vel, mass=mass, period=np.asarray(per), b=16, points=pts,
                point_vel=pv,
                dens_k32=np.array([t.density_position(x, 32) for x in pts]),
                dens_k8=np.array([t.density_position(x, 8) for x in pts]),
                veldens_16_32=np.array([t.veldensity_position(x, v, 16, 32)
                                        for x, v in zip(pts, pv)]))


def phase_space():
    """Phase-space (TPHS) and velocity (TVEL) trees on clustered particles with velocities:
    the tree, FindNearest(tt) and FindNearest(x) with the plain phase distance
    (Aniso = -1) and with the local metric (Aniso = 0, the reference's default), periodic
    and not; CalcDensity / CalcDensityParticle with the local metric (the reference
    reads uninitialised arrays for Aniso = -1); FOFCriterion with the three comparators on
    the phase-space tree."""
    n, box = 1000, 20.0
    pos, mass, vel = syn.clustered_box(n, box, seed=31, velocities=True)
    rng = np.random.default_rng(32)
    ids = np.array([0, 17, 404, 777, n - 1], np.int32)
    pts6 = np.concatenate([pos[ids], vel[ids]], 1) + rng.normal(scale=0.02, size=(len(ids), 6))
    pts3 = vel[ids] + rng.normal(scale=0.02, size=(len(ids), 3))
    out = dict(pos=pos, vel=vel, mass=mass, b=16, box=box, ids=ids, points6=pts6, points3=pts3)

    def mk(tt, aniso, per):
        return oracle.OracleTree(pos, vel, mass, 16, tt, 0, 1000, per, backend="ref",
                                 nthreads=4, aniso=aniso)
    for tag, aniso in (("plain", -1), ("metric", 0)):
        for ptag, per in (("", None), ("_per", [box] * 3)):
            t = mk(3, aniso, per)
            if aniso == -1 and per is None:
                out["phs_num_nodes"] = t.num_nodes
                out["phs_leaf_ids"] = _leaf_sets(t)
            nn, d2 = t.knn(10)
            out[f"phs_{tag}{ptag}_nn"], out[f"phs_{tag}{ptag}_d2"] = nn, d2
            nn, d2 = t.knn_coord(pts6, 10)
            out[f"phs_{tag}{ptag}_pt_nn"], out[f"phs_{tag}{ptag}_pt_d2"] = nn, d2
            if aniso == 0:
                out[f"phs_{tag}{ptag}_rho"] = mk(3, aniso, per).density(16)
                out[f"phs_{tag}{ptag}_rho_id"] = np.array(
                    [t.density_particle(int(i), 16) for i in ids])
    t = mk(2, 0, None)
    out["vel_num_nodes"] = t.num_nodes
    out["vel_leaf_ids"] = _leaf_sets(t)
    out["vel_nn"], out["vel_d2"] = t.knn(10)
    out["vel_pt_nn"], out["vel_pt_d2"] = t.knn_coord(pts3, 10)
    out["vel_rho"] = mk(2, 0, None).density(16)
    # The search region (params[1], params[2] per dimension kind) contains each
    # comparator's linking region, so every link is found from both of its ends; the
    # reference's breadth-first grouping relies on that (otherwise a later group can take
    # a particle of an earlier one, which corrupts its member lists).
    for cmp, (s1, s2, l6, l7) in ((0, (0.09, 1e30, 0.09, 0)), (1, (1e30, 0.0025, 0.0025, 0)),
                                  (2, (0.25, 0.04, 0.25, 0.04))):
        params = np.zeros(20)
        params[:3] = [3, s1, s2]
        params[6:8] = [l6, l7]
        out[f"fof_params_{cmp}"] = params
        for ptag, per in (("", None), ("_per", [box] * 3)):
            g, ng = mk(3, 0, per).fof_criterion(cmp, params, 8, 0)
            out[f"fof{ptag}_{cmp}"], out[f"fof{ptag}_{cmp}_ng"] = g, ng
    return out


FIXTURES = [("uniform_periodic", uniform_periodic), ("clustered", clustered),
            ("nonperiodic", nonperiodic), ("tiny_periodic", tiny_periodic),
            ("smoothing", smoothing), ("phase_space", phase_space),
            ("position_density", position_density)]


def main(names=None):
    """Writes the named fixtures (all of them without names)."""
    oracle.build(ref=True)
    for name, fn in FIXTURES:
        if names and name not in names:
            continue
        d = fn()
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1:])
