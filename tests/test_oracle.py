"""CPU tests: the oracle restatement against the golden fixtures (made by the reference)
and, where the reference checkout exists, against the compiled reference directly."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import synthetic as syn
from tests.helpers import (assert_density_close, assert_knn_equal, assert_same_partition,
                           brute_min_image_knn, golden)


def port(pos, vel=None, mass=None, b=16, kerntype=0, period=None):
    return oracle.OracleTree(pos, vel, mass, b, 0, kerntype, 1000, period, backend="port",
                             nthreads=4)


def test_port_matches_golden_uniform_periodic(port_built):
    g = golden("uniform_periodic")
    t = port(g["pos"], None, g["mass"], int(g["b"]), int(g["kerntype"]), g["period"])
    assert t.num_nodes == g["num_nodes"] and t.num_leaves == g["num_leaves"]
    k = int(g["k"])
    for m, key in [(0, "findnearest"), (1, "findnearestpos")]:
        nn, d2 = t.knn(k, method=m)
        np.testing.assert_array_equal(nn, g["nn_" + key])
        np.testing.assert_array_equal(d2, g["d2_" + key])
    rho = t.density(int(g["k_density"]))
    np.testing.assert_array_equal(rho, g["rho"])
    t2 = port(g["pos"], None, g["mass"], int(g["b"]), int(g["kerntype"]), g["period"])
    grp, ng = t2.fof(float(g["ll"]), int(g["fof_minnum"]))
    assert ng == int(g["fof_ngroup"])
    np.testing.assert_array_equal(grp, g["fof_group"])


def test_port_matches_golden_clustered(port_built):
    g = golden("clustered")
    per = g["period"]
    mk = lambda: port(g["pos"], g["vel"], g["mass"], int(g["b"]), int(g["kerntype"]), per)
    np.testing.assert_array_equal(mk().density(int(g["k"])), g["rho"])
    np.testing.assert_array_equal(mk().veldensity(32, 32), g["veldens_32_32"])
    np.testing.assert_array_equal(mk().veldensity(16, 32), g["veldens_16_32"])
    t = mk()
    ids = g["query_ids"]
    np.testing.assert_array_equal([t.density_particle(i, 32) for i in ids], g["dens_particle"])
    np.testing.assert_array_equal([t.veldensity_particle(i, 16, 32) for i in ids],
                                  g["veldens_particle"])
    grp, ng = mk().fof(float(g["ll"]), 10, 0)
    assert ng == int(g["fof_ngroup"])
    np.testing.assert_array_equal(grp, g["fof_group"])
    grp, ng = mk().fof(float(g["ll"]), 10, 1)
    np.testing.assert_array_equal(grp, g["fof_group_ordered"])
    off = g["ball_offsets"]
    for j, i in enumerate(ids):
        got = t.ball_tagged(int(i), float(g["ball_r2"]))
        np.testing.assert_array_equal(got, np.sort(g["ball_ids"][off[j]:off[j + 1]]))


def test_port_matches_golden_nonperiodic(port_built):
    g = golden("nonperiodic")
    t = port(g["pos"], None, g["mass"], int(g["b"]), int(g["kerntype"]))
    nn, d2 = t.knn(int(g["k"]), 0)
    np.testing.assert_array_equal(nn, g["nn_findnearest"])
    np.testing.assert_array_equal(d2, g["d2_findnearest"])
    np.testing.assert_array_equal(port(g["pos"], None, g["mass"], 8, 2).density(20), g["rho"])
    nnx, d2x = t.knn_pos(g["points"], 12)
    np.testing.assert_array_equal(nnx, g["knn_points_nn"])
    np.testing.assert_array_equal(d2x, g["knn_points_d2"])
    for j, i in enumerate(g["query_ids"][:10]):
        m, d = t.ball_mark(int(i), float(g["ball_r2"]), imark=7)
        np.testing.assert_array_equal(np.where(m == 7, d, -1.0), g["mark_d2"][j])


def test_port_matches_golden_tiny_periodic(port_built):
    g = golden("tiny_periodic")
    t = port(g["pos"], None, g["mass"], 16, 0, g["period"])
    for m, key in [(0, "findnearest"), (1, "findnearestpos")]:
        nn, d2 = t.knn(int(g["k"]), m)
        np.testing.assert_array_equal(nn, g["nn_" + key])
        np.testing.assert_array_equal(d2, g["d2_" + key])


def test_port_periodic_gate_bug_vs_brute_force(port_built):
    """The reference's 2-D/3-D image gate compares a squared distance with a distance
    (KDSplitNode.cxx:1134-1146): near box edges and corners some true neighbours are
    missed. The restatement reproduces that; brute-force minimum image shows it."""
    n, k = 4096, 32
    pos, mass = syn.uniform_box(n, 1.0, seed=21)
    t = port(pos, None, mass, 16, 0, [1, 1, 1])
    nn, d2 = t.knn(k, 0)
    bid, bd2 = brute_min_image_knn(pos, [1, 1, 1], k)
    wrong = np.any(np.sort(nn, 1) != np.sort(bid, 1), axis=1)
    near = ((pos < 0.15) | (pos > 0.85)).sum(1)
    assert wrong.sum() > 0
    assert np.all(near[wrong] >= 2)  # only edge/corner particles are affected


@pytest.mark.parametrize("periodic", [False, True])
def test_port_matches_reference(ref_built, periodic):
    n = 20000
    pos, mass, vel = syn.clustered_box(n, 100.0, seed=22, velocities=True)
    per = [100.0] * 3 if periodic else None
    R = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per, backend="ref", nthreads=4)
    P = port(pos, vel, mass, 16, 0, per)
    np.testing.assert_array_equal(R.ids(), P.ids())
    for m in (0, 1):
        a, b = R.knn(32, m), P.knn(32, m)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(R.density(32), P.density(32))
    np.testing.assert_array_equal(R.veldensity(24, 32), P.veldensity(24, 32))
    ll = syn.linking_length(n, 100.0)
    ga, na = R.fof(ll, 20)
    gb, nb = P.fof(ll, 20)
    assert na == nb
    np.testing.assert_array_equal(ga, gb)
    par = [0, (1.5 * ll) ** 2, 0, 0, 0, 0, ll * ll, 0.01]
    for cmp in (0, 2):
        ga, na = R.fof_criterion(cmp, par, 10)
        gb, nb = P.fof_criterion(cmp, par, 10)
        assert na == nb
        np.testing.assert_array_equal(ga, gb)


def test_port_parallel_density_matches_serial(port_built):
    # the threaded CalcDensity / CalcVelDensity used to check the 256^3 arrays: the
    # density within a few ulps of the serial restatement (summation order only), the
    # velocity density bit-identical
    pos, mass, vel = syn.clustered_box(30000, 30.0, seed=9, velocities=True)
    o = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port", nthreads=4)
    rho = o.density(32)
    rp = o.density_parallel(32, nthreads=4)
    assert np.max(np.abs(rp - rho) / rho) <= 1e-14
    v = o.veldensity(32, 64)
    vp = o.veldensity_parallel(32, 64, nthreads=4)
    assert np.array_equal(v, vp)
    o.close()


def test_adjoint_restatement_finite_differences(port_built):
    """The CPU adjoint (frozen neighbour lists and table cells) against central finite
    differences of the same frozen model."""
    n, k = 3000, 16
    pos, mass = syn.clustered_box(n, 10.0, seed=23)
    t = port(pos, None, mass, 16, 0)
    rho, nn = t.density(k, return_nn=True)
    w = np.random.default_rng(5).normal(size=n)
    rho2, gp, gm = t.density_adjoint(k, nn, w)
    assert_density_close(rho2, rho, "frozen forward")
    rng = np.random.default_rng(6)
    h = 1e-6
    # full-sum differencing on a few coordinates (loose: it cancels)
    for _ in range(5):
        a, d = int(rng.integers(n)), int(rng.integers(3))
        pp, pm = pos.copy(), pos.copy()
        pp[a, d] += h
        pm[a, d] -= h
        lp = np.sum(w * np.log(t.density_frozen(k, nn, pos, pp)))
        lm = np.sum(w * np.log(t.density_frozen(k, nn, pos, pm)))
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gp[a, d]) <= 1e-5 * max(1.0, abs(gp[a, d])), (a, d, fd, gp[a, d])
    # local differencing of the affected terms: the 1e-6 relative bar
    coords = np.stack([rng.integers(0, n, 300), rng.integers(0, 3, 300)], 1)
    fd1 = t.local_fd(k, nn, w, coords, step=h)
    fd2 = t.local_fd(k, nn, w, coords, step=h / 2)
    fd = (4 * fd2 - fd1) / 3  # Richardson: removes the O(h^2) truncation term
    g = gp[coords[:, 0], coords[:, 1]]
    rel = np.abs(fd - g) / np.maximum(np.abs(g), 1e-3 * np.abs(gp).max())
    assert rel.max() <= 1e-6, rel.max()


def _smoothing_inputs():
    pos, mass, vel = syn.clustered_box(2500, 50.0, seed=21, velocities=True)
    return pos, mass, vel


@pytest.mark.parametrize("given_rho", [False, True])
def test_port_smoothing_matches_reference(ref_built, given_rho):
    """CalcSmoothVel / VelDisp / VelSkew / VelKurtosis and the Particle / Position forms of
    CalcSmoothVel, CalcSmoothVelDisp, CalcSmoothLocalMean, CalcSmoothLocalDisp: the
    restatement is bit-identical to the compiled reference, with the densities computed
    inside (densityset != 1) or given (densityset = 1)."""
    pos, mass, vel = _smoothing_inputs()
    R = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="ref")
    P = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port")
    k = 24
    rho = R.density(k) * 1.25 if given_rho else None
    sv = R.smooth_vel_moments(0, k, rho)
    dp = R.smooth_vel_moments(1, k, rho, sv).reshape(-1, 9)
    for which in range(4):
        a = R.smooth_vel_moments(which, k, rho, sv, dp)
        b = P.smooth_vel_moments(which, k, rho, sv, dp)
        assert np.array_equal(a, b), f"moment {which}"
    w = np.random.default_rng(2).random(len(mass))
    for pid in (0, 911, len(mass) - 1):
        for which in (0, 1, 4, 5):
            args = dict(rho=rho, smvel=sv[pid], weight=w, mean=0.4)
            assert np.array_equal(R.smooth_one(which, k, pid=pid, **args),
                                  P.smooth_one(which, k, pid=pid, **args)), (which, pid)
            x = pos[pid] + 0.013
            assert np.array_equal(R.smooth_one(which, k, x=x, **args),
                                  P.smooth_one(which, k, x=x, **args)), (which, pid, "position")


def test_port_veldensity_phys_matches_reference(ref_built):
    """CalcVelDensityWithPhysDensity[Particle], whose physical h is half the largest squared
    distance (KDCalcSmoothQuantities.cxx:428): compared where every neighbour distance is
    above 1, so the reference's table index stays inside its table."""
    rng = np.random.default_rng(11)
    n = 3000
    pos = rng.random((n, 3)) * 200.0
    vel = rng.normal(size=(n, 3))
    mass = rng.random(n) + 0.5
    R = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="ref")
    P = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port")
    for rho in (None, R.density(16) * 1.3):
        a = R.veldensity_phys(16, 32, rho)
        assert np.array_equal(a, P.veldensity_phys(16, 32, rho))
        for pid in (0, 17, n - 1):
            assert R.veldensity_phys_particle(pid, 16, 32, rho) == \
                P.veldensity_phys_particle(pid, 16, 32, rho)


def test_port_matches_golden_smoothing(port_built):
    """The restatement reproduces the reference's smoothing outputs stored in the fixture."""
    g = golden("smoothing")
    P = oracle.OracleTree(g["pos"], g["vel"], g["mass"], int(g["b"]), 0, 0, 1000, None,
                          backend="port")
    k = int(g["k"])
    assert np.array_equal(P.smooth_vel_moments(0, k), g["smvel"])
    assert np.array_equal(P.smooth_vel_moments(1, k, None, g["smvel"]).reshape(-1, 9), g["veldisp"])
    assert np.array_equal(P.smooth_vel_moments(2, k, None, g["smvel"], g["veldisp"]), g["velskew"])
    assert np.array_equal(P.smooth_vel_moments(3, k, None, g["smvel"], g["veldisp"]), g["velkurt"])
    for n, i in enumerate(g["ids"]):
        assert np.array_equal(P.smooth_one(0, k, pid=int(i)), g["vel_id"][n])
        assert np.array_equal(P.smooth_one(4, k, pid=int(i), weight=g["weight"]), g["mean_id"][n])
        assert np.array_equal(P.smooth_one(5, k, x=g["points"][n], weight=g["weight"],
                                           mean=float(g["mean_ref"])), g["disp_pt"][n])
    Q = oracle.OracleTree(g["phys_pos"], g["phys_vel"], g["phys_mass"], 16, 0, 0, 1000, None,
                          backend="port")
    assert np.array_equal(Q.veldensity_phys(int(g["phys_nsmooth"]), int(g["phys_nsearch"])),
                          g["veldensity_phys"])


def test_port_matches_golden_position_density(port_built):
    """CalcDensityPosition / CalcVelDensityPosition: the restatement reproduces the
    reference's outputs bit for bit (period ignored, points inside and outside the box);
    velocity and phase-space trees are not restated (NaN)."""
    g = golden("position_density")
    P = oracle.OracleTree(g["pos"], g["vel"], g["mass"], int(g["b"]), 0, 0, 1000, g["period"],
                          backend="port")
    pts, pv = g["points"], g["point_vel"]
    assert np.array_equal([P.density_position(x, 32) for x in pts], g["dens_k32"])
    assert np.array_equal([P.density_position(x, 8) for x in pts], g["dens_k8"])
    assert np.array_equal([P.veldensity_position(x, v, 16, 32) for x, v in zip(pts, pv)],
                          g["veldens_16_32"])
    V = oracle.OracleTree(g["pos"], g["vel"], g["mass"], int(g["b"]), 2, 0, 1000, None,
                          backend="port")
    assert np.isnan(V.density_position(pv[0], 8))


def test_port_noncubic_period_matches_reference(ref_built):
    """A different period per dimension, particles crowding the faces: FindNearest and
    FindNearestPos (the reference's image gates) and FOF."""
    rng = np.random.default_rng(44)
    per = np.array([100.0, 60.0, 35.0])
    pos = rng.random((6000, 3)) * per
    face = rng.integers(0, 3, 2000)
    pos[np.arange(2000), face] = per[face] * np.where(rng.random(2000) < 0.5, 0.01, 0.99)
    mass = np.full(6000, 1.0 / 6000)
    P = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, list(per), backend="port")
    R = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, list(per), backend="ref")
    for m in (0, 1):
        pn, pd = P.knn(12, m)
        rn, rd = R.knn(12, m)
        assert_knn_equal(pn, pd, rn, rd, f"non-cubic method {m}", dropped_nearest=(m == 0))
    ll = 0.2 * (np.prod(per) / 6000) ** (1.0 / 3.0)
    gp, npg = P.fof(ll, 5)
    gr, nr = R.fof(ll, 5)
    assert npg == nr
    assert_same_partition(gp, gr, "non-cubic FOF")


def test_port_position_density_matches_reference(ref_built):
    pos, mass, vel = syn.clustered_box(4000, 30.0, seed=33, velocities=True)
    rng = np.random.default_rng(34)
    pts = np.concatenate([pos[::200], rng.random((20, 3)) * 30.0])
    pv = rng.normal(size=(len(pts), 3))
    for per in (None, [30.0] * 3):
        P = oracle.OracleTree(pos, vel, mass, 8, 0, 0, 1000, per, backend="port")
        R = oracle.OracleTree(pos, vel, mass, 8, 0, 0, 1000, per, backend="ref")
        # k >= 2: with k = 1 at a particle's own position h = 0, and the reference's table
        # index (int)(0/0) falls outside its table
        for k in (2, 20, 64):
            assert np.array_equal([P.density_position(x, k) for x in pts],
                                  [R.density_position(x, k) for x in pts])
        assert np.array_equal([P.veldensity_position(x, v, 10, 40) for x, v in zip(pts, pv)],
                              [R.veldensity_position(x, v, 10, 40) for x, v in zip(pts, pv)])


@pytest.mark.parametrize("cmp", [0, 1, 2])
def test_port_fof_nn_matches_reference(ref_built, cmp):
    """FOFNNCriterion and FOFNNDistCriterion over FindNearest lists: the restatement gives
    the reference's groups and numbering exactly."""
    pos, mass, vel = syn.clustered_box(4000, 60.0, seed=41 + cmp, velocities=True)
    R = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="ref")
    P = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port")
    rn, rd = R.tree_knn(12)
    pn, pd = P.tree_knn(12)
    params = [0, 0.25, 1.0, 0, 0, 0, 0.25, 0.3]
    gr, ngr = R.fof_nn(cmp, params, rn, 5)
    gp, ngp = P.fof_nn(cmp, params, pn, 5)
    assert ngr == ngp and np.array_equal(gr, gp)
    gr, ngr = R.fof_nn(cmp, params, rn, 5, pidx=[6], dist2=rd * 0.4)
    gp, ngp = P.fof_nn(cmp, params, pn, 5, values=(pd * 0.4).max(1), pidx=[6])
    assert ngr == ngp and np.array_equal(gr, gp)


def _phase_tree(g, treetype, aniso, periodic, backend="port"):
    per = [float(g["box"])] * 3 if periodic else None
    return oracle.OracleTree(g["pos"], g["vel"], g["mass"], int(g["b"]), treetype, 0, 1000, per,
                             backend=backend, nthreads=4, aniso=aniso)


@pytest.mark.parametrize("aniso", [-1, 0])
@pytest.mark.parametrize("periodic", [False, True])
def test_port_phase_space_matches_golden(port_built, aniso, periodic):
    """Phase-space trees: FindNearest(tt), FindNearest(x) and, with the local metric,
    CalcDensity / CalcDensityParticle, bit-identical to the reference's outputs."""
    g = golden("phase_space")
    tag = ("plain" if aniso == -1 else "metric") + ("_per" if periodic else "")
    t = _phase_tree(g, 3, aniso, periodic)
    assert t.num_nodes == int(g["phs_num_nodes"])
    k = g[f"phs_{tag}_nn"].shape[1]
    nn, d2 = t.knn(k)
    np.testing.assert_array_equal(nn, g[f"phs_{tag}_nn"])
    np.testing.assert_array_equal(d2, g[f"phs_{tag}_d2"])
    nn, d2 = t.knn_coord(g["points6"], k)
    np.testing.assert_array_equal(nn, g[f"phs_{tag}_pt_nn"])
    np.testing.assert_array_equal(d2, g[f"phs_{tag}_pt_d2"])
    if aniso == 0:
        np.testing.assert_array_equal(_phase_tree(g, 3, aniso, periodic).density(16),
                                      g[f"phs_{tag}_rho"])
        np.testing.assert_array_equal([t.density_particle(int(i), 16) for i in g["ids"]],
                                      g[f"phs_{tag}_rho_id"])


def test_port_velocity_tree_matches_golden(port_built):
    g = golden("phase_space")
    t = _phase_tree(g, 2, 0, False)
    assert t.num_nodes == int(g["vel_num_nodes"])
    k = g["vel_nn"].shape[1]
    nn, d2 = t.knn(k)
    np.testing.assert_array_equal(nn, g["vel_nn"])
    np.testing.assert_array_equal(d2, g["vel_d2"])
    nn, d2 = t.knn_coord(g["points3"], k)
    np.testing.assert_array_equal(nn, g["vel_pt_nn"])
    np.testing.assert_array_equal(d2, g["vel_pt_d2"])
    np.testing.assert_array_equal(_phase_tree(g, 2, 0, False).density(16), g["vel_rho"])


@pytest.mark.parametrize("cmp", [0, 1, 2])
@pytest.mark.parametrize("periodic", [False, True])
def test_port_phase_space_fof_criterion_matches_golden(port_built, cmp, periodic):
    g = golden("phase_space")
    tag = "_per" if periodic else ""
    grp, ng = _phase_tree(g, 3, 0, periodic).fof_criterion(cmp, g[f"fof_params_{cmp}"], 8, 0)
    assert ng == int(g[f"fof{tag}_{cmp}_ng"])
    np.testing.assert_array_equal(grp, g[f"fof{tag}_{cmp}"])


@pytest.mark.parametrize("aniso", [-1, 0])
@pytest.mark.parametrize("periodic", [False, True])
def test_port_phase_space_matches_reference(ref_built, aniso, periodic):
    """A larger clustered set straight against the compiled reference."""
    pos, mass, vel = syn.clustered_box(4000, 30.0, seed=41, velocities=True)
    per = [30.0] * 3 if periodic else None
    mk = lambda be: oracle.OracleTree(pos, vel, mass, 16, 3, 0, 1000, per, backend=be,
                                      nthreads=4, aniso=aniso)
    R, P = mk("ref"), mk("port")
    np.testing.assert_array_equal(R.ids(), P.ids())
    a, da = R.knn(16)
    b, db = P.knn(16)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(da, db)
    if aniso == 0:
        np.testing.assert_array_equal(mk("ref").density(32), mk("port").density(32))


def _phase_edge_inputs(n, dup, box, seed=3):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)) * box
    vel = rng.normal(size=(n, 3)) * 0.3
    m = rng.random(n) + 0.5
    if dup:  # exact duplicates: zero distances, ties, a metric spacing over zero offsets
        pos[n // 2: n // 2 + dup] = pos[:dup]
        vel[n // 2: n // 2 + dup] = vel[:dup]
    return pos, vel, m


PHASE_EDGE_CASES = [(12, 0, 5.0, 4), (12, 0, None, 4), (9, 0, 3.0, 3), (300, 40, 10.0, 8),
                    (300, 40, None, 8)]


@pytest.mark.parametrize("n,dup,per,k", PHASE_EDGE_CASES)
@pytest.mark.parametrize("aniso", [-1, 0])
def test_port_phase_space_edge_cases_match_reference(ref_built, n, dup, per, k, aniso):
    """Trees that are one leaf (periodic: no images), fewer than 16 particles, exact
    duplicates: FindNearest(tt), FindNearest(x) and CalcDensity bit-identical."""
    pos, vel, m = _phase_edge_inputs(n, dup, per or 10.0)
    mk = lambda be: oracle.OracleTree(pos, vel, m, 16, 3, 0, 1000, per, backend=be, nthreads=2,
                                      aniso=aniso)
    R, P = mk("ref"), mk("port")
    for (a, da), (b, db) in ((R.knn(k), P.knn(k)),
                             (R.knn_coord(np.hstack([pos[:5], vel[:5]]) + 0.01, k),
                              P.knn_coord(np.hstack([pos[:5], vel[:5]]) + 0.01, k))):
        np.testing.assert_array_equal(da, db)
        np.testing.assert_array_equal(a, b)
    if aniso == 0:
        np.testing.assert_array_equal(mk("ref").density(k), mk("port").density(k))
