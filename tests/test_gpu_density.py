"""GPU parity: SPH density (CalcDensity), velocity density (CalcVelDensity) and the
single-particle variants, within the stated 1e-12 relative tolerance."""
import os

import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree, KEPAN, KGAUSS, KSPH, KTH
from nbodylib_gb300 import synthetic as syn
from nbodylib_gb300._capi import NbkError
from tests.helpers import assert_density_close, golden

pytestmark = pytest.mark.gpu


def test_golden_densities(gpu):
    g = golden("uniform_periodic")
    t = KDTree(g["pos"], None, g["mass"], 16, kerntype=0, period=g["period"])
    assert_density_close(t.CalcDensity(int(g["k_density"])), g["rho"], "uniform")
    g = golden("nonperiodic")
    t = KDTree(g["pos"], None, g["mass"], 8, kerntype=KEPAN)
    assert_density_close(t.CalcDensity(20), g["rho"], "epanechnikov")
    g = golden("clustered")
    t = KDTree(g["pos"], g["vel"], g["mass"], 16, kerntype=0, period=g["period"])
    assert_density_close(t.CalcDensity(32), g["rho"], "clustered")
    assert_density_close(t.CalcVelDensity(32, 32), g["veldens_32_32"], "veldens 32/32")
    assert_density_close(t.CalcVelDensity(16, 32), g["veldens_16_32"], "veldens 16/32")
    inv = np.argsort(t.GetPerm())  # ID -> tree index
    tg = inv[g["query_ids"]]
    assert_density_close(t.CalcDensityParticle(tg, 32), g["dens_particle"], "particle")
    assert_density_close(t.CalcVelDensityParticle(tg, 16, 32), g["veldens_particle"],
                         "vel particle")


def test_uniform_32768_k32_density_vs_oracle(gpu, port_built):
    pos, mass = syn.uniform_box(32768, 1.0, seed=1)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, [1, 1, 1], backend="port")
    t = KDTree(pos, None, mass, 16, kerntype=KSPH, period=[1, 1, 1])
    assert_density_close(t.CalcDensity(32), o.density(32), "C1 density")


@pytest.mark.parametrize("kern", [KSPH, KGAUSS, KEPAN, KTH])
def test_kernels_vs_oracle(gpu, port_built, kern):
    pos, mass = syn.clustered_box(20000, 50.0, seed=41)
    o = oracle.OracleTree(pos, None, mass, 16, 0, kern, 500, None, backend="port")
    t = KDTree(pos, None, mass, 16, kerntype=kern, kernres=500)
    tab, _ = t.GetKernel()
    np.testing.assert_array_equal(tab, o.kernel_table())
    assert_density_close(t.CalcDensity(24), o.density(24), f"kernel {kern}")


def test_clustered_density_and_veldensity_fused_vs_oracle(gpu, port_built):
    n = 1 << 17
    pos, mass, vel = syn.clustered_box(n, 250.0, seed=3, velocities=True)
    o = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port")
    rho_o = o.density(64)
    o2 = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port")
    vd_o = o2.veldensity(64, 64)
    t = KDTree(pos, vel, mass, 16, kerntype=0)
    rho, vd = t.CalcDensityAndVelDensity(64, 64)
    assert_density_close(rho, rho_o, "fused rho")
    assert_density_close(vd, vd_o, "fused veldens")
    assert_density_close(t.CalcDensity(64), rho_o, "rho")
    assert_density_close(t.CalcVelDensity(64, 64), vd_o, "veldens")


def test_too_few_neighbours_is_an_error_not_exit(gpu):
    pos = np.random.default_rng(1).random((10, 3))
    t = KDTree(pos, None, None, 4, kerntype=0)
    with pytest.raises(NbkError) as e:
        t.CalcDensity(10)
    assert e.value.status == 5


def test_density_full_size_sampled(gpu, port_built):
    """At the 2^20 clustered size: the gather-only density of 2000 sampled particles and
    the full scatter density satisfy sum_i rho_i = sum over pairs; check the sample
    against the oracle exactly (1e-12)."""
    n = 1 << 20
    pos, mass = syn.clustered_box(n, 100.0, seed=2)
    t = KDTree(pos, None, mass, 16, kerntype=0, period=[100.0] * 3)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, [100.0] * 3, backend="port",
                          nthreads=16)
    ids = np.random.default_rng(7).choice(n, 2000, replace=False)
    inv = np.argsort(t.GetPerm())
    got = t.CalcDensityParticle(inv[ids], 32)
    want = np.array([o.density_particle(int(i), 32) for i in ids])
    assert_density_close(got, want, "sampled particle density")
    rho = t.CalcDensity(32)
    assert np.all(rho > 0) and np.all(np.isfinite(rho))


def test_256cubed_full_arrays(gpu, port_built):
    """The largest configuration, 256^3 = 16,777,216 clustered particles in L = 250 with
    velocities, k = 64, every particle: CalcDensity(64) and CalcVelDensity(64, 64) (the
    separate calls the bench times, and the fused one-traversal form) element by element
    against the restatement run over all host threads, <= 1e-12; FindNearest(x) at 1000
    sampled particles' positions, CalcDensityParticle(64) and CalcVelDensityParticle(64,
    64) at the same particles; and a checksum of the full scatter density: with equal
    masses, every pair's half-weight is added once at each end, so sum_i CalcDensity_i
    equals sum_i CalcDensityParticle_i."""
    from tests.helpers import assert_knn_equal, to_ids
    n = 1 << 24
    pos, mass, vel = syn.clustered_box(n, 250.0, seed=3, velocities=True)
    assert np.all(mass == mass[0])
    t = KDTree(pos, vel, mass, 16, kerntype=0)
    o = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port", nthreads=16)
    ids = np.random.default_rng(11).choice(n, 1000, replace=False)
    perm = np.asarray(t.GetPerm())
    inv = np.argsort(perm)
    x = pos[ids]
    nn, d2 = t.FindNearestPoints(x, 64)
    want_nn, want_d2 = o.knn_coord(x, 64)
    assert_knn_equal(to_ids(np.asarray(nn), perm), d2, want_nn, want_d2, "FindNearest(x) 256^3")
    got = t.CalcDensityParticle(inv[ids], 64)
    want = np.array([o.density_particle(int(i), 64) for i in ids])
    assert_density_close(got, want, "CalcDensityParticle 256^3")
    got = t.CalcVelDensityParticle(inv[ids], 64, 64)
    want = np.array([o.veldensity_particle(int(i), 64, 64) for i in ids])
    assert_density_close(got, want, "CalcVelDensityParticle 256^3")
    rho = np.asarray(t.CalcDensity(64))
    vden = np.asarray(t.CalcVelDensity(64, 64))
    threads = os.cpu_count() or 1
    want_rho = o.density_parallel(64, nthreads=threads)
    assert_density_close(rho, want_rho, "CalcDensity(64), all 256^3 particles")
    want_v = o.veldensity_parallel(64, 64, nthreads=threads)
    assert_density_close(vden, want_v, "CalcVelDensity(64, 64), all 256^3 particles")
    rho2, vden2 = t.CalcDensityAndVelDensity(64, 64)
    assert_density_close(np.asarray(rho2), want_rho, "fused CalcDensity(64), 256^3")
    assert_density_close(np.asarray(vden2), want_v, "fused CalcVelDensity(64, 64), 256^3")
    o.close()
    del want_rho, want_v, rho2, vden2
    gather = np.asarray(t.CalcDensityParticle(np.arange(n, dtype=np.int32), 64))
    assert np.all(rho > 0) and np.all(np.isfinite(rho))
    assert abs(rho.sum() - gather.sum()) <= 1e-10 * gather.sum()
    t.close()


def test_position_density_golden_and_restatement(gpu, port_built):
    """CalcDensityPosition / CalcVelDensityPosition against the reference's outputs in the
    fixture (period ignored; points at particles, inside and outside the box), then on
    2^17 clustered particles at 4000 points against the restatement, host and device
    buffers; refused on velocity trees and for k above the particle count."""
    import torch
    g = golden("position_density")
    t = KDTree(g["pos"], g["vel"], g["mass"], int(g["b"]), kerntype=0, period=g["period"])
    pts, pv = g["points"], g["point_vel"]
    assert_density_close(t.CalcDensityPosition(pts, 32), g["dens_k32"], "position k=32")
    assert_density_close(t.CalcDensityPosition(pts, 8), g["dens_k8"], "position k=8")
    assert_density_close(t.CalcVelDensityPosition(pts, pv, 16, 32), g["veldens_16_32"],
                         "vel position 16/32")
    with pytest.raises(NbkError):
        t.CalcDensityPosition(pts, len(g["mass"]) + 1)
    t.close()
    from nbodylib_gb300.kdtree import TVEL
    tv = KDTree(g["pos"], g["vel"], g["mass"], 16, treetype=TVEL, kerntype=0)
    with pytest.raises(NbkError):
        tv.CalcDensityPosition(pv, 8)
    tv.close()

    n = 1 << 17
    pos, mass, vel = syn.clustered_box(n, 50.0, seed=35, velocities=True)
    rng = np.random.default_rng(36)
    pts = np.concatenate([pos[::64], rng.random((2000, 3)) * 50.0])
    pv = rng.normal(size=(len(pts), 3))
    P = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port")
    t = KDTree(pos, vel, mass, 16, kerntype=0)
    assert_density_close(t.CalcDensityPosition(pts, 40),
                         [P.density_position(x, 40) for x in pts], "position 2^17")
    want_v = [P.veldensity_position(x, v, 24, 48) for x, v in zip(pts, pv)]
    assert_density_close(t.CalcVelDensityPosition(pts, pv, 24, 48), want_v, "vel position 2^17")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    td = KDTree(dev(pos), dev(vel), dev(mass), 16, kerntype=0, device=True)
    got = td.CalcVelDensityPosition(dev(pts), dev(pv), 24, 48).cpu().numpy()
    assert_density_close(got, want_v, "vel position 2^17, device buffers")
    t.close()
    td.close()
