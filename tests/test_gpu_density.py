"""GPU parity: SPH density (CalcDensity), velocity density (CalcVelDensity) and the
single-particle variants, within the stated 1e-12 relative tolerance."""
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
