"""GPU SPH smoothing family (KDCalcSmoothQuantities.cxx: CalcSmoothVel, CalcSmoothVelDisp,
CalcSmoothVelSkew, CalcSmoothVelKurtosis, CalcVelDensityWithPhysDensity and the Particle /
Position forms of CalcSmoothVel, CalcSmoothVelDisp, CalcSmoothLocalMean, CalcSmoothLocalDisp)
against the reference's outputs in the golden fixture and against the C restatement.

The neighbour sets are exact; the sums are FP64 with a different summation order (FP64
atomics for the symmetric forms) and a one-FMA kernel interpolation, so values agree to a
few units in the last place of the terms: the bound below is 1e-12 relative to the largest
magnitude of each quantity (1e-12 of the value itself for the positive-definite ones)."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree
from nbodylib_gb300.kdtree import KSPH
from nbodylib_gb300 import synthetic as syn
from tests.helpers import golden

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def close(got, want, what, positive=False):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    assert got.shape == want.shape, (what, got.shape, want.shape)
    scale = np.abs(want) if positive else np.max(np.abs(want))
    err = np.abs(got - want)
    bad = err > RTOL * scale + 1e-300
    assert not bad.any(), (f"{what}: {bad.sum()} entries differ, worst "
                           f"{np.max(err / np.maximum(scale, 1e-300)):.3e} relative")


def tree_index_of(t, ids):
    perm = t.GetPerm()  # tree index -> input index
    perm = perm.cpu().numpy() if hasattr(perm, "cpu") else np.asarray(perm)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    return inv[np.asarray(ids)]


def test_smoothing_vs_reference_golden(gpu):
    g = golden("smoothing")
    k = int(g["k"])
    t = KDTree(g["pos"], g["vel"], g["mass"], int(g["b"]), kerntype=KSPH)
    rho = t.CalcDensity(k)
    close(rho, g["rho"], "CalcDensity", positive=True)
    sv = t.CalcSmoothVel(k)  # densities computed inside (densityset != 1)
    close(sv, g["smvel"], "CalcSmoothVel")
    close(t.CalcSmoothVel(k, rho=rho), g["smvel"], "CalcSmoothVel with given densities")
    disp = t.CalcSmoothVelDisp(g["smvel"], k)
    close(disp.reshape(-1, 9), g["veldisp"], "CalcSmoothVelDisp")
    close(t.CalcSmoothVelSkew(g["smvel"], g["veldisp"], k), g["velskew"], "CalcSmoothVelSkew")
    close(t.CalcSmoothVelKurtosis(g["smvel"], g["veldisp"], k), g["velkurt"],
          "CalcSmoothVelKurtosis")
    ti = tree_index_of(t, g["ids"])
    close(t.CalcSmoothVelParticle(ti, k), g["vel_id"], "CalcSmoothVelParticle")
    close(t.CalcSmoothVelPosition(g["points"], k), g["vel_pt"], "CalcSmoothVelPosition")
    close(t.CalcSmoothVelDispParticle(ti, g["smvel"][g["ids"]], k).reshape(-1, 9),
          g["veldisp_id"].reshape(-1, 9), "CalcSmoothVelDispParticle")
    close(t.CalcSmoothVelDispPosition(g["points"], g["smvel"][g["ids"]], k).reshape(-1, 9),
          g["veldisp_pt"].reshape(-1, 9), "CalcSmoothVelDispPosition")
    close(t.CalcSmoothLocalMeanParticle(ti, g["weight"], k), g["mean_id"],
          "CalcSmoothLocalMeanParticle", positive=True)
    close(t.CalcSmoothLocalMeanPosition(g["points"], g["weight"], k), g["mean_pt"],
          "CalcSmoothLocalMeanPosition", positive=True)
    m = np.full(len(ti), float(g["mean_ref"]))
    close(t.CalcSmoothLocalDispParticle(ti, g["weight"], m, k), g["disp_id"],
          "CalcSmoothLocalDispParticle", positive=True)
    close(t.CalcSmoothLocalDispPosition(g["points"], g["weight"], m, k), g["disp_pt"],
          "CalcSmoothLocalDispPosition", positive=True)
    t.close()


def test_veldensity_physdensity_vs_reference_golden(gpu):
    g = golden("smoothing")
    ns, nq = int(g["phys_nsmooth"]), int(g["phys_nsearch"])
    t = KDTree(g["phys_pos"], g["phys_vel"], g["phys_mass"], 16, kerntype=KSPH)
    close(t.CalcVelDensityWithPhysDensity(ns, nq), g["veldensity_phys"],
          "CalcVelDensityWithPhysDensity", positive=True)
    ti = tree_index_of(t, g["ids"])
    close(t.CalcVelDensityWithPhysDensityParticle(ti, ns, nq), g["veldensity_phys_id"],
          "CalcVelDensityWithPhysDensityParticle", positive=True)
    t.close()


@pytest.mark.parametrize("k", [16, 40, 64])
def test_smoothing_vs_restatement_device_arrays(gpu, port_built, k):
    """Larger clustered sets, the heap sizes of the three kernel families, device-resident
    inputs and outputs (torch tensors)."""
    import torch
    pos, mass, vel = syn.clustered_box(20000, 80.0, seed=31 + k, velocities=True)
    P = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, None, backend="port", nthreads=8)
    rho = P.density(k)
    want_sv = P.smooth_vel_moments(0, k, rho)
    want_dp = P.smooth_vel_moments(1, k, rho, want_sv).reshape(-1, 9)
    want_sk = P.smooth_vel_moments(2, k, rho, want_sv, want_dp)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    t = KDTree(dev(pos), dev(vel), dev(mass), 16, kerntype=KSPH, device=True)
    drho = dev(rho)
    close(t.CalcSmoothVel(k, rho=drho).cpu().numpy(), want_sv, f"CalcSmoothVel k={k}")
    close(t.CalcSmoothVelDisp(dev(want_sv), k, rho=drho).cpu().numpy().reshape(-1, 9), want_dp,
          f"CalcSmoothVelDisp k={k}")
    close(t.CalcSmoothVelSkew(dev(want_sv), dev(want_dp), k, rho=drho).cpu().numpy(), want_sk,
          f"CalcSmoothVelSkew k={k}")
    w = np.random.default_rng(k).random(len(mass))
    ids = np.arange(0, len(mass), 997)
    ti = dev(tree_index_of(t, ids).astype(np.int32))
    got = t.CalcSmoothLocalMeanParticle(ti, dev(w), k, rho=drho).cpu().numpy()
    want = [P.smooth_one(4, k, pid=int(i), rho=rho, weight=w) for i in ids]
    close(got, want, f"CalcSmoothLocalMeanParticle k={k}", positive=True)
    t.close()


def test_smoothing_rejects_bad_input(gpu):
    pos, mass, vel = syn.clustered_box(500, 10.0, seed=3, velocities=True)
    t = KDTree(pos, vel, mass, 16)
    from nbodylib_gb300._capi import NbkError
    with pytest.raises(NbkError):
        t.CalcSmoothVel(600)  # more neighbours than particles
    with pytest.raises(NbkError):
        t.CalcSmoothVelParticle(np.array([0, 500]), 16)  # target outside the tree
    t.close()
    t2 = KDTree(pos, None, mass, 16)
    with pytest.raises(NbkError):
        t2.CalcSmoothVel(16)  # no velocities
    t2.close()
