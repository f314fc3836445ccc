"""The C++ drop-in NBody::KDTree (include/nbkdt/KDTree.h): it compiles against the
reference's own NBody headers (source compatibility, CPU) and, run on the GPU through a
reference-style call sequence, gives the oracle's results (GPU)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from nbodylib_gb300 import _build
from nbodylib_gb300 import synthetic as syn
from tests.helpers import assert_density_close, assert_knn_equal, assert_same_partition

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cxx", "dropin_demo.cpp")


def compile_demo(out, include_nbody, link=True):
    libdir = os.path.dirname(_build.LIB)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           *sum((["-I", d] for d in include_nbody), []), SRC, "-o", out]
    cmd += ["-L", libdir, "-lnbkdt", f"-Wl,-rpath,{libdir}"] if link else ["-c"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_compiles_against_the_reference_headers(lib_built, tmp_path):
    ref = oracle.ref_src()
    if not os.path.isdir(os.path.join(ref, "src", "NBody")):
        pytest.skip("reference checkout not present on this machine")
    inc = [os.path.join(ROOT, "oracle", "gslshim"), os.path.join(ref, "src", "NBody"),
           os.path.join(ref, "src", "Math")]
    # compile only: linking needs NBodylib's own library (Particle's constructors)
    compile_demo(str(tmp_path / "demo_ref.o"), inc, link=False)


def test_reference_density_smooth_compiles_unmodified(lib_built, tmp_path):
    """The reference's own in-repo caller, src/Analysis/Density.cxx (DensitySmooth:
    KDTree(S, b) + CalcDensity), compiles unmodified against the drop-in through
    include/compat/KDTree.h placed ahead of the reference's KDTree headers."""
    ref = oracle.ref_src()
    src = os.path.join(ref, "src", "Analysis", "Density.cxx")
    if not os.path.exists(src):
        pytest.skip("reference checkout not present on this machine")
    inc = [os.path.join(ROOT, "include", "compat"), os.path.join(ROOT, "include"),
           os.path.join(ROOT, "oracle", "gslshim"), os.path.join(ref, "src", "NBody"),
           os.path.join(ref, "src", "Math"), os.path.join(ref, "src", "Analysis")]
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", *sum((["-I", d] for d in inc), []),
           "-c", src, "-o", str(tmp_path / "density.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_compiles_against_the_standin(lib_built, tmp_path):
    compile_demo(str(tmp_path / "demo"), [os.path.join(HERE, "cxx")])


@pytest.mark.gpu
@pytest.mark.parametrize("periodic", [0, 1])
def test_dropin_runs_like_the_reference(gpu, port_built, tmp_path, periodic):
    exe = str(tmp_path / "demo")
    compile_demo(exe, [os.path.join(HERE, "cxx")])
    n, box = 20000, 100.0
    pos, mass, vel = syn.clustered_box(n, box, seed=8, velocities=True)
    ll = syn.linking_length(n, box)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, periodic], np.int32).tofile(f)
        np.array([box, ll], np.float64).tofile(f)
        np.concatenate([pos, vel, mass[:, None]], 1).astype(np.float64).tofile(f)
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(out, "rb").read()
    off = 0

    def take(dt, cnt):
        nonlocal off
        a = np.frombuffer(raw, dt, cnt, off)
        off += a.nbytes
        return a

    n_, nodes, leaves, ngroup = take(np.int32, 4)
    group = take(np.int32, n)
    rho = take(np.float64, n)
    nnid = take(np.int32, n * 16).reshape(n, 16)
    d2 = take(np.float64, n * 16).reshape(n, 16)
    nb = take(np.int32, 1)[0]
    ball = take(np.int32, nb)
    rho_after = take(np.float64, n)
    smvel = take(np.float64, 3 * n).reshape(n, 3)
    ngroup_nn = take(np.int32, 1)[0]
    group_nn = take(np.int32, n)
    rho_smooth = take(np.float64, n)
    pnn = take(np.int32, n * 16).reshape(n, 16)
    pd2 = take(np.float64, n * 16).reshape(n, 16)
    prho = take(np.float64, n)
    pngroup = take(np.int32, 1)[0]
    pgroup = take(np.int32, n)
    posden = take(np.float64, 100)
    posvden = take(np.float64, 100)
    per = [box] * 3 if periodic else None
    o = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per, backend="port")
    assert nodes == o.num_nodes and leaves == o.num_leaves
    go, no = o.fof(ll, 20)
    assert ngroup == no
    assert_same_partition(group, go, "drop-in FOF")
    oi, od = o.knn(16, 0)
    assert_knn_equal(nnid, d2, oi, od, "drop-in FindNearest")
    ro = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per, backend="port").density(32)
    assert_density_close(rho, ro, "drop-in CalcDensity")
    assert_density_close(rho_after, ro, "input order restored by the destructor")
    np.testing.assert_array_equal(np.sort(ball), o.ball_tagged(0, 4 * ll * ll))
    # CalcSmoothVel with the stored densities (FP64 sums in another order: 1e-12 of the
    # largest magnitude)
    want = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per,
                             backend="port").smooth_vel_moments(0, 32, ro)
    assert np.max(np.abs(smvel - want)) <= 1e-12 * np.max(np.abs(want))
    # FOFNNCriterion over the FindNearest lists (the same lists in tree indices)
    pn, _ = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per, backend="port").tree_knn(16)
    gp, ngp = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per,
                                backend="port").fof_nn(0, [0, 0, 0, 0, 0, 0, 0.35, 0], pn, 5)
    assert ngroup_nn == ngp
    assert_same_partition(group_nn, gp, "drop-in FOFNNCriterion")
    # DensitySmooth(S, 16, 32): System constructor (default Epanechnikov kernel, no period)
    rs = oracle.OracleTree(pos, vel, mass, 16, 0, 2, 1000, None, backend="port").density(32)
    assert_density_close(rho_smooth, rs, "drop-in DensitySmooth")
    # phase-space tree with the local metric
    mk6 = lambda: oracle.OracleTree(pos, vel, mass, 16, 3, 0, 1000, per, backend="port",
                                    nthreads=8, aniso=0)
    oi, od = mk6().knn(16, 0)
    assert_knn_equal(pnn, pd2, oi, od, "drop-in phase-space FindNearest")
    assert_density_close(prho, mk6().density(16), "drop-in phase-space CalcDensity")
    g6, n6 = mk6().fof_criterion(2, [3, 0.25, 0.04, 0, 0, 0, 0.25, 0.04], 8, 0)
    assert pngroup == n6
    assert_same_partition(pgroup, g6, "drop-in phase-space FOFCriterion")
    # CalcDensityPosition / CalcVelDensityPosition next to the first 100 particles
    op = oracle.OracleTree(pos, vel, mass, 16, 0, 0, 1000, per, backend="port")
    assert_density_close(posden, [op.density_position(pos[i] + 0.01, 32) for i in range(100)],
                         "drop-in CalcDensityPosition")
    assert_density_close(posvden, [op.veldensity_position(pos[i] + 0.01, vel[i], 16, 32)
                                   for i in range(100)], "drop-in CalcVelDensityPosition")
