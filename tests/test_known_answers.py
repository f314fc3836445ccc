"""Hand-derived known answers on a cubic lattice (spacing 1, 12^3 particles at (i + 0.5)),
for the restatement (CPU) and the GPU path:

* FOF with ll just above the spacing links every particle into one group; just below it,
  none (periodic box of side 12, so every particle has six neighbours at distance 1);
* the squared distances of the nearest neighbours come in exact shells: 6 at 1, 12 at 2,
  8 at 3 (FindNearestPos, periodic, which keeps the particle itself at 0);
* CalcDensity(18) of a particle at least two spacings from the faces (CalcDensity ignores
  the period) is m h^-3 (6 W(sqrt 2) + 12 W(2)) with h = sqrt(2)/2, W the reference's
  table interpolation (KDCalcSmoothQuantities.cxx:12-15) — every neighbour pair is found
  from both ends with the same h, so the two half-weights add up;
* two particles at separation 0.75 are each other's nearest at d2 = 0.5625.
"""
import numpy as np
import pytest

import oracle

NS = 12


def lattice():
    g = (np.arange(NS) + 0.5).astype(np.float64)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    mass = np.full(len(pos), 0.25)
    return pos, mass


def wsm(q, table):
    kr = len(table)
    delta = 2.0 / (kr - 1)
    i = int(q * 0.5 * (kr - 1))
    if i < kr - 1:
        return table[i] + (table[i + 1] - table[i]) * (q - delta * i) / delta
    return table[i]


def interior(pos):
    return np.all((pos > 2.0) & (pos < NS - 2.0), axis=1)


def expected_density(table, m):
    h = 0.5 * np.sqrt(2.0)
    return m / h**3 * (6 * wsm(1.0 / h, table) + 12 * wsm(np.sqrt(2.0) / h, table))


def check_shells(d2):
    d2 = np.sort(np.asarray(d2), axis=1)
    np.testing.assert_array_equal(d2[:, 0], 0.0)  # FindNearestPos keeps the particle itself
    np.testing.assert_array_equal(d2[:, 1:7], 1.0)
    np.testing.assert_array_equal(d2[:, 7:19], 2.0)
    np.testing.assert_array_equal(d2[:, 19:27], 3.0)


def test_port_lattice_known_answers(port_built):
    pos, mass = lattice()
    per = [float(NS)] * 3
    mk = lambda p=per: oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, p, backend="port",
                                         nthreads=4)
    g, ng = mk().fof(1.01, 2)
    assert ng == 1 and np.all(g == 1)
    g, ng = mk().fof(0.99, 2)
    assert ng == 0 and np.all(g == 0)
    nn, d2 = mk().knn(27, method=1)
    check_shells(d2)
    t = mk(None)
    rho = t.density(18)
    want = expected_density(t.kernel_table(), 0.25)
    sel = interior(pos)
    assert np.max(np.abs(rho[sel] - want)) <= 1e-12 * want


def test_port_two_particles(port_built):
    pos = np.array([[0.25, 0.5, 0.5], [1.0, 0.5, 0.5]])
    nn, d2 = oracle.OracleTree(pos, None, None, 16, 0, 0, 1000, None, backend="port").knn(1)
    np.testing.assert_array_equal(nn[:, 0], [1, 0])
    np.testing.assert_array_equal(d2[:, 0], [0.5625, 0.5625])


@pytest.mark.gpu
def test_gpu_lattice_known_answers(gpu):
    from nbodylib_gb300 import KDTree
    from nbodylib_gb300.kdtree import KSPH
    pos, mass = lattice()
    per = [float(NS)] * 3
    t = KDTree(pos, None, mass, 16, kerntype=KSPH, period=per)
    g, ng = t.FOF(1.01, 2)
    assert ng == 1 and np.all(np.asarray(g) == 1)
    g, ng = t.FOF(0.99, 2)
    assert ng == 0 and np.all(np.asarray(g) == 0)
    nn, d2 = t.FindNearestPos(27)
    check_shells(d2)
    t.close()
    t = KDTree(pos, None, mass, 16, kerntype=KSPH)
    rho = np.asarray(t.CalcDensity(18))
    table, _ = t.GetKernel()
    want = expected_density(table, 0.25)
    sel = interior(pos)
    assert np.max(np.abs(rho[sel] - want)) <= 1e-12 * want
    t.close()


@pytest.mark.gpu
def test_gpu_two_particles(gpu):
    from nbodylib_gb300 import KDTree
    pos = np.array([[0.25, 0.5, 0.5], [1.0, 0.5, 0.5]])
    t = KDTree(pos, None, None, 16)
    nn, d2 = t.FindNearest(1)
    perm = np.asarray(t.GetPerm())
    np.testing.assert_array_equal(np.sort(perm[np.asarray(nn)[:, 0]]), [0, 1])
    np.testing.assert_array_equal(np.asarray(d2)[:, 0], [0.5625, 0.5625])
    t.close()
