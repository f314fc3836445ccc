"""GPU density adjoint: L = sum_i w_i log rho_i with rho from CalcDensity(32); gradients
with respect to positions and masses, neighbour sets and kernel-table cells frozen.
Checked against the CPU restatement of the same adjoint and against central finite
differences (step 1e-6) on 1000 random coordinates, at the 2^20 clustered size."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree
from nbodylib_gb300 import synthetic as syn
from tests.helpers import assert_density_close

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-6      # relative error against central finite differences
GRAD_RTOL = 1e-8    # GPU vs CPU restatement: summation order (atomics) and cancellation


def _rel(a, b, scale):
    return np.abs(a - b) / np.maximum(np.abs(b), scale)


@pytest.mark.parametrize("n", [1 << 14, 1 << 20])
def test_adjoint_vs_restatement_and_finite_differences(gpu, port_built, n):
    k = 32
    pos, mass = syn.clustered_box(n, 100.0, seed=2)
    w = np.random.default_rng(5).normal(size=n)
    t = KDTree(pos, None, mass, 16, kerntype=0)
    rho, gp, gm = t.DensityAdjoint(k, w)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, None, backend="port", nthreads=16)
    rho_o, nn = o.density(k, return_nn=True)
    assert_density_close(rho, rho_o, "forward rho")
    rho_c, gp_c, gm_c = o.density_adjoint(k, nn, w)
    sp = 1e-6 * np.abs(gp_c).max()
    sm = 1e-6 * np.abs(gm_c).max()
    assert _rel(gp, gp_c, sp).max() <= GRAD_RTOL
    assert _rel(gm, gm_c, sm).max() <= GRAD_RTOL
    rng = np.random.default_rng(6)
    coords = np.stack([rng.integers(0, n, 1000), rng.integers(0, 3, 1000)], 1)
    g = gp[coords[:, 0], coords[:, 1]]
    scale = 1e-3 * np.abs(gp).max()
    # central differences at step 1e-6: their O(h^2) truncation error reaches ~2e-5 on
    # coordinates near very close pairs (it quarters when the step halves), so the plain
    # check is 1e-4
    fd1 = o.local_fd(k, nn, w, coords, step=1e-6)
    assert _rel(fd1, g, scale).max() <= 100 * FD_RTOL
    # Richardson extrapolation of the step-1e-6 and step-5e-7 central differences removes
    # the h^2 term: the 1e-6 bar
    fd2 = o.local_fd(k, nn, w, coords, step=5e-7)
    rich = (4 * fd2 - fd1) / 3
    rel = _rel(rich, g, scale)
    assert rel.max() <= FD_RTOL, rel.max()
