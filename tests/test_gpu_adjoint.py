"""GPU density adjoint: L = sum_i w_i log rho_i with rho from CalcDensity(32); gradients
with respect to positions and masses, neighbour sets and kernel-table cells frozen.
Checked against the CPU restatement of the same adjoint and against central finite
differences (step 1e-6) on 1000 random coordinates, at the 2^20 clustered size; and
used through a torch.autograd.Function (defined here, in the test harness only) whose
backward calls nbk_density_adjoint, for any upstream gradient of rho."""
import numpy as np
import pytest

import oracle
from nbodylib_gb300 import KDTree
from nbodylib_gb300 import synthetic as syn
from tests.helpers import assert_density_close

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-6        # relative error against central finite differences (Richardson)
FD_RTOL_PLAIN = 1e-4  # the plain step-1e-6 central difference (its O(h^2) term)
GRAD_RTOL = 1e-8      # GPU vs CPU restatement: summation order (atomics) and cancellation
FLOOR = 1e-3          # relative errors are taken against max(|g|, FLOOR * max|grad|)


def _rel(a, b, scale):
    return np.abs(a - b) / np.maximum(np.abs(b), scale)


def _fd_report(fd, g, scale):
    """(worst pure relative error where |g| >= scale, worst |fd - g| / scale elsewhere,
    number of coordinates with |g| >= scale)."""
    big = np.abs(g) >= scale
    pure = np.abs(fd[big] - g[big]) / np.abs(g[big])
    small = np.abs(fd[~big] - g[~big]) / scale
    return (pure.max() if pure.size else 0.0), (small.max() if small.size else 0.0), int(big.sum())


@pytest.mark.parametrize("n", [1 << 14, 1 << 20])
def test_adjoint_vs_restatement_and_finite_differences(gpu, port_built, n, record_property):
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
    scale = FLOOR * np.abs(gp).max()
    # central differences at step 1e-6: their O(h^2) truncation error reaches ~2e-5 on
    # coordinates near very close pairs (it quarters when the step halves), so the plain
    # check is 1e-4
    fd1 = o.local_fd(k, nn, w, coords, step=1e-6)
    pure1, small1, nbig = _fd_report(fd1, g, scale)
    assert max(pure1, small1) <= FD_RTOL_PLAIN, (pure1, small1)
    # Richardson extrapolation of the step-1e-6 and step-5e-7 central differences removes
    # the h^2 term: the 1e-6 bar
    fd2 = o.local_fd(k, nn, w, coords, step=5e-7)
    rich = (4 * fd2 - fd1) / 3
    pure, small, _ = _fd_report(rich, g, scale)
    record_property("fd_plain_worst_rel", float(pure1))
    record_property("fd_richardson_worst_rel", float(pure))
    record_property("fd_richardson_worst_below_floor", float(small))
    record_property("fd_coords_above_floor", nbig)
    print(f"n={n}: {nbig}/1000 coordinates with |g| >= {FLOOR} max|g|; worst relative error "
          f"there: plain {pure1:.2e}, Richardson {pure:.2e}; below the floor, worst "
          f"|fd - g| / floor: plain {small1:.2e}, Richardson {small:.2e}")
    assert pure <= FD_RTOL, pure
    assert small <= FD_RTOL, small


def _density_function():
    import torch

    class SPHDensity(torch.autograd.Function):
        """rho = CalcDensity(k) of a tree built on (pos, mass); the backward runs the
        hand-written adjoint (nbk_density_adjoint) with the neighbour sets of the forward.

        The adjoint returns the gradient of sum_i w_i log rho_i; for an upstream gradient
        g_i = dL/drho_i the weights w_i = g_i rho_i give sum_i g_i drho_i/d(pos, mass)."""

        @staticmethod
        def forward(ctx, pos, mass, k):
            t = KDTree(pos.detach().contiguous(), None, mass.detach().contiguous(), 16,
                       kerntype=0, device=True)
            rho = t.CalcDensity(k)
            t.sync()
            ctx.tree, ctx.k = t, k
            ctx.save_for_backward(rho)
            return rho

        @staticmethod
        def backward(ctx, grad_rho):
            (rho,) = ctx.saved_tensors
            w = (grad_rho * rho).contiguous()
            _, gp, gm = ctx.tree.DensityAdjoint(ctx.k, w)
            ctx.tree.sync()
            ctx.tree.close()
            return gp, gm, None

    return SPHDensity


def test_autograd_function_wraps_the_adjoint(gpu, port_built):
    import torch
    SPHDensity = _density_function()
    n, k = 1 << 14, 32
    pos, mass = syn.clustered_box(n, 100.0, seed=2)
    w = np.random.default_rng(5).normal(size=n)
    o = oracle.OracleTree(pos, None, mass, 16, 0, 0, 1000, None, backend="port", nthreads=16)
    rho_o, nn = o.density(k, return_nn=True)

    x = torch.tensor(pos, device="cuda", requires_grad=True)
    m = torch.tensor(mass, device="cuda", requires_grad=True)
    wt = torch.tensor(w, device="cuda")
    rho = SPHDensity.apply(x, m, k)
    assert_density_close(rho.detach().cpu().numpy(), rho_o, "autograd forward")
    # the loss the adjoint is written for: L = sum w log rho
    loss = (wt * torch.log(rho)).sum()
    gx, gm = torch.autograd.grad(loss, (x, m))
    _, gp_c, gm_c = o.density_adjoint(k, nn, w)
    gx, gm = gx.cpu().numpy(), gm.cpu().numpy()
    assert _rel(gx, gp_c, 1e-6 * np.abs(gp_c).max()).max() <= GRAD_RTOL
    assert _rel(gm, gm_c, 1e-6 * np.abs(gm_c).max()).max() <= GRAD_RTOL

    # any other upstream gradient: L2 = sum rho^2 (restatement weights 2 rho_i^2)
    rho = SPHDensity.apply(x, m, k)
    loss2 = (rho * rho).sum()
    gx2, gm2 = torch.autograd.grad(loss2, (x, m))
    _, gp_c2, gm_c2 = o.density_adjoint(k, nn, 2.0 * rho_o * rho_o)
    o.close()
    gx2, gm2 = gx2.cpu().numpy(), gm2.cpu().numpy()
    assert _rel(gx2, gp_c2, 1e-6 * np.abs(gp_c2).max()).max() <= GRAD_RTOL
    assert _rel(gm2, gm_c2, 1e-6 * np.abs(gm_c2).max()).max() <= GRAD_RTOL
