"""Solve adjoint: dL/dB = A^-T W, dL/dA = -(A^-T W) X^T for L = sum(W . X),
X = A^-1 B, n = 2048, 64 right-hand sides, cond_1(A) ~ 1e3."""
import numpy as np
import pytest

from helpers import rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu

N, NRHS = 2048, 64
# A = G + s I with G ~ N(0,1) (seed 5): s = 1.4204 sqrt(n) gives a LAPACK
# 1-norm condition estimate of 1.0e3 (bisection on the shift; the 2-norm
# condition is ~12 because ||A||_1 ~ n).
SHIFT = 1.420379516437606 * np.sqrt(N)


def problem():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((N, N)) + SHIFT * np.eye(N)
    b = rng.standard_normal((N, NRHS))
    w = rng.standard_normal((N, NRHS))
    return a, b, w


def test_backward_matches_tmv_transpose_solve(dev, orc):
    import torch

    from tmv_gb300.adjoint import lu_solve

    a, b, w = problem()
    A = to_dev(a, dev, "F").requires_grad_(True)
    B = to_dev(b, dev, "F").requires_grad_(True)
    W = to_dev(w, dev, "F")
    X = lu_solve(A, B)
    L = (W * X).sum()
    L.backward()
    torch.cuda.synchronize()
    # TMV: X = B/A, Gt = W^T % A (LU_RDivEq), gA = -Gt^T X^T
    x_o, lu_o, p_o = orc.divide(np.asfortranarray(a), np.asfortranarray(b))
    gt = np.asfortranarray(w.T.copy())
    orc.rdiveq(lu_o, p_o, gt)
    gB_o = gt.T
    gA_o = np.zeros((N, N), order="F")
    orc.multmm(False, -1.0, np.asfortranarray(gB_o), np.ascontiguousarray(x_o.T), gA_o)
    assert rel_frob(to_host(X.detach()), x_o) <= 1e-12
    assert rel_frob(to_host(B.grad), gB_o) <= 1e-12
    assert rel_frob(to_host(A.grad), gA_o) <= 1e-12


def test_central_finite_differences(dev):
    import torch

    from tmv_gb300 import linalg
    from tmv_gb300.adjoint import lu_solve

    a, b, w = problem()
    A = to_dev(a, dev, "F").requires_grad_(True)
    B = to_dev(b, dev, "F").requires_grad_(True)
    W = to_dev(w, dev, "F")
    L = (W * lu_solve(A, B)).sum()
    L.backward()
    gA, gB = to_host(A.grad), to_host(B.grad)

    def loss(aa, bb):
        X, _, _ = linalg.divide(aa, bb)
        return float((W * X).sum())

    h = 1e-6
    rng = np.random.default_rng(55)
    Ad, Bd = to_dev(a, dev, "F"), to_dev(b, dev, "F")
    worst = 0.0
    for which, grad, base in (("A", gA, Ad), ("B", gB, Bd)):
        rows = rng.integers(0, N, 64)
        cols = rng.integers(0, base.shape[1], 64)
        for i, j in zip(rows, cols):
            orig = base[i, j].item()
            base[i, j] = orig + h
            lp = loss(Ad, Bd)
            base[i, j] = orig - h
            lm = loss(Ad, Bd)
            base[i, j] = orig
            fd = (lp - lm) / (2 * h)
            # rounding of L (|L| ~ 10, relative ~1e-15) over 2h bounds the
            # finite-difference error by ~1e-8; the O(h^2) term is smaller
            err = abs(fd - grad[i, j])
            assert err <= 1e-7 + 1e-5 * abs(grad[i, j]), (which, i, j, fd, grad[i, j])
            worst = max(worst, err)
    assert worst < 1e-7
