"""Mixed-precision LU + FP64 iterative refinement against the FP64 oracle."""
import numpy as np
import pytest

from helpers import diag_shift_matrix, rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu


def haar(n, cond, seed):
    """A = U diag(s) V^T, U, V Haar (Q of QR of a seeded Gaussian, sign-fixed),
    s log-spaced from 1 to 1/cond."""
    rng = np.random.default_rng(seed)
    qs = []
    for _ in range(2):
        q, r = np.linalg.qr(rng.standard_normal((n, n)))
        qs.append(q * np.sign(np.diag(r))[None, :])
    s = np.logspace(0, -np.log10(cond), n)
    return (qs[0] * s[None, :]) @ qs[1].T, rng.standard_normal(n)


def backward_error(a, x, b):
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


@pytest.mark.parametrize("cond", [1e2, 1e4, 1e6])
def test_haar_converges_to_1e12(dev, orc, cond):
    from tmv_gb300 import linalg

    n = 1024
    a, b = haar(n, cond, seed=31)
    X, info = linalg.solve_mixed(to_dev(a, dev, "F"), to_dev(b.reshape(n, 1), dev, "F"),
                                 max_iter=10, tol=1e-12)
    x = to_host(X)[:, 0]
    assert info.converged == 1 and info.iterations <= 10
    assert info.backward_error <= 1e-12
    assert backward_error(a, x, b) <= 1e-12
    # ||A||_inf of the stopping test: FP32 row sums scaled down by
    # (1 - 2^-12), never above the FP64 value and within 5e-4 of it
    norm = np.abs(a).sum(axis=1).max()
    assert norm * (1 - 5e-4) <= info.anorm_inf <= norm * (1 + 1e-12)
    # forward difference from TMV's FP64 LU solution: bounded by the
    # condition number times the backward errors of the two solutions
    x_o, _, _ = orc.divide(np.asfortranarray(a), b.reshape(n, 1))
    eps = np.finfo(float).eps
    assert rel_frob(x, x_o[:, 0]) <= 50 * cond * (info.backward_error + eps)


def test_large_entries_norm_stays_finite(dev):
    # entries near the FP32 limit: each converts to FP32, but a row's sum of
    # |a| overflows FP32, so ||A||_inf for the stopping test must come out of
    # an FP64 sum
    from tmv_gb300 import linalg

    n = 512
    a, b = haar(n, 1e2, seed=35)
    a = a * (1e37 / np.abs(a).max())
    assert np.abs(a).sum(axis=1).max() > np.finfo(np.float32).max
    b = b * 1e37
    X, info = linalg.solve_mixed(to_dev(a, dev, "F"), to_dev(b.reshape(n, 1), dev, "F"),
                                 max_iter=10, tol=1e-12, raise_not_converged=False)
    x = to_host(X)[:, 0]
    norm = np.abs(a).sum(axis=1).max()
    assert np.isfinite(info.anorm_inf) and abs(info.anorm_inf - norm) <= 1e-3 * norm
    # no convergence claimed at the start (an infinite norm would give a zero
    # backward error there); the FP32 factor may itself overflow at this
    # scale, which the refinement reports as not converged
    assert info.iterations >= 1
    if info.converged:
        assert backward_error(a, x, b) <= 1e-12
    else:
        assert not info.backward_error <= 1e-12


@pytest.mark.parametrize("cond", [1e4, 1e6])
def test_refines_to_fp64_lu_accuracy(dev, orc, cond):
    # with a tolerance at FP64 level the refined solution is as accurate as
    # TMV's FP64 LU solve
    from tmv_gb300 import linalg

    n = 1024
    a, b = haar(n, cond, seed=32)
    X, info = linalg.solve_mixed(to_dev(a, dev, "F"), to_dev(b.reshape(n, 1), dev, "F"),
                                 max_iter=40, tol=4e-16)
    assert info.converged == 1
    x = to_host(X)[:, 0]
    x_o, _, _ = orc.divide(np.asfortranarray(a), b.reshape(n, 1))
    assert rel_frob(x, x_o[:, 0]) <= 50 * cond * np.finfo(float).eps


def test_diag_shifted_two_steps(dev, orc):
    from tmv_gb300 import linalg

    rng = np.random.default_rng(8)
    n = 2000
    a = diag_shift_matrix(rng, n, 4 * np.sqrt(n))
    b = rng.standard_normal((n, 3))
    X, info = linalg.solve_mixed(to_dev(a, dev, "F"), to_dev(b, dev, "F"))
    x_o, _, _ = orc.divide(np.asfortranarray(a), np.asfortranarray(b))
    assert info.converged == 1 and info.iterations <= 3
    assert rel_frob(to_host(X), x_o) <= 1e-12


def test_not_converged_status(dev):
    from tmv_gb300 import TmvgError, linalg

    n = 512
    a, b = haar(n, 1e6, seed=5)
    A = to_dev(a, dev, "F")
    B = to_dev(b.reshape(n, 1), dev, "F")
    with pytest.raises(TmvgError) as ei:
        linalg.solve_mixed(A, B, max_iter=0, tol=1e-12)
    assert ei.value.status == 2
    X, info = linalg.solve_mixed(A, B, max_iter=0, tol=1e-12, raise_not_converged=False)
    assert info.converged == 0 and info.iterations == 0 and info.backward_error > 1e-12
    # the same handle still works and converges with the default budget
    X, info = linalg.solve_mixed(A, B)
    assert info.converged == 1


def test_full_size_8192_cond1e6(dev):
    # The headline workload: n = 8192, cond = 1e6, one right-hand side.
    import torch

    from tmv_gb300 import linalg

    n, cond = 8192, 1e6
    rng = np.random.default_rng(3)
    qs = []
    for _ in range(2):
        g = torch.from_numpy(rng.standard_normal((n, n))).to(dev)
        q, r = torch.linalg.qr(g)
        qs.append(q * torch.sign(torch.diagonal(r)).unsqueeze(0))
        del g, r
    s = torch.logspace(0, -np.log10(cond), n, dtype=torch.float64, device=dev)
    A = linalg.colmajor((qs[0] * s.unsqueeze(0)) @ qs[1].t())
    del qs
    b = torch.from_numpy(rng.standard_normal((n, 1))).to(dev)
    X, info = linalg.solve_mixed(A, b, max_iter=10, tol=1e-12)
    assert info.converged == 1 and info.iterations <= 10
    r = b - A @ X
    berr = float(r.abs().max() / (A.abs().sum(dim=1).max() * X.abs().max() + b.abs().max()))
    assert berr <= 1e-12
    # against the plain FP64 GPU LU solution of the same system
    X64, _, _ = linalg.divide(A, b)
    fe = float((X - X64).norm() / X64.norm())
    assert fe <= 50 * cond * (info.backward_error + np.finfo(float).eps)


@pytest.mark.parametrize("n", [512, 500])
def test_zero_column_reports_singular(dev, n):
    # a zero column of A gives the FP32 factor an exact zero U(j,j); the
    # refinement's triangular solve meets it in a diagonal block (the
    # substitution branch of both solve forms: n = 512 streams whole 128-row
    # blocks, n = 500 takes the register form) and the call reports SINGULAR,
    # as TMV's solve throws on a singular U; the handle stays usable
    from tmv_gb300 import TmvgError, linalg

    a, b = haar(n, 1e2, seed=41)
    a[:, 300] = 0.0
    A = to_dev(a, dev, "F")
    B = to_dev(b.reshape(n, 1), dev, "F")
    with pytest.raises(TmvgError) as ei:
        linalg.solve_mixed(A, B, max_iter=3, tol=1e-12)
    assert ei.value.status == 1
    a2, b2 = haar(n, 1e2, seed=42)
    X, info = linalg.solve_mixed(to_dev(a2, dev, "F"), to_dev(b2.reshape(n, 1), dev, "F"))
    assert info.converged == 1 and backward_error(a2, to_host(X)[:, 0], b2) <= 1e-14
