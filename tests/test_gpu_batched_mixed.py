"""Batched uneven solves with FP32 factors and FP64 refinement.

tmvg_batched_lu_solve_mixed_f64: each system's FP32 LU (pivots chosen by
FP64 comparisons) and FP64 residual refinement in one persistent launch.
Checked against TMV's own FP64 solutions (tests/golden/batched_small.npz)
and the oracle's FP64 LU solutions: every column's normwise backward error
<= tol, and the solution within 1e-12 (relative, per system) of the FP64
one for these well-conditioned systems (2 sqrt(n) on the diagonal).
"""
from pathlib import Path

import numpy as np
import pytest

from test_gpu_batched import make_batch

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def run_mixed(dev, n, r, A, B, max_iter=10, tol=1e-12):
    import torch

    from tmv_gb300.batched import BatchPlan

    plan = BatchPlan(n, r, tune=False)
    dA = torch.from_numpy(A.copy()).to(dev)
    dB = torch.from_numpy(B.copy()).to(dev)
    P, st, it, be = plan.solve_mixed(dA, dB, max_iter=max_iter, tol=tol)
    torch.cuda.synchronize()
    out = (dA.cpu().numpy(), dB.cpu().numpy(), P.cpu().numpy(), st.cpu().numpy(), it.cpu().numpy(),
           be.cpu().numpy())
    plan.close()
    return out


def backward_errors(n, r, a_off, b_off, A, B, X):
    worst = []
    for s in range(len(n)):
        ns, rs = int(n[s]), int(r[s])
        if rs == 0:
            worst.append(0.0)
            continue
        a = A[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F")
        b = B[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
        x = X[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
        res = np.abs(b - a @ x).max(axis=0)
        den = np.abs(a).sum(axis=1).max() * np.abs(x).max(axis=0) + np.abs(b).max(axis=0)
        worst.append(float((res / den).max()))
    return np.array(worst)


def test_golden_batch_matches_tmv(dev):
    g = np.load(GOLD / "batched_small.npz")
    A0 = g["A"]
    LUa, X, P, st, it, be = run_mixed(dev, g["n"], g["nrhs"], A0, g["B"], tol=1e-14)
    assert not st.any()
    assert np.array_equal(LUa, A0), "A must not be modified"
    assert np.abs(X - g["X"]).max() <= 1e-12 * np.abs(g["X"]).max()


def test_random_batch_vs_oracle(dev, orc):
    rng = np.random.default_rng(77)
    n, r, a_off, b_off, A, B = make_batch(rng, 300, 1, 256, 0, 16, shift=2.0)
    _, X, P, st, it, be = run_mixed(dev, n, r, A, B, tol=1e-12)
    assert not st.any()
    assert be.max() <= 1e-12
    assert it.max() <= 4
    # the backward errors recomputed on the host agree with the reported ones
    host_be = backward_errors(n, r, a_off, b_off, A, B, X)
    assert host_be.max() <= 2e-12
    for s in range(len(n)):
        ns, rs = int(n[s]), int(r[s])
        if rs == 0:
            continue
        a = A[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F")
        b = B[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
        x_o, _, _ = orc.divide(np.asfortranarray(a), np.asfortranarray(b))
        x = X[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
        assert np.abs(x - x_o).max() <= 1e-12 * max(np.abs(x_o).max(), 1e-300), s


def test_edges_not_converged_singular_and_replay(dev):
    rng = np.random.default_rng(3)
    n, r, a_off, b_off, A, B = make_batch(rng, 40, 1, 64, 1, 4, shift=2.0)
    # max_iter = 0: no correction applied, x = 0, status 2
    _, X0, _, st0, it0, _ = run_mixed(dev, n, r, A, B, max_iter=0)
    assert (st0 == 2).all() and not X0.any() and not it0.any()
    # a zero column in system 5: its FP32 U has an exact zero pivot
    A2 = A.copy()
    s = 5
    ns = int(n[s])
    col = a_off[s] + 2 * ns if ns > 2 else a_off[s]
    A2[col:col + ns] = 0.0
    _, X2, _, st2, _, _ = run_mixed(dev, n, r, A2, B)
    assert st2[s] == 1
    others = np.arange(len(n)) != s
    assert not st2[others].any()
    # the same launch twice: identical results
    _, Xa, _, sa, ia, ba = run_mixed(dev, n, r, A, B)
    _, Xb, _, sb, ib, bb = run_mixed(dev, n, r, A, B)
    assert np.array_equal(Xa, Xb) and np.array_equal(ia, ib)
