"""The whole batched workload (20000 systems, n ~ U{8..256}, nrhs ~ U{1..16},
A_i ~ N(0,1) + 2 sqrt(n_i) I, B_i ~ N(0,1)) against the oracle, system by
system: the FP64 kernel's pivot vectors are TMV's (LU_Decompose of each
system) and its solutions are within 1e-12 of TMV's B_i / A_i (relative to
the system's largest |x|); the FP32-refined kernel's solutions are within
the same bound of TMV's and every column's backward error is at most 1e-12.
The inputs are generated here with numpy (seeded) in the workload's layout
(column-major blocks packed in order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUNT = 20000


def workload(seed=4):
    rng = np.random.default_rng(seed)
    n = rng.integers(8, 257, size=COUNT).astype(np.int64)
    r = rng.integers(1, 17, size=COUNT).astype(np.int64)
    a_off = np.concatenate([[0], np.cumsum(n * n)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(n * r)[:-1]]).astype(np.int64)
    A = rng.standard_normal(int((n * n).sum()))
    B = rng.standard_normal(int((n * r).sum()))
    for s in range(COUNT):  # + 2 sqrt(n) on the diagonal
        A[a_off[s] + np.arange(n[s]) * (n[s] + 1)] += 2.0 * np.sqrt(n[s])
    return n, r, a_off, b_off, A, B


def per_system_max(v, off, sizes):
    """max over each system's slice [off, off + size) of v."""
    return np.maximum.reduceat(v, off) if np.all(sizes > 0) else None


@pytest.fixture(scope="module")
def full(orc):
    n, r, a_off, b_off, A, B = workload()
    Xo = B.copy()
    assert not orc.batched_divide(n, r, a_off, b_off, A.copy(), Xo).any()
    return n, r, a_off, b_off, A, B, Xo


def check_solutions(X, Xo, b_off, n, r):
    diff = per_system_max(np.abs(X - Xo), b_off, n * r)
    scale = np.maximum(per_system_max(np.abs(Xo), b_off, n * r), 1.0)
    worst = int(np.argmax(diff / scale))
    assert (diff <= 1e-12 * scale).all(), f"system {worst}: {diff[worst] / scale[worst]:.2e}"


def test_full_batch_fp64_pivots_and_solutions(dev, orc, full):
    import torch

    from tmv_gb300.batched import BatchPlan

    n, r, a_off, b_off, A, B, Xo = full
    plan = BatchPlan(n, r, tune=True)
    dA = torch.from_numpy(A).to(dev)
    dB = torch.from_numpy(B).to(dev)
    P, st = plan.solve(dA, dB)
    torch.cuda.synchronize()
    X, Pg, st = dB.cpu().numpy(), P.cpu().numpy(), st.cpu().numpy()
    plan.close()
    del dA, dB
    assert not st.any()
    check_solutions(X, Xo, b_off, n, r)
    # every system's pivot vector is TMV's
    p_off = np.concatenate([[0], np.cumsum(n)[:-1]])
    for s in range(COUNT):
        ns = int(n[s])
        lu = A[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F").copy(order="F")
        p_o = orc.lu_decompose(lu)
        assert np.array_equal(Pg[p_off[s]:p_off[s] + ns], p_o), s


def test_full_batch_fp32_refined(dev, full):
    import torch

    from tmv_gb300.batched import BatchPlan

    n, r, a_off, b_off, A, B, Xo = full
    plan = BatchPlan(n, r, tune=True)
    dA = torch.from_numpy(A).to(dev)
    dB = torch.from_numpy(B).to(dev)
    P, st, iters, berr = plan.solve_mixed(dA, dB, max_iter=10, tol=1e-12)
    torch.cuda.synchronize()
    X = dB.cpu().numpy()
    st, berr = st.cpu().numpy(), berr.cpu().numpy()
    plan.close()
    assert not st.any()
    assert berr.max() <= 1e-12
    check_solutions(X, Xo, b_off, n, r)
