"""The batched band LU (tmv_gb300/csrc/band.cu) against the oracle's
restatement of TMV's band LU (pinned to TMV bit for bit by
test_band_oracle.py): for every shape class of the kernel (the tridiagonal
algorithm, the three register-window capacities and the wide kernel) the
pivots, every band slot of the factors (signed zeros and NaNs included), the
solutions and the singular status are the oracle's bit for bit.  Fill
diagonals hold NaN on input (they are outputs, never read) and the gap slots
of a wider ldab keep their contents.  At the benchmark's size the whole batch
is checked by residual and a sample of systems bit for bit."""
import numpy as np
import pytest

import oracle
from tests.helpers import band_matrix, band_pack, bits

pytestmark = pytest.mark.gpu

# (lo, hi, algo): tridiagonal algorithm, register classes (1,2), (2,4), (4,8), wide kernel
SHAPES = [(1, 1, "tridiag"), (0, 0, "general"), (0, 2, "general"), (1, 0, "general"),
          (1, 1, "general"), (2, 1, "general"), (1, 3, "general"), (2, 2, "general"),
          (2, 6, "general"), (3, 3, "general"), (4, 4, "general"), (5, 3, "general"),
          (7, 7, "general")]
ALGO = {"general": 0, "tridiag": 1}


def make_batch(rng, count, n, lo, hi, kind, nrhs, ldab=None):
    from tmv_gb300.band import band_layout

    lay = band_layout(n, lo, hi, ldab=ldab)
    ab = np.full(count * lay.stride_ab, np.nan)
    mats = []
    for s in range(count):
        a = band_matrix(rng, n, lo, hi, kind)
        band_pack(a, lo, hi, lay.ldab, out=ab[s * lay.stride_ab:(s + 1) * lay.stride_ab])
        mats.append(a)
    B = rng.standard_normal(count * n * nrhs)
    B[rng.random(B.size) < 0.15] = 0.0
    return lay, ab, B


def slots(lay):
    n, lo, hu, ld = lay.n, lay.lo, lay.hu, lay.ldab
    return np.array([i + j * ld for j in range(n) for i in range(max(0, j - hu), min(n, j + lo + 1))],
                    dtype=np.int64)


def oracle_batch(orc, lay, ab, B, count, nrhs, algo):
    """Per system: factors (in a copy of ab), P, status, X (in a copy of B)."""
    ab, X = ab.copy(), B.copy()
    n = lay.n
    P = np.zeros((count, n), dtype=np.int64)
    st = np.zeros(count, dtype=np.int32)
    for s in range(count):
        sys_ab = ab[s * lay.stride_ab:(s + 1) * lay.stride_ab]
        P[s] = orc.band_lu_decompose(sys_ab, n, lay.lo, lay.hi, lay.ldab, ALGO[algo])
        Xs = X[s * n * nrhs:(s + 1) * n * nrhs].reshape(nrhs, n).T  # column-major view
        try:
            orc.band_lu_ldiveq(sys_ab, n, lay.lo, lay.hi, lay.ldab, P[s], Xs, ALGO[algo], ldb=n)
        except oracle.OracleSingular:
            st[s] = 1
    return ab, P, st, X


def gpu_batch(dev, lay, ab, B, count, nrhs, algo):
    import torch

    from tmv_gb300.band import band_lu_solve

    dab = torch.from_numpy(ab).to(dev)
    dB = torch.from_numpy(B).to(dev)
    P, st = band_lu_solve(dab, count, lay, dB, nrhs, algo=algo)
    torch.cuda.synchronize()
    return dab.cpu().numpy(), P.cpu().numpy().reshape(count, -1)[:, :lay.n], st.cpu().numpy(), \
        dB.cpu().numpy()


def compare(lay, count, nrhs, gpu, ref, ab_in):
    g_ab, g_P, g_st, g_X = gpu
    o_ab, o_P, o_st, o_X = ref
    n = lay.n
    assert np.array_equal(g_P, o_P)
    assert np.array_equal(g_st, o_st)
    sl = slots(lay)
    for s in range(count):
        base = s * lay.stride_ab
        assert np.array_equal(bits(g_ab[base + sl]), bits(o_ab[base + sl])), f"system {s} factors"
        # every other slot of the system's stride keeps its input
        rest = np.setdiff1d(np.arange(lay.stride_ab), sl) + base
        assert np.array_equal(bits(g_ab[rest]), bits(ab_in[rest])), f"system {s} gap slots"
        if o_st[s] == 0:
            xs = slice(s * n * nrhs, (s + 1) * n * nrhs)
            assert np.array_equal(bits(g_X[xs]), bits(o_X[xs])), f"system {s} solution"


@pytest.mark.parametrize("lo,hi,algo", SHAPES)
@pytest.mark.parametrize("kind", ["normal", "int", "tiny"])
def test_band_matches_oracle_bitwise(dev, orc, lo, hi, algo, kind):
    rng = np.random.default_rng(100 + 10 * lo + hi)
    count, nrhs = 37, 2
    for n in [1, 2, 3, 8, 65, 300]:
        if lo > n - 1 or hi > n - 1:
            continue
        lay, ab, B = make_batch(rng, count, n, lo, hi, kind, nrhs)
        ref = oracle_batch(orc, lay, ab, B, count, nrhs, algo)
        gpu = gpu_batch(dev, lay, ab, B, count, nrhs, algo)
        compare(lay, count, nrhs, gpu, ref, ab)


def test_band_wider_ldab_and_singular(dev, orc):
    rng = np.random.default_rng(7)
    count, n, lo, hi, nrhs = 20, 40, 2, 3, 3
    lay, ab, B = make_batch(rng, count, n, lo, hi, "normal", nrhs, ldab=11)
    # zero columns in some systems: the underflow branch, then a singular solve
    for s in (3, 9):
        for i in range(max(0, 17 - hi), min(n, 17 + lo + 1)):
            ab[s * lay.stride_ab + i + 17 * lay.ldab] = 0.0
    ref = oracle_batch(orc, lay, ab, B, count, nrhs, "general")
    assert ref[2][3] == 1 and ref[2][9] == 1
    gpu = gpu_batch(dev, lay, ab, B, count, nrhs, "general")
    compare(lay, count, nrhs, gpu, ref, ab)


def test_band_decompose_then_ldiveq_equals_fused(dev):
    import torch

    from tmv_gb300.band import band_lu_decompose, band_lu_ldiveq

    rng = np.random.default_rng(8)
    for lo, hi, algo in [(1, 1, "tridiag"), (2, 2, "general"), (6, 2, "general")]:
        count, n, nrhs = 50, 77, 3
        lay, ab, B = make_batch(rng, count, n, lo, hi, "normal", nrhs)
        f_ab, f_P, f_st, f_X = gpu_batch(dev, lay, ab, B, count, nrhs, algo)
        dab = torch.from_numpy(ab).to(dev)
        dB = torch.from_numpy(B).to(dev)
        P = torch.empty(count * n, dtype=torch.int64, device=dev)
        band_lu_decompose(dab, count, lay, P, algo=algo)
        st = band_lu_ldiveq(dab, count, lay, P, dB, nrhs, algo=algo)
        torch.cuda.synchronize()
        assert np.array_equal(bits(dab.cpu().numpy()), bits(f_ab))
        assert np.array_equal(P.cpu().numpy().reshape(count, n), f_P)
        assert np.array_equal(st.cpu().numpy(), f_st)
        assert np.array_equal(bits(dB.cpu().numpy()), bits(f_X))


def test_band_interchange_outside_band_is_reported(dev):
    import torch

    from tmv_gb300.band import band_lu_decompose, band_lu_ldiveq

    rng = np.random.default_rng(9)
    for lo, hi in [(2, 1), (6, 6)]:  # register and wide kernels
        count, n = 4, 30
        lay, ab, B = make_batch(rng, count, n, lo, hi, "normal", 1)
        dab = torch.from_numpy(ab).to(dev)
        P = torch.empty(count * n, dtype=torch.int64, device=dev)
        band_lu_decompose(dab, count, lay, P)
        P[1 * n + 5] = 5 + lo + 1  # beyond the band
        P[2 * n + 7] = 3           # above the diagonal
        st = band_lu_ldiveq(dab, count, lay, P, torch.from_numpy(B).to(dev), 1)
        assert st.cpu().tolist() == [0, 2, 2, 0]


def test_band_one_by_one_row_rhs(dev, orc):
    """A 1 x nrhs B with ldb == 1 is row-major to TMV (a reciprocal scaling)."""
    import torch

    from tmv_gb300.band import band_layout, band_lu_solve

    lay = band_layout(1, 0, 0)
    for d in [3.0, 0.0]:
        ab = np.array([d])
        B = np.array([1.0, -2.0, 7.0])
        o_ab = ab.copy()
        o_P = orc.band_lu_decompose(o_ab, 1, 0, 0, 1)
        Xo = B.copy().reshape(1, 3, order="F")
        try:
            orc.band_lu_ldiveq(o_ab, 1, 0, 0, 1, o_P, Xo, ldb=1)
            o_st = 0
        except oracle.OracleSingular:
            o_st = 1
        dab, dB = torch.tensor(ab, device=dev), torch.tensor(B, device=dev)
        P, st = band_lu_solve(dab, 1, lay, dB, 3, ldb=1, stride_b=3)
        assert int(st.item()) == o_st
        if o_st == 0:
            assert np.array_equal(bits(dB.cpu().numpy()), bits(Xo.ravel(order="F")))


def test_band_rejects_bad_arguments(dev):
    import torch

    from tmv_gb300._lib import TmvgError
    from tmv_gb300.band import band_layout, band_lu_solve

    ab = torch.zeros(1000, dtype=torch.float64, device=dev)
    B = torch.zeros(100, dtype=torch.float64, device=dev)
    with pytest.raises(TmvgError):  # ldab < lo + hu
        band_lu_solve(ab, 2, band_layout(10, 2, 2, ldab=3), B, 1)
    with pytest.raises(TmvgError):  # the tridiagonal algorithm is lo == hi == 1 only
        band_lu_solve(ab, 2, band_layout(10, 2, 1), B, 1, algo="tridiag")
    with pytest.raises(TmvgError):  # overlapping systems
        band_lu_solve(ab, 2, band_layout(10, 1, 1, stride_ab=5), B, 1)
    with pytest.raises(TmvgError):  # lo >= n
        band_lu_solve(ab, 1, band_layout(3, 3, 0), B, 1)


def band_matvec(ab, lay, count, x):
    """y = A x for every system of the (unfactored) band batch, on the GPU."""
    import torch

    n, ld = lay.n, lay.ldab
    A = ab.view(count, lay.stride_ab)
    y = torch.zeros(count, n, dtype=torch.float64, device=ab.device)
    for d in range(-lay.lo, lay.hi + 1):
        i = torch.arange(max(0, -d), min(n, n - d), device=ab.device)
        y[:, i] += A[:, i * (ld + 1) + d * ld] * x[:, i + d]
    return y


@pytest.mark.parametrize("lo,hi,algo", [(1, 1, "tridiag"), (2, 2, "general")])
def test_band_benchmark_size(dev, orc, lo, hi, algo):
    """The benchmark's batch (65536 systems of n = 1024, one right-hand side,
    N(0,1) entries with lo + hi + 2 added to the diagonal): all statuses 0,
    every system's normwise backward error at most 1e-14, and 24 sampled
    systems bit for bit against the oracle."""
    import torch

    from tmv_gb300.band import band_layout, band_lu_solve

    count, n = 65536, 1024
    lay = band_layout(n, lo, hi)
    g = torch.Generator(device=dev).manual_seed(5)
    ab0 = torch.randn(count * lay.stride_ab, dtype=torch.float64, device=dev, generator=g)
    A = ab0.view(count, lay.stride_ab)
    i = torch.arange(n, device=dev)
    A[:, i * (lay.ldab + 1)] += lo + hi + 2.0  # dominant diagonal
    b = torch.randn(count, n, dtype=torch.float64, device=dev, generator=g)
    ab = ab0.clone()
    X = b.clone().reshape(-1)
    P, st = band_lu_solve(ab, count, lay, X, 1, algo=algo)
    torch.cuda.synchronize()
    assert int(st.abs().sum().item()) == 0
    x = X.view(count, n)
    # normwise backward error from the input band (diagonals -lo..hi; the
    # fill slots are outputs): ||A x - b|| / (||A|| ||x|| + ||b||), inf-norms
    res = (band_matvec(ab0, lay, count, x) - b).abs().amax(dim=1)
    ones = torch.ones(count, n, dtype=torch.float64, device=dev)
    norm_a = band_matvec(ab0.abs(), lay, count, ones).amax(dim=1)
    berr = res / (norm_a * x.abs().amax(dim=1) + b.abs().amax(dim=1))
    assert float(berr.max()) <= 1e-14
    # sampled systems against the oracle, bit for bit
    sl = slots(lay)
    for s in np.random.default_rng(1).choice(count, size=24, replace=False):
        s = int(s)
        seg = slice(s * lay.stride_ab, (s + 1) * lay.stride_ab)
        sys_ab = ab0[seg].cpu().numpy().copy()
        Po = orc.band_lu_decompose(sys_ab, n, lo, hi, lay.ldab, ALGO[algo])
        xo = b[s].cpu().numpy().copy()
        orc.band_lu_ldiveq(sys_ab, n, lo, hi, lay.ldab, Po, xo, ALGO[algo])
        assert np.array_equal(P[s * n:(s + 1) * n].cpu().numpy(), Po)
        assert np.array_equal(bits(ab[seg].cpu().numpy()[sl]), bits(sys_ab[sl]))
        assert np.array_equal(bits(X[s * n:(s + 1) * n].cpu().numpy()), bits(xo))


def rdiv_rows(rng, count, n, nrhs):
    """Each system's nrhs rows (contiguous, ldb = n) with zeros and negative
    zeros, leading and trailing runs in some rows: the trims and signed-zero
    paths of both passes."""
    M = rng.standard_normal((count, nrhs, n))
    M[rng.random(M.shape) < 0.15] = 0.0
    M[rng.random(M.shape) < 0.05] = -0.0
    if n > 3:
        M[::3, 0, : n // 3] = 0.0
        M[1::3, -1, -(n // 3):] = -0.0
    return M.reshape(-1)


def oracle_rdiv(orc, lay, ab, M, count, nrhs, algo):
    """Per system: factors and P from the oracle's decompose, then its
    LU_RDivEq of the rows; returns (P, status, X)."""
    ab, X = ab.copy(), M.copy()
    n = lay.n
    P = np.zeros((count, n), dtype=np.int64)
    st = np.zeros(count, dtype=np.int32)
    for s in range(count):
        sys_ab = ab[s * lay.stride_ab:(s + 1) * lay.stride_ab]
        P[s] = orc.band_lu_decompose(sys_ab, n, lay.lo, lay.hi, lay.ldab, ALGO[algo])
        Xs = X[s * n * nrhs:(s + 1) * n * nrhs].reshape(nrhs, n)
        try:
            orc.band_lu_rdiveq(sys_ab, n, lay.lo, lay.hi, lay.ldab, P[s], Xs, ALGO[algo], ldb=n)
        except oracle.OracleSingular:
            st[s] = 1
    return P, st, X


def gpu_rdiv(dev, lay, ab, M, count, nrhs, algo):
    import torch

    from tmv_gb300.band import band_lu_decompose, band_lu_rdiveq

    dab = torch.from_numpy(ab).to(dev)
    dM = torch.from_numpy(M).to(dev)
    P = torch.empty(count * lay.n, dtype=torch.int64, device=dev)
    band_lu_decompose(dab, count, lay, P, algo=algo)
    st = band_lu_rdiveq(dab, count, lay, P, dM, nrhs, algo=algo)
    torch.cuda.synchronize()
    return P.cpu().numpy().reshape(count, lay.n), st.cpu().numpy(), dM.cpu().numpy()


@pytest.mark.parametrize("lo,hi,algo", SHAPES)
@pytest.mark.parametrize("kind", ["normal", "int", "tiny"])
def test_band_rdiveq_matches_oracle_bitwise(dev, orc, lo, hi, algo, kind):
    """LU_RDivEq (x P L U = m) for every kernel class: solutions (signed zeros
    included) and statuses bit for bit against the oracle."""
    rng = np.random.default_rng(200 + 10 * lo + hi)
    count, nrhs = 37, 3
    for n in [1, 2, 3, 8, 65, 300]:
        if lo > n - 1 or hi > n - 1:
            continue
        lay, ab, _ = make_batch(rng, count, n, lo, hi, kind, 1)
        M = rdiv_rows(rng, count, n, nrhs)
        o_P, o_st, o_X = oracle_rdiv(orc, lay, ab, M, count, nrhs, algo)
        g_P, g_st, g_X = gpu_rdiv(dev, lay, ab, M, count, nrhs, algo)
        assert np.array_equal(g_P, o_P)
        assert np.array_equal(g_st, o_st), f"n={n}"
        for s in range(count):
            if o_st[s] == 0:
                xs = slice(s * n * nrhs, (s + 1) * n * nrhs)
                assert np.array_equal(bits(g_X[xs]), bits(o_X[xs])), f"n={n} system {s}"


def test_band_rdiveq_singular_and_bad_interchange(dev, orc):
    import torch

    from tmv_gb300.band import band_lu_decompose, band_lu_rdiveq

    rng = np.random.default_rng(17)
    for lo, hi in [(2, 1), (6, 6)]:  # register and wide kernels
        count, n, nrhs = 6, 30, 2
        lay, ab, _ = make_batch(rng, count, n, lo, hi, "normal", 1)
        # a zero column in system 3: a zero U(j,j), met by the forward pass
        for i in range(max(0, 12 - hi), min(n, 12 + lo + 1)):
            ab[3 * lay.stride_ab + i + 12 * lay.ldab] = 0.0
        M = rdiv_rows(rng, count, n, nrhs)
        o_P, o_st, o_X = oracle_rdiv(orc, lay, ab, M, count, nrhs, "general")
        assert o_st[3] == 1
        g_P, g_st, g_X = gpu_rdiv(dev, lay, ab, M, count, nrhs, "general")
        assert np.array_equal(g_st, o_st)
        dab = torch.from_numpy(ab).to(dev)
        P = torch.empty(count * n, dtype=torch.int64, device=dev)
        band_lu_decompose(dab, count, lay, P)
        P[1 * n + 5] = 5 + lo + 1  # beyond the band
        P[2 * n + 7] = 3           # above the diagonal
        st = band_lu_rdiveq(dab, count, lay, P, torch.from_numpy(M).to(dev), nrhs)
        assert st.cpu().tolist() == [0, 2, 2, 1, 0, 0]


def test_band_rdiveq_one_unknown_rows(dev, orc):
    """n = 1 with several rows stored at unit stride (ldb = 1): TMV scales the
    whole row by the reciprocal, as for ldiveq's 1 x nrhs B."""
    import torch

    from tmv_gb300.band import band_layout, band_lu_decompose, band_lu_rdiveq

    lay = band_layout(1, 0, 0)
    for d in [3.0, 0.0]:
        o_ab = np.array([d])
        o_P = orc.band_lu_decompose(o_ab, 1, 0, 0, 1)
        Mo = np.array([[1.0], [-2.0], [7.0]])
        try:
            orc.band_lu_rdiveq(o_ab, 1, 0, 0, 1, o_P, Mo, ldb=1)
            o_st = 0
        except oracle.OracleSingular:
            o_st = 1
        dab = torch.tensor([d], dtype=torch.float64, device=dev)
        P = torch.empty(1, dtype=torch.int64, device=dev)
        band_lu_decompose(dab, 1, lay, P)
        dM = torch.tensor([1.0, -2.0, 7.0], dtype=torch.float64, device=dev)
        st = band_lu_rdiveq(dab, 1, lay, P, dM, 3, ldb=1, stride_b=3)
        assert int(st.item()) == o_st
        if o_st == 0:
            assert np.array_equal(bits(dM.cpu().numpy()), bits(Mo.ravel()))


@pytest.mark.parametrize("lo,hi,algo", [(1, 1, "tridiag"), (2, 2, "general")])
def test_band_rdiveq_benchmark_size(dev, orc, lo, hi, algo):
    """65536 systems of n = 1024 (the band benchmark's batch): x A = m solved
    from the factors; every system's normwise backward error of x A = m at
    most 1e-14, 16 sampled systems bit for bit against the oracle."""
    import torch

    from tmv_gb300.band import band_layout, band_lu_decompose, band_lu_rdiveq

    count, n = 65536, 1024
    lay = band_layout(n, lo, hi)
    g = torch.Generator(device=dev).manual_seed(6)
    ab0 = torch.randn(count * lay.stride_ab, dtype=torch.float64, device=dev, generator=g)
    A = ab0.view(count, lay.stride_ab)
    i = torch.arange(n, device=dev)
    A[:, i * (lay.ldab + 1)] += lo + hi + 2.0
    m = torch.randn(count, n, dtype=torch.float64, device=dev, generator=g)
    ab = ab0.clone()
    P = torch.empty(count * n, dtype=torch.int64, device=dev)
    band_lu_decompose(ab, count, lay, P, algo=algo)
    X = m.clone().reshape(-1)
    st = band_lu_rdiveq(ab, count, lay, P, X, 1, algo=algo)
    torch.cuda.synchronize()
    assert int(st.abs().sum().item()) == 0
    x = X.view(count, n)
    # x A: column j of A against x (the band of the input, diagonals -lo..hi)
    n_, ld = lay.n, lay.ldab
    xa = torch.zeros(count, n, dtype=torch.float64, device=dev)
    na = torch.zeros(count, n, dtype=torch.float64, device=dev)
    for d in range(-lo, hi + 1):
        r = torch.arange(max(0, -d), min(n_, n_ - d), device=dev)  # rows r, columns r + d
        xa[:, r + d] += x[:, r] * A[:, r * (ld + 1) + d * ld]
        na[:, r + d] += A[:, r * (ld + 1) + d * ld].abs()
    res = (xa - m).abs().amax(dim=1)
    # for rows x A the bound is ||x||_inf ||A||_1 (column sums of |A|)
    berr = res / (na.amax(dim=1) * x.abs().amax(dim=1) + m.abs().amax(dim=1))
    assert float(berr.max()) <= 1e-14
    for s in np.random.default_rng(2).choice(count, size=16, replace=False):
        s = int(s)
        seg = slice(s * lay.stride_ab, (s + 1) * lay.stride_ab)
        sys_ab = ab0[seg].cpu().numpy().copy()
        Po = orc.band_lu_decompose(sys_ab, n, lo, hi, lay.ldab, ALGO[algo])
        xo = m[s].cpu().numpy().copy()
        orc.band_lu_rdiveq(sys_ab, n, lo, hi, lay.ldab, Po, xo, ALGO[algo])
        assert np.array_equal(bits(x[s].cpu().numpy()), bits(xo))


@pytest.mark.parametrize("lo,hi", [(1, 1), (2, 2), (0, 3), (3, 0), (1, 0), (2, 1), (3, 1), (5, 2),
                                   (4, 4), (7, 3), (6, 1)])
@pytest.mark.parametrize("kind", ["normal", "int"])
def test_band_divide_matches_bandludiv_composition(dev, orc, lo, hi, kind):
    """B /= A as BandLUDiv runs it (tridiagonal algorithm for lo == hi == 1,
    the transpose factored and solved by rows when hi < lo), for the register
    and wide kernels: solutions, factors and statuses bit for bit against the
    oracle's composition (pinned to TMV's BandLUDiv by test_band_oracle.py)."""
    import torch

    from tests.helpers import band_divide_plan, band_hu, band_pack, oracle_band_divide
    from tmv_gb300.band import band_divide, band_layout

    rng = np.random.default_rng(300 + 10 * lo + hi)
    count, nrhs = 23, 2
    for n in [1, 2, 5, 64, 257]:
        if lo > n - 1 or hi > n - 1:
            continue
        lay = band_layout(n, lo, hi)
        ab = np.full(count * lay.stride_ab, np.nan)  # slots outside the band are never read
        mats = []
        for s in range(count):
            a = band_matrix(rng, n, lo, hi, kind)
            band_pack(a, lo, hi, lay.ldab, out=ab[s * lay.stride_ab:(s + 1) * lay.stride_ab])
            mats.append(a)
        B = rng.standard_normal((count, nrhs, n))
        B[rng.random(B.shape) < 0.15] = 0.0
        dab = torch.from_numpy(ab).to(dev)
        dB = torch.from_numpy(B.reshape(-1).copy()).to(dev)
        lu, lay_lu, P, st, trans = band_divide(dab, count, lay, dB, nrhs)
        torch.cuda.synchronize()
        assert trans == band_divide_plan(lo, hi)[1]
        assert torch.equal(dab.cpu(), torch.from_numpy(ab)) or np.array_equal(
            bits(dab.cpu().numpy()), bits(ab))  # A is not modified
        g_X = dB.cpu().numpy().reshape(count, nrhs, n)
        g_st = st.cpu().numpy()
        g_lu = lu.cpu().numpy()
        for s in range(count):
            Xo, so = oracle_band_divide(orc, mats[s], lo, hi, B[s].T)
            assert g_st[s] == so, f"n={n} system {s}"
            if so == 0:
                assert np.array_equal(bits(g_X[s].T), bits(Xo)), f"n={n} system {s}"
            # the factors: the oracle's decompose of A (or A^T)
            algo, tr = band_divide_plan(lo, hi)
            lo2, hi2 = (hi, lo) if tr else (lo, hi)
            ob = band_pack(mats[s].T if tr else mats[s], lo2, hi2, lay_lu.ldab)
            orc.band_lu_decompose(ob, n, lo2, hi2, lay_lu.ldab, algo)
            hu = band_hu(n, lo2, hi2)
            sl = [i + j * lay_lu.ldab for j in range(n) for i in range(max(0, j - hu), min(n, j + lo2 + 1))]
            seg = g_lu[s * lay_lu.stride_ab:(s + 1) * lay_lu.stride_ab]
            assert np.array_equal(bits(seg[sl]), bits(ob[sl])), f"n={n} system {s} factors"
