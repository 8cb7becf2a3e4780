"""The band LU restatement (oracle/tmv_oracle_band.c) against TMV itself:
LU_Decompose(BandMatrixView) and LU_LDivEq on band factors, TMV's general
band algorithm (src/TMV_BandLUDecompose.cpp:49-143) and its tridiagonal one
(:144-200), bit for bit: pivots, factors (signed zeros included), solutions
and the singular status.  Runs only where TMV was compiled (oracle/_ref)."""
import numpy as np
import pytest

import oracle
from tests.helpers import band_hu, band_len, band_matrix, band_pack, bits

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built")

SHAPES = [(0, 0), (0, 2), (1, 0), (1, 1), (2, 1), (1, 3), (2, 2), (3, 3), (4, 2), (7, 7)]


def run(be, a, lo, hi, algo, B, ldab=None):
    n = a.shape[0]
    hu = band_hu(n, lo, hi)
    ldab = lo + hu if ldab is None else ldab
    ab = band_pack(a, lo, hi, ldab, fill=np.nan)
    P = be.band_lu_decompose(ab, n, lo, hi, ldab, algo)
    X = np.asfortranarray(B.copy())
    try:
        be.band_lu_ldiveq(ab, n, lo, hi, ldab, P, X, algo)
        st = 0
    except oracle.OracleSingular:
        st = 1
    return ab, P, X, st


def check(a, lo, hi, algo, B, ldab=None):
    orc, ref = oracle.port(), oracle.ref()
    ab1, P1, X1, s1 = run(orc, a, lo, hi, algo, B, ldab)
    ab2, P2, X2, s2 = run(ref, a, lo, hi, algo, B, ldab)
    n = a.shape[0]
    ctx = f"n={n} lo={lo} hi={hi} algo={algo}"
    assert np.array_equal(P1, P2), ctx
    # band slots only (gap slots of a wider ldab are never touched)
    hu = band_hu(n, lo, hi)
    ld = lo + hu if ldab is None else ldab
    sl = [i + j * ld for j in range(n) for i in range(max(0, j - hu), min(n, j + lo + 1))]
    assert np.array_equal(bits(ab1[sl]), bits(ab2[sl])), ctx
    assert s1 == s2, ctx
    if s1 == 0:
        assert np.array_equal(bits(X1), bits(X2)), ctx
    return s1


@pytest.mark.parametrize("kind", ["normal", "int", "dom", "tiny"])
def test_band_general_bitwise(kind):
    rng = np.random.default_rng(11)
    for n in [1, 2, 3, 5, 17, 64, 150]:
        for lo, hi in SHAPES:
            if lo > n - 1 or hi > n - 1:
                continue
            a = band_matrix(rng, n, lo, hi, kind)
            B = rng.standard_normal((n, 3))
            B[rng.random((n, 3)) < 0.2] = 0.0  # zeros: TMV's zero-skipping branches
            check(a, lo, hi, 0, B)


@pytest.mark.parametrize("kind", ["normal", "int", "dom", "tiny"])
def test_band_tridiag_bitwise(kind):
    rng = np.random.default_rng(12)
    for n in [2, 3, 4, 9, 100, 257]:
        a = band_matrix(rng, n, 1, 1, kind)
        B = rng.standard_normal((n, 2))
        B[rng.random((n, 2)) < 0.2] = 0.0
        check(a, 1, 1, 1, B)


def test_band_edge_cases():
    rng = np.random.default_rng(13)
    # a zero column: the underflow branch, then a singular solve
    a = band_matrix(rng, 12, 2, 1)
    a[:, 5] = 0.0
    assert check(a, 2, 1, 0, rng.standard_normal((12, 1))) == 1
    assert check(a.copy(), 1, 1, 1, rng.standard_normal((12, 1))) in (0, 1)
    # zero right-hand side past the singular row: trimmed, no throw
    b = np.zeros((12, 1))
    b[:3] = 1.0
    check(a, 2, 1, 0, b)
    # a diagonal band: every diagonal entry checked up to the last nonzero
    d = np.diag(rng.standard_normal(8))
    d[2, 2] = 0.0
    b = np.zeros((8, 1))
    b[5] = 1.0
    assert check(d, 0, 0, 0, b) == 1
    # 1 x nrhs right-hand side with ldb = 1 (row-major to TMV)
    check(np.array([[4.0]]), 0, 0, 0, np.array([[1.0, -2.0, 3.0]]))
    check(np.array([[0.0]]), 0, 0, 0, np.array([[1.0, -2.0, 3.0]]))
    # NaN and infinity
    a = band_matrix(rng, 10, 2, 2)
    a[4, 4] = np.nan
    a[7, 6] = np.inf
    check(a, 2, 2, 0, rng.standard_normal((10, 2)))
    # a wider leading dimension than lo + hu
    a = band_matrix(rng, 20, 2, 3)
    check(a, 2, 3, 0, rng.standard_normal((20, 2)), ldab=9)


def rcheck(a, lo, hi, algo, M, ldab=None, ldb=None):
    """LU_RDivEq from the same factors through the restatement and TMV:
    solutions (signed zeros included) and status bit for bit."""
    orc, ref = oracle.port(), oracle.ref()
    n = a.shape[0]
    hu = band_hu(n, lo, hi)
    ldab = lo + hu if ldab is None else ldab
    ab = band_pack(a, lo, hi, ldab, fill=np.nan)
    P = orc.band_lu_decompose(ab, n, lo, hi, ldab, algo)
    out = []
    for be in (orc, ref):
        X = M.copy()
        try:
            be.band_lu_rdiveq(ab, n, lo, hi, ldab, P, X, algo, ldb)
            st = 0
        except oracle.OracleSingular:
            st = 1
        out.append((X, st))
    ctx = f"n={n} lo={lo} hi={hi} algo={algo}"
    assert out[0][1] == out[1][1], ctx
    if out[0][1] == 0:
        assert np.array_equal(bits(out[0][0]), bits(out[1][0])), ctx
    return out[0][1]


def rhs_rows(rng, nrhs, n):
    """nrhs rows with zeros (leading, trailing and scattered) and negative
    zeros: the trims and the signed-zero paths of both passes."""
    M = rng.standard_normal((nrhs, n))
    M[rng.random((nrhs, n)) < 0.2] = 0.0
    M[rng.random((nrhs, n)) < 0.1] = -0.0
    if nrhs > 1 and n > 3:
        M[1, : n // 3] = 0.0
    if nrhs > 2 and n > 3:
        M[2, -(n // 3):] = -0.0
    return M


@pytest.mark.parametrize("kind", ["normal", "int", "dom", "tiny"])
def test_band_rdiveq_general_bitwise(kind):
    rng = np.random.default_rng(21)
    for n in [1, 2, 3, 5, 17, 64, 150]:
        for lo, hi in SHAPES:
            if lo > n - 1 or hi > n - 1:
                continue
            rcheck(band_matrix(rng, n, lo, hi, kind), lo, hi, 0, rhs_rows(rng, 3, n))


@pytest.mark.parametrize("kind", ["normal", "int", "dom", "tiny"])
def test_band_rdiveq_tridiag_bitwise(kind):
    rng = np.random.default_rng(22)
    for n in [2, 3, 4, 9, 100, 257]:
        rcheck(band_matrix(rng, n, 1, 1, kind), 1, 1, 1, rhs_rows(rng, 3, n))


def test_band_rdiveq_edge_cases():
    rng = np.random.default_rng(23)
    # a zero column gives a zero U(j,j): every diagonal from the first
    # nonzero entry on is checked by the forward row form
    a = band_matrix(rng, 12, 2, 1)
    a[:, 5] = 0.0
    assert rcheck(a, 2, 1, 0, rng.standard_normal((1, 12))) == 1
    m = np.zeros((1, 12))
    m[0, 7:] = 1.0  # leading zeros past the singular row: trimmed, no throw
    assert rcheck(a, 2, 1, 0, m) == 0
    # a diagonal band: trailing zeros trimmed, every diagonal before checked
    d = np.diag(rng.standard_normal(8))
    d[2, 2] = 0.0
    m = np.zeros((1, 8))
    m[0, 5] = 1.0
    assert rcheck(d, 0, 0, 0, m) == 1
    m = np.zeros((1, 8))
    m[0, 1] = 1.0
    assert rcheck(d, 0, 0, 0, m) == 0
    # one unknown, several rows stored with unit stride (ldb = 1): a whole
    # row scaled by the reciprocal
    rcheck(np.array([[4.0]]), 0, 0, 0, np.array([[1.0], [-2.0], [3.0]]), ldb=1)
    rcheck(np.array([[0.0]]), 0, 0, 0, np.array([[1.0], [-2.0], [3.0]]), ldb=1)
    # all-zero and negative-zero rows
    a = band_matrix(rng, 9, 1, 2)
    rcheck(a, 1, 2, 0, np.zeros((2, 9)))
    rcheck(a, 1, 2, 0, np.full((2, 9), -0.0))
    rcheck(band_matrix(rng, 9, 1, 1, "int"), 1, 1, 1, np.full((2, 9), -0.0))
    # NaN and infinity
    a = band_matrix(rng, 10, 2, 2)
    a[4, 4] = np.nan
    a[7, 6] = np.inf
    rcheck(a, 2, 2, 0, rng.standard_normal((2, 10)))
    # a wider leading dimension than lo + hu, rows with a gap (ldb > n)
    a = band_matrix(rng, 20, 2, 3)
    M = np.zeros((2, 25))
    M[:, :20] = rng.standard_normal((2, 20))
    rcheck(a, 2, 3, 0, M, ldab=9, ldb=25)


def test_band_divide_composition_matches_bandludiv():
    """TMV's B /= A for a band matrix (BandLUDiv: the tridiagonal algorithm
    for lo == hi == 1, A's transpose factored and LU_RDivEq when hi < lo)
    equals the composition of the restated steps, bit for bit."""
    from tests.helpers import oracle_band_divide

    orc, ref = oracle.port(), oracle.ref()
    rng = np.random.default_rng(31)
    shapes = SHAPES + [(3, 1), (5, 2), (2, 0), (6, 1)]
    for kind in ["normal", "int", "tiny"]:
        for n in [1, 2, 3, 7, 40, 150]:
            for lo, hi in shapes:
                if lo > n - 1 or hi > n - 1:
                    continue
                a = band_matrix(rng, n, lo, hi, kind)
                B = rng.standard_normal((n, 3))
                B[rng.random((n, 3)) < 0.2] = 0.0
                X1, s1 = oracle_band_divide(orc, a, lo, hi, B)
                X2 = np.asfortranarray(B.copy())
                try:
                    ref.band_divide(band_pack(a, lo, hi, max(lo + hi, 1)), n, lo, hi, max(lo + hi, 1), X2)
                    s2 = 0
                except oracle.OracleSingular:
                    s2 = 1
                ctx = f"n={n} lo={lo} hi={hi} {kind}"
                assert s1 == s2, ctx
                if s1 == 0:
                    assert np.array_equal(bits(X1), bits(X2)), ctx
