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
