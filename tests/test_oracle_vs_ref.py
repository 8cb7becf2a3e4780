"""The oracle's C restatement against TMV itself on seeded inputs.

Runs only where the reference library was compiled from the TMV sources
(oracle/_ref); elsewhere the committed golden fixtures pin the oracle.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built")


@pytest.fixture(scope="module")
def ref():
    return oracle.ref()


@pytest.mark.parametrize("generic", [False, True])
def test_lu_pivots_match(orc, generic):
    r = oracle.ref(generic=generic)
    rng = np.random.default_rng(99)
    for n in [6, 34, 70, 130, 300, 513]:
        a = rng.standard_normal((n, n))
        A1, A2 = np.asfortranarray(a.copy()), np.asfortranarray(a.copy())
        p1, p2 = orc.lu_decompose(A1), r.lu_decompose(A2)
        assert np.array_equal(p1, p2), n
        assert np.abs(A1 - A2).max() <= 1e-11 * np.abs(A2).max()


def test_row_major_lu(orc, ref):
    # LU_Decompose of a row-major view factors A's own values
    rng = np.random.default_rng(3)
    a = rng.standard_normal((90, 90))
    A1, A2 = np.ascontiguousarray(a.copy()), np.ascontiguousarray(a.copy())
    p1, p2 = orc.lu_decompose(A1), ref.lu_decompose(A2)
    assert np.array_equal(p1, p2)
    assert np.abs(A1 - A2).max() <= 1e-12 * np.abs(A2).max()


@pytest.mark.parametrize("la,lb,lc", [("F", "F", "F"), ("F", "C", "F"), ("C", "F", "F"),
                                      ("C", "C", "F"), ("F", "F", "C")])
def test_products(orc, ref, la, lb, lc):
    rng = np.random.default_rng(5)
    for (m, n, k) in [(3, 4, 5), (17, 65, 33), (130, 70, 257), (300, 301, 64)]:
        a, b = rng.uniform(-1, 1, (m, k)), rng.uniform(-1, 1, (k, n))
        c0 = rng.uniform(-1, 1, (m, n))
        A = np.asfortranarray(a) if la == "F" else np.ascontiguousarray(a)
        B = np.asfortranarray(b) if lb == "F" else np.ascontiguousarray(b)
        for add, alpha in [(False, 1.0), (True, -1.0), (True, 3.0)]:
            C1 = np.asfortranarray(c0) if lc == "F" else np.ascontiguousarray(c0)
            C2 = C1.copy(order="K")
            orc.multmm(add, alpha, A, B, C1)
            ref.multmm(add, alpha, A, B, C2)
            assert np.abs(C1 - C2).max() <= 1e-14 * max(np.abs(C2).max(), 1.0)


def test_solves_and_det(orc, ref):
    rng = np.random.default_rng(8)
    for n, nrhs in [(5, 1), (64, 3), (200, 8)]:
        a = rng.standard_normal((n, n))
        b = rng.standard_normal((n, nrhs))
        x1, lu1, p1 = orc.divide(a, b)
        x2, lu2, p2 = ref.divide(a, b)
        assert np.array_equal(p1, p2)
        assert np.abs(x1 - x2).max() <= 1e-11 * np.abs(x2).max()
        w = rng.standard_normal((nrhs, n))
        y1 = np.asfortranarray(w.copy())
        orc.rdiveq(lu1, p1, y1)
        y2 = ref.rdivide(a, w)
        assert np.abs(y1 - y2).max() <= 1e-11 * np.abs(y2).max()
        d1 = orc.det(lu1, p1)
        d2 = ref.det_of(a)
        assert abs(d1[1] - d2[1]) <= 1e-12 * max(abs(d2[1]), 1.0) and d1[2] == d2[2]


def test_singular_solve_agrees(orc, ref):
    rng = np.random.default_rng(1)
    n = 10
    a = rng.standard_normal((n, n))
    a[:, 3] = 0.0
    b = rng.standard_normal((n, 2))
    with pytest.raises(oracle.OracleSingular):
        orc.divide(a, b)
    with pytest.raises(oracle.OracleSingular):
        ref.divide(a, b)


def test_inverse_ata_singular_match_tmv(orc, ref):
    # LU_Inverse, makeInverseATA and isSingular (src/TMV_LUInverse.cpp:236-299,
    # src/TMV_LUD.cpp:172-209) restated against TMV's own results
    rng = np.random.default_rng(17)
    for n in [1, 3, 8, 64, 65, 129, 200]:
        a = np.asfortranarray(rng.standard_normal((n, n)) + 2.0 * np.sqrt(n) * np.eye(n))
        rc, inv_t, ata_t, sing_t = ref.inverse_of(a)
        assert rc == 0
        LU = a.copy(order="F")
        P = orc.lu_decompose(LU)
        assert np.linalg.norm(orc.lu_inverse(LU, P) - inv_t) <= 1e-13 * np.linalg.norm(inv_t), n
        assert np.linalg.norm(orc.lu_inverse_ata(LU) - ata_t) <= 1e-13 * np.linalg.norm(ata_t), n
        assert orc.lu_is_singular(LU) == sing_t
    # a zero pivot: TMV throws SingularUpperTriMatrix, the oracle reports it
    s = np.asfortranarray(np.arange(36, dtype=np.float64).reshape(6, 6) % 7.0)
    s[:, 3] = s[:, 1]
    rc, _, _, sing_t = ref.inverse_of(s)
    LU = s.copy(order="F")
    P = orc.lu_decompose(LU)
    assert rc == 1 and sing_t and orc.lu_is_singular(LU)
    with pytest.raises(RuntimeError):
        orc.lu_inverse(LU, P)


def test_multmv_and_tri_ldiveq_match_tmv(orc, ref):
    # MultMV<add> (src/TMV_MultMV.cpp:1134) over TMV's layouts and alpha/add
    # branches; TriLDivEq (src/TMV_TriDiv_M.cpp:583) for both triangles
    rng = np.random.default_rng(23)
    for m, n in [(1, 1), (5, 3), (3, 5), (77, 40), (40, 77), (300, 301)]:
        a = rng.standard_normal((m, n))
        big = np.zeros((2 * m + 1, 3 * n + 2))
        big[: 2 * m : 2, : 3 * n : 3] = a
        for A in (np.asfortranarray(a), np.ascontiguousarray(a), big[: 2 * m : 2, : 3 * n : 3]):
            x = rng.standard_normal(n)
            y0 = rng.standard_normal(m)
            for add in (False, True):
                for alpha in (1.0, -0.75):
                    y1, y2 = y0.copy(), y0.copy()
                    orc.multmv(add, alpha, A, x, y1)
                    ref.multmv(add, alpha, A, x, y2)
                    assert np.abs(y1 - y2).max() <= 1e-14 * max(np.abs(y2).max(), 1.0)
    for n in [1, 7, 64, 65, 200]:
        T = np.asfortranarray(rng.standard_normal((n, n)) + 2.0 * np.sqrt(n) * np.eye(n))
        for upper in (True, False):
            for unit in (True, False):
                for b in (rng.standard_normal((n, 1)), rng.standard_normal((n, 5))):
                    for B1 in (np.array(b, order="F", copy=True), np.array(b, order="C", copy=True)):
                        B2 = B1.copy(order="K")
                        assert orc.tri_ldiveq(upper, unit, T, B1) == ref.tri_ldiveq(upper, unit, T, B2) == 0
                        assert np.abs(B1 - B2).max() <= 1e-13 * max(np.abs(B2).max(), 1.0)


@pytest.mark.parametrize("generic", [False, True])
def test_complex_lu_and_solve_match_tmv(orc, generic):
    # complex<double>: TMV's modulus for the pivot search, its guarded
    # reciprocal for the scaling and the divisions; the block steps round
    # differently from TMV's blocked complex product, so values to 1e-12
    r = oracle.ref(generic=generic)
    rng = np.random.default_rng(41)
    for n in [1, 2, 3, 4, 5, 17, 64, 65, 130, 300]:
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        A1, A2 = np.asfortranarray(a.copy()), np.asfortranarray(a.copy())
        p1, p2 = orc.lu_decompose_z(A1), r.lu_decompose_z(A2)
        assert np.array_equal(p1, p2), n
        assert np.abs(A1 - A2).max() <= 1e-12 * np.abs(A2).max(), n
        if n <= 3:  # the leaves alone: the same operations in the same order
            assert np.array_equal(A1, A2), n
        b = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
        x1, x2 = np.asfortranarray(b.copy()), np.asfortranarray(b.copy())
        orc.ldiveq_z(A1, p1, x1)
        r.ldiveq_z(A2, p2, x2)
        scale = np.abs(a).sum(axis=1).max() * np.abs(x2).max()
        assert np.abs(a @ x1 - b).max() <= 1e-13 * scale, n
        assert np.abs(x1 - x2).max() <= 1e-11 * np.abs(x2).max(), n


def test_complex_pivot_rule_and_special_entries(orc, ref):
    # ties under TMV's modulus keep the first index; an entry whose |re| + |im|
    # is larger but whose modulus is smaller loses; a zero column underflows
    cases = [
        np.array([[3 + 4j, 1], [5 + 0j, 2], [0 + 5j, 3]]),
        np.array([[1 + 1j, 1], [1.5 + 0j, 2], [0.1 + 0.1j, 3]]),
        np.array([[0j, 1], [0j, 2], [0j, 3]]),
    ]
    for c in cases:
        m = c.shape[0]
        a = np.zeros((m, m), dtype=np.complex128)
        a[:, :2] = c
        if m > 2:
            a[:, 2] = np.arange(1, m + 1) * (1 - 1j)
        A1, A2 = np.asfortranarray(a.copy()), np.asfortranarray(a.copy())
        p1, p2 = orc.lu_decompose_z(A1), ref.lu_decompose_z(A2)
        assert np.array_equal(p1, p2)
        np.testing.assert_array_equal(A1, A2)


def test_complex_rdiveq_and_det_match_tmv(orc, ref):
    # b % m (row-oriented transposed solves) and det/logDet for complex
    rng = np.random.default_rng(43)
    for n in [1, 2, 3, 5, 17, 65, 130]:
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        A1, A2 = np.asfortranarray(a.copy()), np.asfortranarray(a.copy())
        p1, p2 = orc.lu_decompose_z(A1), ref.lu_decompose_z(A2)
        for rows in [1, 3]:
            w = rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))
            y1, y2 = np.asfortranarray(w.copy()), np.asfortranarray(w.copy())
            orc.rdiveq_z(A1, p1, y1)
            ref.rdiveq_z(A2, p2, y2)
            assert np.abs(y1 - y2).max() <= 1e-11 * np.abs(y2).max(), (n, rows)
            if n <= 3 and rows == 1:
                assert np.array_equal(y1, y2), n
            scale = np.abs(a).sum(axis=0).max() * np.abs(y1).max()
            assert np.abs(y1 @ a - w).max() <= 1e-13 * scale
        d1, l1, s1 = orc.lu_det_z(A1, p1)
        d2, l2, s2 = ref.det_z(a)
        assert abs(d1 - d2) <= 1e-12 * abs(d2) and abs(l1 - l2) <= 1e-12 * max(1.0, abs(l2))
        assert abs(s1 - s2) <= 1e-12
    # a zero column: det 0, logdet -inf, sign 0, and b % m singular in both
    a = np.array([[1 + 1j, 2, 0], [0, 0, 0], [3j, 1, 0]], dtype=np.complex128)
    A1, A2 = np.asfortranarray(a.copy()), np.asfortranarray(a.copy())
    p1, p2 = orc.lu_decompose_z(A1), ref.lu_decompose_z(A2)
    assert orc.lu_det_z(A1, p1) == ref.det_z(a) == (0j, -np.inf, 0j)
    for backend, (f, p) in ((orc, (A1, p1)), (ref, (A2, p2))):
        with pytest.raises(oracle.OracleSingular):
            backend.rdiveq_z(f, p, np.asfortranarray(np.ones((1, 3), dtype=np.complex128)))


@pytest.mark.parametrize("layouts", ["FFF", "CFF", "FCF", "FFC", "CCC"])
def test_complex_products_match_tmv(orc, ref, layouts):
    # MultMM<add> for complex<double> in TMV's layouts (F: column-major,
    # C: row-major for A, B, C), C = alpha A B and C += alpha A B
    rng = np.random.default_rng(47)
    for (m, n, k) in [(1, 1, 1), (7, 5, 3), (64, 64, 64), (100, 37, 80)]:
        def mk(r, c, o):
            return np.asarray(rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c)), order=o)
        A, B, C0 = mk(m, k, layouts[0]), mk(k, n, layouts[1]), mk(m, n, layouts[2])
        for add in (0, 1):
            c1, c2 = C0.copy(order="K"), C0.copy(order="K")
            orc.multmm_z(add, 0.7 - 1.3j, A, B, c1)
            ref.multmm_z(add, 0.7 - 1.3j, A, B, c2)
            assert np.abs(c1 - c2).max() <= 1e-13 * np.abs(c2).max(), (m, n, k, add)
