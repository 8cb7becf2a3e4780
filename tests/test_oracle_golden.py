"""Pin the oracle (the C restatement of TMV) to outputs of TMV itself.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py
running TMV 0.76 compiled from its sources.  These tests need no GPU.
"""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from helpers import arith8_operands, rel_frob

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    return np.load(GOLD / name, allow_pickle=False)


def sha(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def test_arith8_products_bitwise(orc):
    # tests/TMV_TestMatrixArith_8.cpp: integer-valued operands, every product
    # exact in FP64, so the oracle must reproduce TMV's output bit for bit.
    g = load("arith8.npz")
    sizes = [2, 5, 77, 637]
    for m in sizes:
        for n in sizes:
            for k in sizes:
                a, b = arith8_operands(m, n, k)
                exact = (a.astype(np.int64) @ b.astype(np.int64)).astype(np.float64)
                for la, lb in [("F", "F"), ("C", "F"), ("F", "C")]:
                    key = f"{m}_{n}_{k}_{la}{lb}"
                    A = np.asfortranarray(a) if la == "F" else np.ascontiguousarray(a)
                    B = np.asfortranarray(b) if lb == "F" else np.ascontiguousarray(b)
                    C = np.zeros((m, n), order="F")
                    orc.multmm(False, 1.0, A, B, C)
                    assert sha(C) == str(g["sha_" + key]), key
                    assert sha(exact) == str(g["sha_" + key]), key
                    if "C_" + key in g.files:
                        assert np.array_equal(C, g["C_" + key])


def test_square4_known_answers(orc):
    # tests/TMV_TestMatrixDiv.cpp:11-24,76: det = 28800
    g = load("square4.npz")
    A = np.asfortranarray(g["m"].copy())
    P = orc.lu_decompose(A)
    assert np.array_equal(P, g["P"])
    assert np.abs(A - g["LU"]).max() <= 1e-14 * np.abs(g["LU"]).max()
    det, logdet, sign = orc.det(A, P)
    assert abs(det - 28800) <= 1e-10 * 28800 and abs(det - float(g["det"])) <= 1e-10 * 28800
    assert abs(logdet - float(g["logdet"])) <= 1e-13 and sign == float(g["sign"]) == 1.0
    X, _, _ = orc.divide(g["m"], g["b"].reshape(4, 1))
    assert rel_frob(X, g["X"]) <= 1e-14
    Y = np.asfortranarray(g["b"].reshape(1, 4).copy())
    orc.rdiveq(A, P, Y)
    assert rel_frob(Y, g["Y"]) <= 1e-14


def test_decomp200(orc):
    # tests/TMV_TestMatrixDecomp.cpp:27-55,133-150
    g = load("decomp200.npz")
    for mt in (0, 3):
        a = g[f"m{mt}"]
        A = np.asfortranarray(a.copy())
        P = orc.lu_decompose(A)
        if mt == 0:
            assert np.array_equal(P, g["P0"])
            assert np.abs(A - g["LU0"]).max() <= 1e-12 * np.abs(g["LU0"]).max()
        else:
            # pivots are determined by the data for the first 5 steps only
            # (the rest pivots on rounding noise)
            assert np.array_equal(P[:5], g["P3"][:5])


def test_bign100_system(orc):
    # tests/TMV_TestMatrixDiv.cpp:156-261 (real BIGN=100 system): b/m and b%m
    g = load("bign100.npz")
    M = g["M"]
    A = np.asfortranarray(M.copy())
    P = orc.lu_decompose(A)
    assert np.array_equal(P, g["P"])
    assert np.abs(A - g["LU"]).max() <= 1e-12 * np.abs(g["LU"]).max()
    X, _, _ = orc.divide(M, g["R"].reshape(-1, 1))
    assert rel_frob(X, g["X"]) <= 1e-12
    Y = np.asfortranarray(g["R"].reshape(1, -1).copy())
    orc.rdiveq(A, P, Y)
    assert rel_frob(Y, g["Y"]) <= 1e-12
    # the reference test's own residual criterion: |M x - R| < eps |R|
    assert np.linalg.norm(M @ X[:, 0] - g["R"]) <= 1e-10 * np.linalg.norm(g["R"])


def test_random_pivots_and_factors(orc):
    g = load("random_lu.npz")
    for n in [1, 2, 3, 4, 5, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129]:
        A = np.asfortranarray(g[f"A{n}"].copy())
        P = orc.lu_decompose(A)
        assert np.array_equal(P, g[f"P{n}"]), n
        if f"LU{n}" in g.files:
            ref = g[f"LU{n}"]
            assert np.abs(A - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0), n
        else:
            d = g[f"LUdiag{n}"]
            assert np.abs(np.diag(A) - d).max() <= 1e-12 * np.abs(d).max(), n
    rng = np.random.default_rng(512)
    n = 512
    a = rng.standard_normal((n, n)) + 4 * np.sqrt(n) * np.eye(n)
    A = np.asfortranarray(a)
    assert np.array_equal(orc.lu_decompose(A), g["Pshift512"])


def test_special_inputs(orc):
    # zero / duplicate / tiny / underflowing columns, ties and NaNs.  TMV's
    # underflow test is |pivot| < DBL_MIN: a 1e-160 column is pivoted, a
    # subnormal one is zeroed with P[j] = j.
    g = load("special.npz")
    assert g["P_underflow"][2] == 2 and not g["LU_underflow"][2:, 2].any()
    assert g["P_tiny"][2] != 2
    names = sorted(k[2:] for k in g.files if k.startswith("A_"))
    assert len(names) == 12
    for name in names:
        A = np.asfortranarray(g["A_" + name].copy())
        P = orc.lu_decompose(A)
        assert np.array_equal(P, g["P_" + name]), name
        ref = g["LU_" + name]
        assert np.array_equal(np.isnan(A), np.isnan(ref)), name
        ok = ~np.isnan(ref)
        scale = max(np.abs(ref[ok]).max() if ok.any() else 1.0, 1.0)
        assert np.abs(A[ok] - ref[ok]).max() <= 1e-13 * scale, name


def test_batched_small(orc):
    g = load("batched_small.npz")
    X = g["B"].copy()
    st = orc.batched_divide(g["n"], g["nrhs"], g["a_off"], g["b_off"], g["A"].copy(), X)
    assert not st.any()
    assert np.abs(X - g["X"]).max() <= 1e-13 * np.abs(g["X"]).max()


def test_inverse_fixtures(orc):
    # TMV's m.inverse(), makeInverseATA() and isSingular() (inverse.npz)
    g = load("inverse.npz")
    for name in ["sq4", "r96", "sing6"]:
        M = np.asfortranarray(g[name])
        LU = M.copy(order="F")
        P = orc.lu_decompose(LU)
        assert orc.lu_is_singular(LU) == bool(g[name + "_singular"]), name
        if int(g[name + "_rc"]) == 0:
            assert rel_frob(orc.lu_inverse(LU, P), g[name + "_inv"]) <= 1e-13, name
            assert rel_frob(orc.lu_inverse_ata(LU), g[name + "_ata"]) <= 1e-13, name
        else:
            with pytest.raises(RuntimeError):
                orc.lu_inverse(LU, P)
    # the 4x4 known answer: det 28800 (tests/TMV_TestMatrixDiv.cpp:76), so
    # A * A^-1 = I to rounding
    m = g["sq4"]
    assert np.abs(m @ g["sq4_inv"] - np.eye(4)).max() < 1e-14


def test_multmv_tri_fixtures(orc):
    # TMV's MultMV and TriLDivEq on their special cases (multmv_tri.npz)
    g = load("multmv_tri.npz")
    a, x, y0 = g["mv_A"], g["mv_x"], g["mv_y0"]
    for lay, A in (("F", np.asfortranarray(a)), ("C", np.ascontiguousarray(a))):
        for add in (0, 1):
            y = y0.copy()
            orc.multmv(bool(add), 0.5, A, x, y)
            ref = g[f"mv_{lay}_{add}"]
            assert np.array_equal(np.isnan(y), np.isnan(ref))
            ok = ~np.isnan(ref)
            assert np.abs(y[ok] - ref[ok]).max() <= 1e-14 * np.abs(ref[ok]).max()
    U, b = np.asfortranarray(g["tri_U"]), g["tri_b"]
    for name, B in (("v", np.asfortranarray(b[:, :1])), ("F", np.asfortranarray(b)),
                    ("C", np.ascontiguousarray(b))):
        rc = orc.tri_ldiveq(True, False, U, B)
        assert rc == int(g[f"tri_{name}_rc"]), name
        if rc == 0:
            assert rel_frob(B, g[f"tri_{name}"]) <= 1e-14


def test_complex_lu_fixtures(orc):
    # TMV's own complex<double> LU_Decompose / LU_LDivEq / LU_RDivEq /
    # det (complex_lu.npz)
    g = load("complex_lu.npz")
    for n in [1, 4, 17, 65]:
        a, b = g[f"a{n}"], g[f"b{n}"]
        A = np.asfortranarray(a.copy())
        P = orc.lu_decompose_z(A)
        assert np.array_equal(P, g[f"P{n}"]), n
        LU = g[f"LU{n}"]
        assert np.abs(A - LU).max() <= 1e-12 * np.abs(LU).max(), n
        X = np.asfortranarray(b.copy())
        orc.ldiveq_z(A, P, X)
        assert np.abs(X - g[f"X{n}"]).max() <= 1e-11 * np.abs(g[f"X{n}"]).max(), n
        Y = np.asfortranarray(g[f"w{n}"].copy())
        orc.rdiveq_z(A, P, Y)
        assert np.abs(Y - g[f"Y{n}"]).max() <= 1e-11 * np.abs(g[f"Y{n}"]).max(), n
        det, logdet, sign = orc.lu_det_z(A, P)
        assert abs(det - g[f"det{n}"][0]) <= 1e-12 * abs(g[f"det{n}"][0]), n
        assert abs(logdet - g[f"logdet{n}"][0]) <= 1e-12 * max(1.0, abs(logdet)), n
        assert abs(sign - g[f"sign{n}"][0]) <= 1e-12, n
    for q in range(3):
        A = np.asfortranarray(g[f"s{q}"].copy())
        P = orc.lu_decompose_z(A)
        assert np.array_equal(P, g[f"sP{q}"])
        np.testing.assert_array_equal(A, g[f"sLU{q}"])


def test_band_lu_fixtures(orc):
    # TMV's own band LU_Decompose, LU_LDivEq, LU_RDivEq and BandLUDiv's
    # B /= A (band_lu.npz), bit for bit: pivots, factors, solutions (signed
    # zeros included) and singular statuses
    import oracle
    from helpers import band_hu, band_unpack, bits, oracle_band_divide

    g = load("band_lu.npz")
    for c in range(int(g["count"][0])):
        n, lo, hi, algo, ldab, xst, yst, dst = (int(v) for v in g[f"c{c}_meta"])
        lu = g[f"c{c}_ab"].copy()  # the input band (fill slots zero)
        a = band_unpack(lu, n, lo, band_hu(n, lo, hi), ldab)
        P = orc.band_lu_decompose(lu, n, lo, hi, ldab, algo)
        ctx = f"case {c}: n={n} lo={lo} hi={hi} algo={algo}"
        assert np.array_equal(P, g[f"c{c}_P"]), ctx
        hu = band_hu(n, lo, hi)
        sl = [i + j * ldab for j in range(n) for i in range(max(0, j - hu), min(n, j + lo + 1))]
        assert np.array_equal(bits(lu[sl]), bits(g[f"c{c}_lu"][sl])), ctx
        X = np.asfortranarray(g[f"c{c}_B"].copy())
        try:
            orc.band_lu_ldiveq(lu, n, lo, hi, ldab, P, X, algo)
            st = 0
        except oracle.OracleSingular:
            st = 1
        assert st == xst, ctx
        if st == 0:
            assert np.array_equal(bits(X), bits(g[f"c{c}_X"])), ctx
        Y = g[f"c{c}_M"].copy()
        try:
            orc.band_lu_rdiveq(lu, n, lo, hi, ldab, P, Y, algo)
            st = 0
        except oracle.OracleSingular:
            st = 1
        assert st == yst, ctx
        if st == 0:
            assert np.array_equal(bits(Y), bits(g[f"c{c}_Y"])), ctx
        D, st = oracle_band_divide(orc, a, lo, hi, g[f"c{c}_B"])
        assert st == dst, ctx
        if st == 0:
            assert np.array_equal(bits(D), bits(g[f"c{c}_D"])), ctx
