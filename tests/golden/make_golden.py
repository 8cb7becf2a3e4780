"""Generate the golden fixtures in tests/golden/ from TMV 0.76 itself.

Runs the reference library compiled from the TMV sources (oracle/_ref, built
by ``make -C oracle ref``) on the known-answer inputs of TMV's own tests and
on seeded inputs, and stores inputs and TMV's outputs as compressed .npz
files.  It needs the TMV source tree, given as $TMV_REFERENCE, because it
reads the BIGN=100 system's data out of tests/TMV_TestMatrixDiv.cpp; the
fixtures it writes are committed so that the tests run without it.

    TMV_REFERENCE=<TMV 0.76 tree> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle  # noqa: E402
from helpers import arith8_operands, tmv_decomp_matrix, tmv_square4  # noqa: E402

if not os.environ.get("TMV_REFERENCE"):
    sys.exit("make_golden.py: set TMV_REFERENCE to the TMV 0.76 source tree")
REFERENCE = Path(os.environ["TMV_REFERENCE"])


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def fortran(a):
    return np.asfortranarray(np.array(a, dtype=np.float64))


def arith8(ref):
    # tests/TMV_TestMatrixArith_8.cpp:327-396: integer-valued operands, sizes
    # {2,5,77,637}; TMV's product for every (m,n,k) and the CC/RC/CR layouts.
    sizes = [2, 5, 77, 637]
    out = {}
    for m in sizes:
        for n in sizes:
            for k in sizes:
                a, b = arith8_operands(m, n, k)
                for la, lb in [("F", "F"), ("C", "F"), ("F", "C")]:
                    A = np.asfortranarray(a) if la == "F" else np.ascontiguousarray(a)
                    B = np.asfortranarray(b) if lb == "F" else np.ascontiguousarray(b)
                    C = np.zeros((m, n), order="F")
                    ref.multmm(False, 1.0, A, B, C)
                    key = f"{m}_{n}_{k}_{la}{lb}"
                    if max(m, n) <= 77:
                        out["C_" + key] = C
                    out["sha_" + key] = np.array(sha(C))
    np.savez_compressed(HERE / "arith8.npz", **out)


def square4(ref):
    # tests/TMV_TestMatrixDiv.cpp:11-24,76: the 4x4 known answer (det 28800)
    m, b = tmv_square4()
    A = fortran(m)
    P = ref.lu_decompose(A)
    X, LU2, P2 = ref.divide(m, b.reshape(4, 1))
    Y = ref.rdivide(m, b.reshape(1, 4))
    det, logdet, sign = ref.det_of(m)
    np.savez_compressed(HERE / "square4.npz", m=m, b=b, LU=A, P=P, X=X, Y=Y, det=det,
                        logdet=logdet, sign=sign)


def decomp200(ref):
    # tests/TMV_TestMatrixDecomp.cpp:27-55: N=200 square (0) and singular (3)
    out = {}
    for mt in (0, 3):
        a = tmv_decomp_matrix(mt)
        A = fortran(a)
        P = ref.lu_decompose(A)
        out[f"m{mt}"] = a
        out[f"LU{mt}"] = A
        out[f"P{mt}"] = P
    np.savez_compressed(HERE / "decomp200.npz", **out)


def parse_vector(text: str, name: str) -> list[float]:
    mt = re.search(name + r"\s*<<\s*([^;]+);", text)
    return [float(x) for x in re.split(r"[,\s]+", mt.group(1).strip()) if x]


def bign(ref):
    # tests/TMV_TestMatrixDiv.cpp:156-196: the BIGN=100 real system, read from
    # the reference test file: M = P ^ Q (outer product), diagonal += 215, row
    # 23 scaled by 12, M(12,1) -= 142, two strided sub-vector updates.
    src = (REFERENCE / "tests" / "TMV_TestMatrixDiv.cpp").read_text()
    Pv = np.array(parse_vector(src, r"\bP"))
    Qv = np.array(parse_vector(src, r"\bQ"))
    Rv = np.array(parse_vector(src, r"\bR"))
    N = 100
    assert len(Pv) == len(Qv) == len(Rv) == N
    M = np.outer(Pv, Qv)
    M[np.arange(N), np.arange(N)] += 215.0
    M[int(np.floor(0.23 * N))] *= 12.0
    M[int(np.floor(0.12 * N)), 1] -= 142.0
    # M.subVector(i=65, j=5, istep=1, jstep=3, size=29) *= 2
    i0, j0 = int(np.floor(0.65 * N)), int(np.floor(0.05 * N))
    for t in range(int(np.floor(0.29 * N))):
        M[i0 + t, j0 + 3 * t] *= 2.0
    # M.subVector(i=98, j=12, istep=-1, jstep=2, size=18).addToAll(197)
    i0, j0 = int(np.floor(0.98 * N)), int(np.floor(0.12 * N))
    for t in range(int(np.floor(0.18 * N))):
        M[i0 - t, j0 + 2 * t] += 197.0
    A = fortran(M)
    P = ref.lu_decompose(A)
    X, _, _ = ref.divide(M, Rv.reshape(N, 1))
    Y = ref.rdivide(M, Rv.reshape(1, N))
    np.savez_compressed(HERE / "bign100.npz", M=M, R=Rv, LU=A, P=P, X=X, Y=Y)


def random_lu(ref):
    out = {}
    for n in [1, 2, 3, 4, 5, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129]:
        rng = np.random.default_rng(1000 + n)
        a = rng.standard_normal((n, n))
        A = fortran(a)
        P = ref.lu_decompose(A)
        out[f"A{n}"] = a
        out[f"P{n}"] = P
        if n <= 65:
            out[f"LU{n}"] = A
        else:
            out[f"LUsha{n}"] = np.array(sha(A))
            out[f"LUdiag{n}"] = np.diag(A).copy()
    # the diagonally shifted LU workload family (N(0,1) + 4 sqrt(n) I)
    rng = np.random.default_rng(512)
    n = 512
    a = rng.standard_normal((n, n)) + 4 * np.sqrt(n) * np.eye(n)
    A = fortran(a)
    out["Pshift512"] = ref.lu_decompose(A)
    out["seed_shift512"] = np.array(512)
    np.savez_compressed(HERE / "random_lu.npz", **out)


def special(ref):
    # singular, underflow, ties and NaN inputs: TMV's pivots and factors
    out = {}
    rng = np.random.default_rng(77)
    n = 20
    cases = {}
    a = rng.standard_normal((n, n)); a[:, 6] = 0.0; cases["zerocol"] = a
    a = rng.standard_normal((n, n)); a[11] = a[3]; cases["duprow"] = a
    cases["zeros"] = np.zeros((n, n))
    a = rng.standard_normal((n, n)); a[:, 2] = 1e-160 * rng.standard_normal(n); cases["tiny"] = a
    a = rng.standard_normal((n, n)); a[:, 2] = 1e-310 * rng.standard_normal(n); cases["underflow"] = a
    a = rng.standard_normal((n, n)); a[:, 0] = 0.5; a[[4, 9, 15], 0] = [-2.0, 2.0, -2.0]
    cases["ties"] = a
    for w in [(0, 0), (5, 0), (1, 1), (6, 1), (3, 3), (2, 3)]:
        a = rng.standard_normal((n, n)); a[w] = np.nan; cases[f"nan_{w[0]}_{w[1]}"] = a
    for name, a in cases.items():
        A = fortran(a)
        P = ref.lu_decompose(A)
        out["A_" + name] = a
        out["LU_" + name] = A
        out["P_" + name] = P
    np.savez_compressed(HERE / "special.npz", **out)


def batched_small(ref):
    # ragged batch of small systems solved one by one by TMV (B_i / A_i)
    rng = np.random.default_rng(4)
    count = 24
    ns = rng.integers(8, 49, size=count)
    rs = rng.integers(1, 5, size=count)
    a_off = np.zeros(count, dtype=np.int64)
    b_off = np.zeros(count, dtype=np.int64)
    a_off[1:] = np.cumsum(ns * ns)[:-1]
    b_off[1:] = np.cumsum(ns * rs)[:-1]
    Abuf = np.zeros(int((ns * ns).sum()))
    Bbuf = np.zeros(int((ns * rs).sum()))
    for i, (nn, rr) in enumerate(zip(ns, rs)):
        a = rng.standard_normal((nn, nn)) + 2 * np.sqrt(nn) * np.eye(nn)
        Abuf[a_off[i]:a_off[i] + nn * nn] = a.ravel(order="F")
        Bbuf[b_off[i]:b_off[i] + nn * rr] = rng.standard_normal(nn * rr)
    X = Bbuf.copy()
    st = ref.batched_divide(ns, rs, a_off, b_off, Abuf, X)
    assert not st.any()
    np.savez_compressed(HERE / "batched_small.npz", n=ns, nrhs=rs, a_off=a_off, b_off=b_off,
                        A=Abuf, B=Bbuf, X=X)


def inverse(ref):
    # m.inverse(), m.makeInverseATA(), m.isSingular() as TMV computes them
    # (src/TMV_LUInverse.cpp:236-299, src/TMV_LUD.cpp:158-209): the 4x4
    # known-answer matrix of tests/TMV_TestMatrixDiv.cpp:11-18, a seeded
    # 96 x 96 system with 2*sqrt(n) on the diagonal, and a matrix whose U has
    # an exact zero pivot (TMV throws SingularUpperTriMatrix: rc 1).
    m4, _ = tmv_square4()
    rng = np.random.default_rng(20240607)
    n = 96
    A = rng.standard_normal((n, n)) + 2.0 * np.sqrt(n) * np.eye(n)
    S = np.asfortranarray(np.arange(36, dtype=np.float64).reshape(6, 6) % 7.0)
    S[:, 3] = S[:, 1]  # rank deficient: an exact zero pivot in U
    out = {}
    for name, M in (("sq4", m4), ("r96", A), ("sing6", S)):
        M = fortran(M)
        rc, Minv, Mata, sing = ref.inverse_of(M)
        out[name] = M
        out[name + "_rc"] = np.array(rc)
        out[name + "_singular"] = np.array(sing)
        if rc == 0:
            out[name + "_inv"] = Minv
            out[name + "_ata"] = Mata
    np.savez_compressed(HERE / "inverse.npz", **out)


def multmv_tri(ref):
    # MultMV<add> (src/TMV_MultMV.cpp:1134) and TriLDivEq (src/TMV_TriDiv_M.cpp:583)
    # as TMV computes them, on the cases whose semantics a GPU must keep:
    # a NaN in a column whose x_j is zero (the column form skips it, the row
    # form does not), and a zero U(j,j) met by a zero entry (one column or a
    # column-major block: skipped) or by a row-major block (TMV throws: rc 1).
    rng = np.random.default_rng(20240612)
    out = {}
    a = rng.standard_normal((37, 23))
    a[6, 5] = np.nan
    x = rng.standard_normal(23)
    x[5] = 0.0
    y0 = rng.standard_normal(37)
    out["mv_A"], out["mv_x"], out["mv_y0"] = a, x, y0
    for lay in ("F", "C"):
        A = np.asfortranarray(a) if lay == "F" else np.ascontiguousarray(a)
        for add in (0, 1):
            y = y0.copy()
            ref.multmv(add, 0.5, A, x, y)
            out[f"mv_{lay}_{add}"] = y
    n = 9
    U = np.triu(rng.standard_normal((n, n)) + 3.0 * np.eye(n))
    U[4, 4] = 0.0
    U[4, 5:] = 0.0
    out["tri_U"] = U
    b = rng.standard_normal((n, 3))
    b[4, :] = 0.0
    out["tri_b"] = b
    for name, B in (("v", np.asfortranarray(b[:, :1])), ("F", np.asfortranarray(b)),
                    ("C", np.ascontiguousarray(b))):
        Bc = B.copy(order="K")
        rc = ref.tri_ldiveq(True, False, np.asfortranarray(U), Bc)
        out[f"tri_{name}_rc"] = np.array(rc)
        if rc == 0:
            out[f"tri_{name}"] = np.asfortranarray(Bc)
    np.savez_compressed(HERE / "multmv_tri.npz", **out)


def complex_lu(ref):
    # LU_Decompose, LU_LDivEq, LU_RDivEq, det/logDet and inverse() for
    # std::complex<double> as TMV computes them: seeded complex systems, and
    # 3 x 3 cases for the pivot rule (TMV's
    # modulus: a tie keeps the first index, a larger |re| + |im| with a
    # smaller modulus loses; a zero column underflows)
    rng = np.random.default_rng(20241203)
    rng_w = np.random.default_rng(20241204)  # the right-division operands
    out = {}
    for n in [1, 4, 17, 65]:
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        b = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
        w = rng_w.standard_normal((2, n)) + 1j * rng_w.standard_normal((2, n))
        A = np.asfortranarray(a.copy())
        P = ref.lu_decompose_z(A)
        X = np.asfortranarray(b.copy())
        ref.ldiveq_z(A, P, X)
        Y = np.asfortranarray(w.copy())
        ref.rdiveq_z(A, P, Y)
        det, logdet, sign = ref.det_z(a)
        out[f"inv{n}"] = ref.inverse_z(a)
        out.update({f"a{n}": a, f"b{n}": b, f"w{n}": w, f"LU{n}": A, f"P{n}": P, f"X{n}": X,
                    f"Y{n}": Y, f"det{n}": np.array([det]), f"logdet{n}": np.array([logdet]),
                    f"sign{n}": np.array([sign])})
    cases = [
        [[3 + 4j, 1, 1 - 1j], [5 + 0j, 2, 2 - 2j], [0 + 5j, 3, 3 - 3j]],
        [[1 + 1j, 1, 1 - 1j], [1.5 + 0j, 2, 2 - 2j], [0.1 + 0.1j, 3, 3 - 3j]],
        [[0j, 1, 1 - 1j], [0j, 2, 2 - 2j], [0j, 3, 3 - 3j]],
    ]
    for q, c in enumerate(cases):
        a = np.array(c, dtype=np.complex128)
        A = np.asfortranarray(a.copy())
        P = ref.lu_decompose_z(A)
        out.update({f"s{q}": a, f"sLU{q}": A, f"sP{q}": P})
    np.savez_compressed(HERE / "complex_lu.npz", **out)


def band_lu(ref):
    # TMV's band LU_Decompose (general and tridiagonal algorithms), band
    # LU_LDivEq / LU_RDivEq from those factors, and BandLUDiv's B /= A (the
    # transpose factored when hi < lo), on seeded inputs with exact zeros
    from helpers import band_hu, band_matrix, band_pack

    rng = np.random.default_rng(2024)
    out = {}
    cases = [(n, lo, hi, algo, kind)
             for n in (1, 2, 5, 33)
             for lo, hi, algo in ((0, 0, 0), (0, 2, 0), (1, 0, 0), (1, 1, 0), (1, 1, 1), (2, 1, 0),
                                  (1, 3, 0), (2, 2, 0), (4, 3, 0), (7, 7, 0))
             for kind in ("normal", "int")
             if lo <= n - 1 and hi <= n - 1]
    for c, (n, lo, hi, algo, kind) in enumerate(cases):
        a = band_matrix(rng, n, lo, hi, kind)
        hu = band_hu(n, lo, hi)
        ldab = max(lo + hu, 1)
        ab = band_pack(a, lo, hi, ldab)
        lu = ab.copy()
        P = ref.band_lu_decompose(lu, n, lo, hi, ldab, algo)
        B = rng.standard_normal((n, 2))
        B[rng.random((n, 2)) < 0.2] = 0.0
        X = np.asfortranarray(B.copy())
        try:
            ref.band_lu_ldiveq(lu, n, lo, hi, ldab, P, X, algo)
            xst = 0
        except oracle.OracleSingular:
            xst = 1
        M = rng.standard_normal((2, n))
        M[rng.random((2, n)) < 0.2] = 0.0
        M[rng.random((2, n)) < 0.1] = -0.0
        Y = M.copy()
        try:
            ref.band_lu_rdiveq(lu, n, lo, hi, ldab, P, Y, algo)
            yst = 0
        except oracle.OracleSingular:
            yst = 1
        D = np.asfortranarray(B.copy())
        ldd = max(lo + hi, 1)
        try:
            ref.band_divide(band_pack(a, lo, hi, ldd), n, lo, hi, ldd, D)
            dst = 0
        except oracle.OracleSingular:
            dst = 1
        out.update({f"c{c}_meta": np.array([n, lo, hi, algo, ldab, xst, yst, dst]), f"c{c}_ab": ab,
                    f"c{c}_lu": lu, f"c{c}_P": P, f"c{c}_B": B, f"c{c}_X": X, f"c{c}_M": M,
                    f"c{c}_Y": Y, f"c{c}_D": D})
    out["count"] = np.array([len(cases)])
    np.savez_compressed(HERE / "band_lu.npz", **out)


FIXTURES = [arith8, square4, decomp200, bign, random_lu, special, batched_small, inverse,
            multmv_tri, complex_lu, band_lu]


def main(names: list[str]):
    """Regenerates every fixture, or only those named on the command line."""
    if not oracle.ref_available():
        oracle.build_ref(str(REFERENCE))
    ref = oracle.ref()
    for fx in FIXTURES:
        if not names or fx.__name__ in names:
            fx(ref)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main(sys.argv[1:])
