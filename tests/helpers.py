"""Shared test helpers: seeded inputs in TMV's layouts and device transfers."""
from __future__ import annotations

import numpy as np


def to_dev(a: np.ndarray, dev, layout: str = "F"):
    """A torch CUDA tensor holding `a` in column-major ("F") or row-major ("C") storage."""
    import torch

    if layout == "F":
        t = torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)
        return t.t()
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def to_host(t) -> np.ndarray:
    return t.detach().cpu().numpy()


def rel_frob(x: np.ndarray, ref: np.ndarray) -> float:
    d = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (d if d > 0 else 1.0))


def arith8_operands(m: int, n: int, k: int):
    """The integer-valued operands of TMV's real product test
    (tests/TMV_TestMatrixArith_8.cpp:327-336): ac(i,j) = i+j+5 (m x k),
    bc(i,j) = 2i-3j+13 (k x n).  Every product is exact in FP64."""
    i = np.arange(m)[:, None]
    j = np.arange(k)[None, :]
    a = (i + j + 5).astype(np.float64)
    i2 = np.arange(k)[:, None]
    j2 = np.arange(n)[None, :]
    b = (2 * i2 - 3 * j2 + 13).astype(np.float64)
    return a, b


def tmv_square4():
    """TMV's 4x4 known-answer matrix and right-hand side
    (tests/TMV_TestMatrixDiv.cpp:11-24); det = 28800 (:76)."""
    m = np.array([[2 + 4 * i - 5 * j for j in range(4)] for i in range(4)], dtype=np.float64)
    m[0, 0], m[1, 0], m[2, 0], m[3, 0], m[2, 2] = 14, -2, 7, -10, 30
    b = np.array([2.0, -10.0, 5.0, -5.0])
    return m, b


def tmv_decomp_matrix(mattype: int, N: int = 200) -> np.ndarray:
    """The square real test matrix of tests/TMV_TestMatrixDecomp.cpp:27-55
    (mattype 0: well conditioned, 3: singular)."""
    M = N
    singular = mattype >= 3
    i = np.arange(M)[:, None]
    j = np.arange(N)[None, :]
    m = (2 + 4 * i - 5 * j).astype(np.float64)
    if not singular:
        m /= 10 * N
    m[3, 3] = 14
    m[3, 4] = -2
    m[0, 2] = 7
    m[M - 1, N - 4] = 23
    m[M - 1, N - 2] = 13
    m[M - 1, N - 1] = -10
    if singular:
        m[:, 1] = 0
        m[7, :] = m[6, :]
    else:
        m[np.arange(N), np.arange(N)] *= 30 * N
    return m


def diag_shift_matrix(rng, n: int, shift: float) -> np.ndarray:
    """A_ij ~ N(0,1) plus `shift` on the diagonal (the workloads' LU matrices)."""
    a = rng.standard_normal((n, n))
    a[np.arange(n), np.arange(n)] += shift
    return a


# --- band storage -----------------------------------------------------------
# TMV's column-major band layout: element (i,j) of an n x n band matrix at
# ab[i + j*ldab] from the (0,0) slot, for j-hu <= i <= j+lo; a batch puts
# system s at ab[s*sab + ...].

def band_hu(n: int, lo: int, hi: int) -> int:
    return min(lo + hi, n - 1) if n > 0 else 0


def band_len(n: int, ldab: int) -> int:
    """Slots from (0,0) to (n-1,n-1), inclusive."""
    return (n - 1) * (ldab + 1) + 1 if n > 0 else 0


def band_pack(a: np.ndarray, lo: int, hi: int, ldab: int, out: np.ndarray | None = None,
              fill: float = 0.0) -> np.ndarray:
    """The band of the dense a (entries outside -lo..hi ignored) in band
    storage; the fill diagonals hi+1..hu and any gap slots hold `fill`."""
    n = a.shape[0]
    hu = band_hu(n, lo, hi)
    ab = np.full(band_len(n, ldab), fill) if out is None else out
    for j in range(n):
        for i in range(max(0, j - hi), min(n, j + lo + 1)):
            ab[i + j * ldab] = a[i, j]
    return ab


def band_unpack(ab: np.ndarray, n: int, lo: int, hu: int, ldab: int) -> np.ndarray:
    a = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - hu), min(n, j + lo + 1)):
            a[i, j] = ab[i + j * ldab]
    return a


def band_matrix(rng, n: int, lo: int, hi: int, kind: str = "normal") -> np.ndarray:
    """A dense n x n matrix with lo subdiagonals and hi superdiagonals.
    kind: normal (N(0,1)), int (integers in -2..2: exact zeros, ties and unit
    pivots), dom (N(0,1) + (lo+hi+1) on the diagonal), tiny (normal with
    subnormal columns that take TMV's underflow branch)."""
    if kind == "int":
        a = rng.integers(-2, 3, size=(n, n)).astype(np.float64)
    else:
        a = rng.standard_normal((n, n))
    if kind == "dom":
        a += (lo + hi + 1) * np.eye(n)
    if kind == "tiny" and n > 2:
        for j in rng.choice(n - 1, size=max(1, n // 8), replace=False):
            a[:, j] *= 1e-310
    return np.triu(np.tril(a, hi), -lo)


def bits(x: np.ndarray) -> np.ndarray:
    """Bit patterns, so that equality also sees signed zeros and infinities;
    every NaN maps to one pattern (the sign and payload of a NaN that an
    operation creates differ between x86, aarch64 and the GPU)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    return np.where(np.isnan(x), np.float64(np.nan), x).view(np.int64)


def band_divide_plan(lo: int, hi: int) -> tuple[int, bool]:
    """BandLUDiv's choices for a column-major tmv::BandMatrix (src/
    TMV_BandLUD.cpp:60-93): the tridiagonal algorithm for lo == hi == 1, the
    transpose factored (and the solve a right division) when hi < lo."""
    return (1 if lo == 1 and hi == 1 else 0), hi < lo


def oracle_band_divide(orc, a: np.ndarray, lo: int, hi: int, B: np.ndarray):
    """X = A^-1 B as BandLUDiv computes it, composed from the oracle's band
    LU_Decompose and LU_LDivEq / LU_RDivEq.  Returns (X, status)."""
    import oracle

    n = a.shape[0]
    algo, trans = band_divide_plan(lo, hi)
    lo2, hi2 = (hi, lo) if trans else (lo, hi)
    ldab = max(lo2 + band_hu(n, lo2, hi2), 1)
    ab = band_pack(a.T if trans else a, lo2, hi2, ldab)
    P = orc.band_lu_decompose(ab, n, lo2, hi2, ldab, algo)
    X = np.asfortranarray(B.copy())
    try:
        if trans:
            orc.band_lu_rdiveq(ab, n, lo2, hi2, ldab, P, X.T, algo)
        else:
            orc.band_lu_ldiveq(ab, n, lo2, hi2, ldab, P, X, algo)
        return X, 0
    except oracle.OracleSingular:
        return X, 1
