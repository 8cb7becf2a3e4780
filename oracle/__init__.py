"""CPU checkers for the GPU path -- TEST INFRASTRUCTURE ONLY.

Two interchangeable backends with one numpy interface:

* ``port()``  -- oracle/_build/liboracle.so, the C restatement of TMV's
  MultMM / LU_Decompose / LU_LDivEq / LU_RDivEq (tmv_oracle.c).  Builds on any
  machine with gcc (``make -C oracle port``).
* ``ref()``   -- oracle/_ref/libtmvref.so, TMV 0.76 itself compiled from the
  reference sources (``make -C oracle ref``; only where those sources exist).
  ``ref(generic=True)`` uses TMV's generic (non-SSE) product kernels, the ones
  an aarch64 build runs.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this
package.  The product (tmv_gb300/) never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libtmvref.so"
REF_GENERIC_LIB = HERE / "_ref" / "libtmvref_generic.so"

i64 = C.c_int64
vp = C.c_void_p
dbl = C.c_double

SINGULAR = 1


class OracleSingular(RuntimeError):
    pass


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_LIB


def build_ref(reference: str | Path, jobs: int | None = None,
              tmv_obj: str | Path | None = None) -> Path | None:
    """Compile TMV from the source tree `reference` into oracle/_ref
    (tmv_obj: a directory holding TMV's objects already compiled from that
    tree with the same flags, linked instead of compiled again)."""
    import os

    if not Path(reference, "src", "TMV_LUDecompose.cpp").exists():
        return None
    jobs = jobs or (os.cpu_count() or 4)
    cmd = ["make", "-s", f"-j{jobs}", "-C", str(HERE), "ref", f"REF={reference}"]
    if tmv_obj is not None:
        cmd.append(f"TMV_OBJ={tmv_obj}")
    subprocess.run(cmd, check=True)
    return REF_LIB


def _p(a: np.ndarray) -> vp:
    return vp(a.ctypes.data)


def _strides(a: np.ndarray):
    it = a.itemsize
    if a.ndim == 1:
        return a.strides[0] // it, a.size * (a.strides[0] // it)
    return a.strides[0] // it, a.strides[1] // it


class _Backend:
    prefix = ""

    def __init__(self, path: Path):
        if not path.exists():
            raise FileNotFoundError(f"{path} not built")
        self.lib = C.CDLL(str(path))
        self.path = path

    def _f(self, name, res, args):
        f = getattr(self.lib, self.prefix + name)
        f.restype = res
        f.argtypes = args
        return f

    # numpy-level interface -------------------------------------------------
    def multmm(self, add: bool, alpha: float, A: np.ndarray, B: np.ndarray, Cm: np.ndarray) -> None:
        m, k = A.shape
        n = B.shape[1]
        f = self._f("multmm", C.c_int, [C.c_int, dbl, i64, i64, i64, vp, i64, i64, vp, i64, i64,
                                        vp, i64, i64])
        rc = f(int(add), alpha, m, n, k, _p(A), *_strides(A), _p(B), *_strides(B), _p(Cm),
               *_strides(Cm))
        if rc:
            raise RuntimeError(f"multmm rc={rc}")

    def lu_decompose(self, A: np.ndarray) -> np.ndarray:
        """In place; returns P (int64)."""
        n = A.shape[0]
        P = np.zeros(min(A.shape), dtype=np.int64)
        rc = self._lu(A, P)
        if rc:
            raise RuntimeError(f"lu rc={rc}")
        return P

    # complex<double>: column-major (Fortran-order) complex128 arrays
    def multmm_z(self, add: bool, alpha: complex, A: np.ndarray, B: np.ndarray, Cm: np.ndarray) -> None:
        """C (+)= alpha A B for complex128 arrays of any strides."""
        for x in (A, B, Cm):
            assert x.dtype == np.complex128
        m, k = A.shape
        n = B.shape[1]
        al = np.array([complex(alpha).real, complex(alpha).imag])
        f = self._f("multmm_z", C.c_int, [C.c_int, vp, i64, i64, i64, vp, i64, i64, vp, i64, i64,
                                          vp, i64, i64])
        rc = f(int(add), _p(al), m, n, k, _p(A), *_strides(A), _p(B), *_strides(B), _p(Cm),
               *_strides(Cm))
        if rc:
            raise RuntimeError(f"multmm_z rc={rc}")

    def lu_decompose_z(self, A: np.ndarray) -> np.ndarray:
        """In place; returns P (int64)."""
        assert A.dtype == np.complex128 and A.flags.f_contiguous and A.shape[0] == A.shape[1]
        n = A.shape[0]
        P = np.zeros(n, dtype=np.int64)
        f = self._f("lu_decompose_z", C.c_int, [i64, vp, i64, vp])
        rc = f(n, _p(A), n, _p(P))
        if rc:
            raise RuntimeError(f"lu_z rc={rc}")
        return P

    def ldiveq_z(self, LU: np.ndarray, P: np.ndarray, B: np.ndarray) -> None:
        """B (n x nrhs, Fortran-order complex128) := (P L U)^-1 B in place."""
        assert LU.dtype == np.complex128 and LU.flags.f_contiguous
        assert B.dtype == np.complex128 and B.flags.f_contiguous
        n = LU.shape[0]
        nrhs = 1 if B.ndim == 1 else B.shape[1]
        f = self._f("lu_ldiveq_z", C.c_int, [i64, vp, i64, vp, i64, vp, i64])
        rc = f(n, _p(LU), n, _p(P), nrhs, _p(B), n)
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"ldiveq_z rc={rc}")

    def rdiveq_z(self, LU: np.ndarray, P: np.ndarray, B: np.ndarray) -> None:
        """B (nrows x n, Fortran-order complex128) := B (P L U)^-1 in place."""
        assert LU.dtype == np.complex128 and LU.flags.f_contiguous
        assert B.dtype == np.complex128 and B.flags.f_contiguous and B.ndim == 2
        n = LU.shape[0]
        f = self._f("lu_rdiveq_z", C.c_int, [i64, vp, i64, vp, i64, vp, i64])
        rc = f(n, _p(LU), n, _p(P), B.shape[0], _p(B), max(B.shape[0], 1))
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"rdiveq_z rc={rc}")

    def ldiveq(self, LU: np.ndarray, P: np.ndarray, B: np.ndarray) -> None:
        n = LU.shape[0]
        Bv = B.reshape(n, -1) if B.ndim == 1 else B
        f = self._f("lu_ldiveq", C.c_int, [i64, vp, i64, vp, i64, vp, i64, i64])
        rc = f(n, _p(LU), LU.strides[1] // 8, _p(P), Bv.shape[1], _p(Bv), *_strides(Bv))
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"ldiveq rc={rc}")

    def rdiveq(self, LU: np.ndarray, P: np.ndarray, B: np.ndarray) -> None:
        n = LU.shape[0]
        Bv = B.reshape(1, n) if B.ndim == 1 else B
        f = self._f("lu_rdiveq", C.c_int, [i64, vp, i64, vp, i64, vp, i64, i64])
        rc = f(n, _p(LU), LU.strides[1] // 8, _p(P), Bv.shape[0], _p(Bv), *_strides(Bv))
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"rdiveq rc={rc}")

    def divide(self, A: np.ndarray, B: np.ndarray):
        """X = B / A with A column-major; returns (X, LU, P)."""
        n = A.shape[0]
        A = np.asfortranarray(A)
        B2 = np.asfortranarray(B.reshape(n, -1))
        X = np.zeros_like(B2, order="F")
        LU = np.zeros((n, n), order="F")
        P = np.zeros(n, dtype=np.int64)
        rc = self._divide(n, A, B2, X, LU, P)
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"divide rc={rc}")
        return X, LU, P

    def batched_divide(self, n, nrhs, a_off, b_off, A, B) -> np.ndarray:
        cnt = len(n)
        st = np.zeros(cnt, dtype=np.int32)
        f = self._f("batched_divide", C.c_int, [i64, vp, vp, vp, vp, vp, vp, vp])
        n = np.ascontiguousarray(n, dtype=np.int64)
        nrhs = np.ascontiguousarray(nrhs, dtype=np.int64)
        a_off = np.ascontiguousarray(a_off, dtype=np.int64)
        b_off = np.ascontiguousarray(b_off, dtype=np.int64)
        f(cnt, _p(n), _p(nrhs), _p(a_off), _p(b_off), _p(A), _p(B), _p(st))
        return st

    # band LU: TMV's column-major band storage, element (i,j) at ab[i + j*ldab]
    def band_lu_decompose(self, ab: np.ndarray, n: int, lo: int, hi: int, ldab: int,
                          algo: int = 0) -> np.ndarray:
        """LU_Decompose of the band matrix in the float64 buffer ab (in place,
        (0,0) at ab[0]); algo 0 is TMV's general band algorithm, 1 its
        tridiagonal one.  Returns P (int64)."""
        assert ab.dtype == np.float64 and ab.flags.c_contiguous
        P = np.zeros(max(n, 0), dtype=np.int64)
        f = self._f("band_lu_decompose", C.c_int, [i64, i64, i64, C.c_int, vp, i64, vp])
        rc = f(n, lo, hi, algo, _p(ab), ldab, _p(P))
        if rc:
            raise RuntimeError(f"band_lu_decompose rc={rc}")
        return P

    def band_lu_ldiveq(self, lu: np.ndarray, n: int, lo: int, hi: int, ldab: int, P: np.ndarray,
                       B: np.ndarray, algo: int = 0, ldb: int | None = None) -> None:
        """B (n x nrhs, column-major in a flat or Fortran-order float64 array)
        := (P L U)^-1 B in place from band factors."""
        assert B.dtype == np.float64
        nrhs = 1 if B.ndim == 1 else B.shape[1]
        if ldb is None:
            ldb = n if B.ndim == 1 else B.strides[1] // 8
        f = self._f("band_lu_ldiveq", C.c_int, [i64, i64, i64, C.c_int, vp, i64, vp, i64, vp, i64])
        rc = f(n, lo, hi, algo, _p(lu), ldab, _p(np.ascontiguousarray(P, dtype=np.int64)), nrhs,
               _p(B), ldb)
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"band_lu_ldiveq rc={rc}")

    def band_lu_rdiveq(self, lu: np.ndarray, n: int, lo: int, hi: int, ldab: int, P: np.ndarray,
                       M: np.ndarray, algo: int = 0, ldb: int | None = None) -> None:
        """M (nrhs x n, each row contiguous: a flat or C-order float64 array)
        := M (P L U)^-1 in place from band factors (LU_RDivEq)."""
        assert M.dtype == np.float64
        nrhs = 1 if M.ndim == 1 else M.shape[0]
        if ldb is None:
            ldb = n if M.ndim == 1 else M.strides[0] // 8
        f = self._f("band_lu_rdiveq", C.c_int, [i64, i64, i64, C.c_int, vp, i64, vp, i64, vp, i64])
        rc = f(n, lo, hi, algo, _p(lu), ldab, _p(np.ascontiguousarray(P, dtype=np.int64)), nrhs,
               _p(M), ldb)
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"band_lu_rdiveq rc={rc}")

    def band_divide(self, ab: np.ndarray, n: int, lo: int, hi: int, ldab: int, B: np.ndarray) -> None:
        """B := A^-1 B through TMV's BandLUDiv (B /= A for a tmv::BandMatrix;
        TMV itself only): A's band (lo, hi) at ab[i + j*ldab], j-hi <= i <= j+lo;
        B n x nrhs column-major."""
        assert B.dtype == np.float64
        nrhs = 1 if B.ndim == 1 else B.shape[1]
        ldb = n if B.ndim == 1 else B.strides[1] // 8
        f = self._f("band_divide", C.c_int, [i64, i64, i64, vp, i64, i64, vp, i64])
        rc = f(n, lo, hi, _p(np.ascontiguousarray(ab, dtype=np.float64)), ldab, nrhs, _p(B), ldb)
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"band_divide rc={rc}")

    def band_batched_solve(self, count: int, n: int, lo: int, hi: int, algo: int, ab: np.ndarray,
                           ldab: int, sab: int, nrhs: int, B: np.ndarray, ldb: int, sb: int):
        """The batched band workload in place on the host cores (OpenMP over
        systems); returns (P, status)."""
        P = np.zeros(count * max(n, 1), dtype=np.int64)
        st = np.zeros(count, dtype=np.int32)
        f = self._f("band_batched_solve", C.c_int, [i64, i64, i64, i64, C.c_int, vp, i64, i64, vp,
                                                    i64, i64, vp, i64, i64, vp])
        f(count, n, lo, hi, algo, _p(ab), ldab, sab, _p(P), max(n, 1), nrhs, _p(B), ldb, sb, _p(st))
        return P, st

    def set_threads(self, t: int) -> None:
        self._f("set_threads", None, [C.c_int])(t)

    def max_threads(self) -> int:
        return int(self._f("max_threads", C.c_int, [])())


class Port(_Backend):
    prefix = "oracle_"

    def lu_det_z(self, LU: np.ndarray, P: np.ndarray):
        """(det, logdet, sign) from complex LU factors."""
        d, s = np.zeros(2), np.zeros(2)
        ld = C.c_double()
        f = self._f("lu_det_z", None, [i64, vp, i64, vp, vp, C.POINTER(C.c_double), vp])
        f(LU.shape[0], _p(LU), LU.shape[0], _p(P), _p(d), C.byref(ld), _p(s))
        return complex(d[0], d[1]), ld.value, complex(s[0], s[1])

    def _lu(self, A, P):
        f = self._f("lu_decompose", C.c_int, [i64, i64, vp, i64, i64, vp])
        return f(A.shape[0], A.shape[1], _p(A), *_strides(A), _p(P))

    def _divide(self, n, A, B, X, LU, P):
        f = self._f("divide", C.c_int, [i64, vp, i64, vp, vp, vp, vp])
        return f(n, _p(A), B.shape[1], _p(B), _p(X), _p(LU), _p(P))

    def det(self, LU: np.ndarray, P: np.ndarray):
        d, ld, s = dbl(), dbl(), dbl()
        f = self._f("lu_det", None, [i64, vp, i64, vp, C.POINTER(dbl), C.POINTER(dbl),
                                     C.POINTER(dbl)])
        f(LU.shape[0], _p(LU), LU.strides[1] // 8, _p(P), C.byref(d), C.byref(ld), C.byref(s))
        return d.value, ld.value, s.value


    def lu_inverse(self, LU: np.ndarray, P: np.ndarray) -> np.ndarray:
        """LU_Inverse: A^-1 from the factors (column-major)."""
        n = LU.shape[0]
        LU = np.asfortranarray(LU)
        M = np.zeros((n, n), order="F")
        f = self._f("lu_inverse", C.c_int, [i64, vp, i64, vp, vp, i64])
        rc = f(n, _p(LU), max(n, 1), _p(np.ascontiguousarray(P, dtype=np.int64)), _p(M), max(n, 1))
        if rc:
            raise RuntimeError(f"lu_inverse rc={rc}")
        return M

    def lu_inverse_ata(self, LU: np.ndarray) -> np.ndarray:
        """LUDiv::makeInverseATA: (A^T A)^-1 from the factors."""
        n = LU.shape[0]
        LU = np.asfortranarray(LU)
        M = np.zeros((n, n), order="F")
        f = self._f("lu_inverse_ata", C.c_int, [i64, vp, i64, vp, i64])
        rc = f(n, _p(LU), max(n, 1), _p(M), max(n, 1))
        if rc:
            raise RuntimeError(f"lu_inverse_ata rc={rc}")
        return M

    def lu_is_singular(self, LU: np.ndarray) -> bool:
        LU = np.asfortranarray(LU)
        f = self._f("lu_is_singular", C.c_int, [i64, vp, i64])
        return bool(f(LU.shape[0], _p(LU), max(LU.shape[0], 1)))


    def multmv(self, add: bool, alpha: float, A: np.ndarray, x: np.ndarray, y: np.ndarray) -> None:
        """y (+)= alpha A x in place (MultMV<add>); A any strides, x and y 1-D."""
        f = self._f("multmv", C.c_int, [C.c_int, dbl, i64, i64, vp, i64, i64, vp, i64, vp, i64])
        rc = f(int(add), alpha, A.shape[0], A.shape[1], _p(A), *_strides(A), _p(x),
               x.strides[0] // 8, _p(y), y.strides[0] // 8)
        if rc:
            raise RuntimeError(f"multmv rc={rc}")

    def tri_ldiveq(self, upper: bool, unit: bool, T: np.ndarray, B: np.ndarray) -> int:
        """B := T^-1 B in place for the upper or lower triangle of T (TriLDivEq);
        returns the status (1: singular, as TMV throws)."""
        f = self._f("tri_ldiveq", C.c_int, [C.c_int, C.c_int, i64, vp, i64, i64, vp, i64, i64])
        if T.strides[0] != 8:
            raise ValueError("the port's tri_ldiveq takes a column-major triangle")
        return f(int(upper), int(unit), T.shape[0], _p(T), max(T.strides[1] // 8, 1), B.shape[1],
                 _p(B), *_strides(B))


class Ref(_Backend):
    prefix = "tmvref_"

    def inverse_z(self, a: np.ndarray) -> np.ndarray:
        """m.inverse() of a complex matrix through LUDiv (LU_Inverse)."""
        A = np.asfortranarray(a, dtype=np.complex128)
        M = np.zeros_like(A, order="F")
        f = self._f("inverse_z", C.c_int, [i64, vp, vp])
        rc = f(A.shape[0], _p(A), _p(M))
        if rc == SINGULAR:
            raise OracleSingular("singular")
        if rc:
            raise RuntimeError(f"inverse_z rc={rc}")
        return M

    def det_z(self, a: np.ndarray):
        """(det, logdet, sign) of a complex matrix through LUDiv."""
        A = np.asfortranarray(a, dtype=np.complex128)
        d, s = np.zeros(2), np.zeros(2)
        ld = C.c_double()
        f = self._f("det_z", C.c_int, [i64, vp, vp, C.POINTER(C.c_double), vp])
        rc = f(A.shape[0], _p(A), _p(d), C.byref(ld), _p(s))
        if rc:
            raise RuntimeError(f"det_z rc={rc}")
        return complex(d[0], d[1]), ld.value, complex(s[0], s[1])

    def _lu(self, A, P):
        if A.shape[0] != A.shape[1]:
            raise ValueError("ref binding factors square matrices")
        f = self._f("lu_decompose", C.c_int, [i64, vp, i64, i64, vp])
        return f(A.shape[0], _p(A), *_strides(A), _p(P))

    def _divide(self, n, A, B, X, LU, P):
        f = self._f("divide", C.c_int, [i64, C.c_int, vp, i64, vp, vp, vp, vp])
        return f(n, 0, _p(A), B.shape[1], _p(B), _p(X), _p(LU), _p(P))

    def rdivide(self, A: np.ndarray, W: np.ndarray) -> np.ndarray:
        """X = W % A (X A = W), W nrows x n."""
        n = A.shape[0]
        A = np.asfortranarray(A)
        W = np.asfortranarray(W)
        X = np.zeros_like(W, order="F")
        f = self._f("rdivide", C.c_int, [i64, vp, i64, vp, vp])
        rc = f(n, _p(A), W.shape[0], _p(W), _p(X))
        if rc:
            raise RuntimeError(f"rdivide rc={rc}")
        return X

    def multmv(self, add: bool, alpha: float, A: np.ndarray, x: np.ndarray, y: np.ndarray) -> None:
        f = self._f("multmv", C.c_int, [C.c_int, dbl, i64, i64, vp, i64, i64, vp, i64, vp, i64])
        rc = f(int(add), alpha, A.shape[0], A.shape[1], _p(A), *_strides(A), _p(x),
               x.strides[0] // 8, _p(y), y.strides[0] // 8)
        if rc:
            raise RuntimeError(f"multmv rc={rc}")

    def tri_ldiveq(self, upper: bool, unit: bool, T: np.ndarray, B: np.ndarray) -> int:
        f = self._f("tri_ldiveq", C.c_int, [C.c_int, C.c_int, i64, vp, i64, i64, i64, vp, i64, i64])
        return f(int(upper), int(unit), T.shape[0], _p(T), *_strides(T), B.shape[1], _p(B),
                 *_strides(B))

    def inverse_of(self, A: np.ndarray):
        """TMV's own m.inverse(), m.makeInverseATA() and m.isSingular()."""
        n = A.shape[0]
        A = np.asfortranarray(A)
        M = np.zeros((n, n), order="F")
        T = np.zeros((n, n), order="F")
        s = C.c_int(0)
        f = self._f("inverse", C.c_int, [i64, vp, vp, vp, C.POINTER(C.c_int)])
        rc = f(n, _p(A), _p(M), _p(T), C.byref(s))
        return rc, M, T, bool(s.value)

    def det_of(self, A: np.ndarray):
        d, ld, s = dbl(), dbl(), dbl()
        A = np.asfortranarray(A)
        f = self._f("det", C.c_int, [i64, vp, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(dbl)])
        rc = f(A.shape[0], _p(A), C.byref(d), C.byref(ld), C.byref(s))
        if rc:
            raise RuntimeError(f"det rc={rc}")
        return d.value, ld.value, s.value


_port = None


def port() -> Port:
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            build_port()
        _port = Port(PORT_LIB)
    return _port


def ref(generic: bool = False) -> Ref:
    return Ref(REF_GENERIC_LIB if generic else REF_LIB)


def ref_available() -> bool:
    return REF_LIB.exists()
