"""Tensor-level entry points over the C ABI (device-resident float64 data).

Matrices are torch tensors on a CUDA device.  TMV stores column-major; here a
column-major n x m matrix is a tensor whose stride is (1, ld) with ld >= n,
e.g. ``colmajor(x)``.  Each function names the TMV routine it mirrors.
"""
from __future__ import annotations

import ctypes as C
import threading

import torch

from . import _lib

_handles: dict[int, _lib.Handle] = {}
_lock = threading.Lock()


def handle(device: int | None = None) -> _lib.Handle:
    """The per-device context, bound to torch's current stream."""
    if device is None:
        device = torch.cuda.current_device()
    with _lock:
        h = _handles.get(device)
        if h is None:
            h = _lib.Handle(device)
            _handles[device] = h
    h.set_stream(torch.cuda.current_stream(device).cuda_stream)
    return h


def colmajor(x: torch.Tensor) -> torch.Tensor:
    """A column-major (Fortran-order) copy of a 2-D tensor."""
    return x.t().contiguous().t()


def is_colmajor(x: torch.Tensor) -> bool:
    return x.dim() == 2 and (x.stride(0) == 1 or x.shape[0] <= 1) and (
        x.shape[1] <= 1 or x.stride(1) >= max(x.shape[0], 1))


def _ptr(x: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(x.data_ptr())


def _check_f64_cuda(*ts: torch.Tensor) -> None:
    for t in ts:
        if t.dtype != torch.float64 or not t.is_cuda:
            raise TypeError("expected float64 CUDA tensors")


def _ld(x: torch.Tensor) -> int:
    return max(x.stride(1) if x.shape[1] > 1 else x.shape[0], 1)


def multmm(add: bool, alpha: float, A: torch.Tensor, B: torch.Tensor, C_: torch.Tensor) -> None:
    """C (+)= alpha*A*B in place (tmv::MultMM<add>, src/TMV_MultMM.cpp:405).

    A, B and C are 2-D float64 CUDA tensors with any of TMV's dense layouts
    (column- or row-major strides)."""
    _check_f64_cuda(A, B, C_)
    m, k = A.shape
    k2, n = B.shape
    if k2 != k or tuple(C_.shape) != (m, n):
        raise ValueError("multmm: shape mismatch")
    h = handle(C_.device.index)
    h.check(h.call("tmvg_multmm_f64", int(bool(add)), float(alpha), m, n, k,
                   _ptr(A), A.stride(0), A.stride(1), _ptr(B), B.stride(0), B.stride(1),
                   _ptr(C_), C_.stride(0), C_.stride(1)), "multmm")


def lu_decompose(A: torch.Tensor, P: torch.Tensor | None = None) -> torch.Tensor:
    """In-place P A = L U of a column-major square A; returns the int64
    interchange vector (tmv::LU_Decompose, src/TMV_LUDecompose.cpp:514)."""
    _check_f64_cuda(A)
    n = A.shape[0]
    if A.shape[1] != n or not is_colmajor(A):
        raise ValueError("lu_decompose: A must be square and column-major")
    if P is None:
        P = torch.empty(n, dtype=torch.int64, device=A.device)
    h = handle(A.device.index)
    h.check(h.call("tmvg_lu_decompose_f64", n, _ptr(A), _ld(A), _ptr(P)), "lu_decompose")
    return P


def lu_ldiveq(LU: torch.Tensor, P: torch.Tensor, B: torch.Tensor) -> None:
    """B := (P L U)^-1 B in place (tmv::LU_LDivEq, src/TMV_LUDiv.cpp:186)."""
    _check_f64_cuda(LU, B)
    n = LU.shape[0]
    if B.dim() == 1:
        B = B.view(-1, 1)
    if B.shape[0] != n or not is_colmajor(B) or not is_colmajor(LU):
        raise ValueError("lu_ldiveq: B must be column-major n x nrhs")
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_ldiveq_f64", n, _ptr(LU), _ld(LU), _ptr(P), B.shape[1], _ptr(B),
                   _ld(B)), "lu_ldiveq")


def _check_z_cuda(*ts: torch.Tensor) -> None:
    for t in ts:
        if not (t.is_cuda and t.dtype == torch.complex128):
            raise TypeError("complex128 CUDA tensors required")


def lu_decompose_z(A: torch.Tensor) -> torch.Tensor:
    """LU_Decompose of a column-major complex128 n x n CUDA tensor in place
    (tmvg_lu_decompose_z64, TMV's complex<double> instantiation); returns
    the int64 interchanges."""
    _check_z_cuda(A)
    n = A.shape[0]
    if A.shape[1] != n or not is_colmajor(A):
        raise ValueError("lu_decompose_z: A must be a column-major square matrix")
    P = torch.empty(n, dtype=torch.int64, device=A.device)
    h = handle(A.device.index)
    h.check(h.call("tmvg_lu_decompose_z64", n, _ptr(A), _ld(A), _ptr(P)), "lu_decompose_z")
    return P


def lu_ldiveq_z(LU: torch.Tensor, P: torch.Tensor, B: torch.Tensor) -> None:
    """B := (P L U)^-1 B for complex128 column-major CUDA tensors
    (tmvg_lu_ldiveq_z64); raises SingularError like TMV."""
    _check_z_cuda(LU, B)
    n = LU.shape[0]
    if B.dim() != 2 or B.shape[0] != n or not is_colmajor(B) or not is_colmajor(LU):
        raise ValueError("lu_ldiveq_z: B must be column-major n x nrhs")
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_ldiveq_z64", n, _ptr(LU), _ld(LU), _ptr(P), B.shape[1], _ptr(B), _ld(B)),
            "lu_ldiveq_z")


def lu_rdiveq_z(LU: torch.Tensor, P: torch.Tensor, B: torch.Tensor) -> None:
    """B (nrows x n) := B (P L U)^-1 for complex128 column-major CUDA tensors
    (tmvg_lu_rdiveq_z64, TMV's b % m); raises SingularError like TMV."""
    _check_z_cuda(LU, B)
    n = LU.shape[0]
    if B.dim() != 2 or B.shape[1] != n or not is_colmajor(B) or not is_colmajor(LU):
        raise ValueError("lu_rdiveq_z: B must be column-major nrows x n")
    h = handle(LU.device.index)
    ldb = max(B.stride(1) if B.shape[1] > 1 else B.shape[0], 1)
    h.check(h.call("tmvg_lu_rdiveq_z64", n, _ptr(LU), _ld(LU), _ptr(P), B.shape[0], _ptr(B), ldb),
            "lu_rdiveq_z")


def lu_inverse_z(LU: torch.Tensor, P: torch.Tensor) -> torch.Tensor:
    """m.inverse() from complex128 factors (tmvg_lu_inverse_z64): a new
    column-major n x n tensor; raises SingularError like TMV."""
    _check_z_cuda(LU)
    n = LU.shape[0]
    M = torch.empty((n, n), dtype=torch.complex128, device=LU.device).t()
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_inverse_z64", n, _ptr(LU), _ld(LU), _ptr(P), _ptr(M), max(n, 1)), "lu_inverse_z")
    return M


def lu_det_z(LU: torch.Tensor, P: torch.Tensor):
    """(det, logdet, sign) of the matrix factored in LU (complex128), as
    LUDiv::det / logDet (tmvg_lu_det_z64)."""
    import numpy as np

    _check_z_cuda(LU)
    d, s = np.zeros(2), np.zeros(2)
    ld = C.c_double()
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_det_z64", LU.shape[0], _ptr(LU), _ld(LU), _ptr(P), C.c_void_p(d.ctypes.data),
                   C.byref(ld), C.c_void_p(s.ctypes.data)), "lu_det_z")
    return complex(d[0], d[1]), ld.value, complex(s[0], s[1])


def lu_rdiveq(LU: torch.Tensor, P: torch.Tensor, B: torch.Tensor) -> None:
    """B := B (P L U)^-1 in place (tmv::LU_RDivEq, src/TMV_LUDiv.cpp:370)."""
    _check_f64_cuda(LU, B)
    n = LU.shape[0]
    if B.dim() == 1:
        B = B.view(1, -1)
    if B.shape[1] != n or not is_colmajor(B) or not is_colmajor(LU):
        raise ValueError("lu_rdiveq: B must be column-major nrows x n")
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_rdiveq_f64", n, _ptr(LU), _ld(LU), _ptr(P), B.shape[0], _ptr(B),
                   _ld(B)), "lu_rdiveq")


def divide(A: torch.Tensor, B: torch.Tensor):
    """X = B/A with the LU of a copy of A (LUDiv<double>, src/TMV_LUD.cpp:74-120).

    Returns (X, LU, P); LU and P can be reused for further solves."""
    _check_f64_cuda(A, B)
    n = A.shape[0]
    if B.dim() == 1:
        B = B.view(-1, 1)
    nrhs = B.shape[1]
    if not is_colmajor(A):
        A = colmajor(A)
    if not is_colmajor(B):
        B = colmajor(B)
    LU = torch.empty((n, n), dtype=torch.float64, device=A.device).t()
    X = torch.empty((nrhs, n), dtype=torch.float64, device=A.device).t()
    P = torch.empty(n, dtype=torch.int64, device=A.device)
    h = handle(A.device.index)
    h.check(h.call("tmvg_divide_f64", n, _ptr(A), _ld(A), nrhs, _ptr(B), _ld(B), _ptr(X),
                   max(n, 1), _ptr(LU), _ptr(P)), "divide")
    return X, LU, P


def lu_det(LU: torch.Tensor, P: torch.Tensor):
    """(det, logdet, sign) of stored factors (LUDiv::det/logDet, src/TMV_LUD.cpp:132-156)."""
    _check_f64_cuda(LU)
    n = LU.shape[0]
    d, ld, s = C.c_double(), C.c_double(), C.c_double()
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_det_f64", n, _ptr(LU), _ld(LU), _ptr(P), C.byref(d), C.byref(ld),
                   C.byref(s)), "lu_det")
    return d.value, ld.value, s.value


def multmv(add: bool, alpha: float, A: torch.Tensor, x: torch.Tensor, y: torch.Tensor) -> None:
    """y (+)= alpha A x in place (tmv::MultMV<add>, src/TMV_MultMV.cpp:1134-1175).

    A is a 2-D float64 CUDA tensor with any strides, x and y 1-D (any
    stride); x may be y itself."""
    _check_f64_cuda(A, x, y)
    m, n = A.shape
    if x.dim() != 1 or y.dim() != 1 or x.shape[0] != n or y.shape[0] != m:
        raise ValueError("multmv: size mismatch")
    h = handle(A.device.index)
    h.check(h.call("tmvg_multmv_f64", int(add), float(alpha), m, n, _ptr(A), A.stride(0), A.stride(1),
                   _ptr(x), x.stride(0), _ptr(y), y.stride(0)), "multmv")


def tri_ldiveq(T: torch.Tensor, upper: bool, unit: bool, B: torch.Tensor) -> None:
    """B := T^-1 B in place for the upper or lower triangle of T (m /= U,
    m /= L: TriLDivEq, src/TMV_TriDiv_M.cpp:583-710).  Raises SingularError
    where TMV throws SingularUpper/LowerTriMatrix."""
    _check_f64_cuda(T, B)
    n = T.shape[0]
    if B.dim() == 1:
        B = B.view(-1, 1)
    if T.shape[1] != n or B.shape[0] != n:
        raise ValueError("tri_ldiveq: size mismatch")
    h = handle(T.device.index)
    h.check(h.call("tmvg_tri_ldiveq_f64", int(upper), int(unit), n, _ptr(T), T.stride(0), T.stride(1),
                   B.shape[1], _ptr(B), B.stride(0), B.stride(1)), "tri_ldiveq")


def tri_rdiveq(T: torch.Tensor, upper: bool, unit: bool, B: torch.Tensor) -> None:
    """B := B T^-1 in place (m %= U, m %= L); B is nrows x n."""
    _check_f64_cuda(T, B)
    n = T.shape[0]
    if B.dim() == 1:
        B = B.view(1, -1)
    if T.shape[1] != n or B.shape[1] != n:
        raise ValueError("tri_rdiveq: size mismatch")
    h = handle(T.device.index)
    h.check(h.call("tmvg_tri_rdiveq_f64", int(upper), int(unit), n, _ptr(T), T.stride(0), T.stride(1),
                   B.shape[0], _ptr(B), B.stride(0), B.stride(1)), "tri_rdiveq")


def lu_inverse(LU: torch.Tensor, P: torch.Tensor) -> torch.Tensor:
    """A^-1 from stored factors, column-major (LU_Inverse, src/TMV_LUInverse.cpp:236-299)."""
    _check_f64_cuda(LU)
    n = LU.shape[0]
    M = torch.empty((n, n), dtype=torch.float64, device=LU.device).t()
    if n == 0:
        return M
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_inverse_f64", n, _ptr(LU), _ld(LU), _ptr(P), _ptr(M), _ld(M)),
            "lu_inverse")
    return M


def lu_inverse_ata(LU: torch.Tensor) -> torch.Tensor:
    """(A^T A)^-1 from stored factors (LUDiv::makeInverseATA, src/TMV_LUD.cpp:172-200)."""
    _check_f64_cuda(LU)
    n = LU.shape[0]
    M = torch.empty((n, n), dtype=torch.float64, device=LU.device).t()
    if n == 0:
        return M
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_inverse_ata_f64", n, _ptr(LU), _ld(LU), _ptr(M), _ld(M)),
            "lu_inverse_ata")
    return M


def lu_is_singular(LU: torch.Tensor) -> bool:
    """LUDiv::isSingular (src/TMV_LUD.cpp:204-209): min |U_jj| <= eps * max |U_jj|."""
    _check_f64_cuda(LU)
    s = C.c_int(0)
    h = handle(LU.device.index)
    h.check(h.call("tmvg_lu_is_singular_f64", LU.shape[0], _ptr(LU), _ld(LU), C.byref(s)),
            "lu_is_singular")
    return bool(s.value)


def solve_mixed(A: torch.Tensor, B: torch.Tensor, max_iter: int = 10, tol: float = 1e-12,
                X: torch.Tensor | None = None, raise_not_converged: bool = True):
    """X = A^-1 B by FP32 LU + FP64 iterative refinement (tmvg_lu_solve_mixed_f64).

    Returns (X, info) where info has iterations, converged, backward_error,
    anorm_inf.  Raises TmvgError(NOT_CONVERGED) unless raise_not_converged is
    False."""
    _check_f64_cuda(A, B)
    n = A.shape[0]
    if B.dim() == 1:
        B = B.view(-1, 1)
    if not is_colmajor(A):
        A = colmajor(A)
    if not is_colmajor(B):
        B = colmajor(B)
    nrhs = B.shape[1]
    if X is None:
        X = torch.empty((nrhs, n), dtype=torch.float64, device=A.device).t()
    info = _lib.IRInfo()
    h = handle(A.device.index)
    st = h.call("tmvg_lu_solve_mixed_f64", n, _ptr(A), _ld(A), nrhs, _ptr(B), _ld(B), _ptr(X),
                _ld(X), int(max_iter), float(tol), C.byref(info))
    if st == 2 and not raise_not_converged:
        return X, info
    h.check(st, "solve_mixed")
    return X, info
