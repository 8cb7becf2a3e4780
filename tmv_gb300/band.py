"""Batched band LU over the C ABI (device-resident float64 data).

A batch holds `count` n x n band systems of one shape, lo subdiagonals and hi
superdiagonals, in TMV's column-major band storage: system s's element (i,j)
at ``ab[s*stride_ab + i + j*ldab]`` for ``j-hu <= i <= j+lo`` with
``hu = min(lo+hi, n-1)`` (the superdiagonals the interchanges fill) and
``ldab >= lo + hu``.  ``band_layout`` gives the packed defaults.

The calls mirror, per system, tmv::LU_Decompose(BandMatrixView<double>, P,
Anhi) (src/TMV_BandLUDecompose.cpp:383-425) and tmv::LU_LDivEq / LU_RDivEq
on band factors (src/TMV_BandLUDiv.cpp:811-851), bit for bit;
``algo="tridiag"`` runs TMV's tridiagonal algorithm, the one BandLUDiv uses
for lo == hi == 1.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from .linalg import _ptr, handle

ALGOS = {"general": 0, "tridiag": 1}


@dataclass(frozen=True)
class BandLayout:
    n: int
    lo: int
    hi: int
    hu: int
    ldab: int
    stride_ab: int

    @property
    def slots(self) -> int:
        """Band slots of one system from (0,0) to (n-1,n-1)."""
        return (self.n - 1) * (self.ldab + 1) + 1 if self.n > 0 else 0


def band_layout(n: int, lo: int, hi: int, ldab: int | None = None,
                stride_ab: int | None = None) -> BandLayout:
    """The packed layout: ldab = lo + hu, stride_ab = n (ldab + 1)."""
    hu = min(lo + hi, n - 1) if n > 0 else 0
    ldab = max(lo + hu, 1) if ldab is None else ldab
    stride_ab = n * (ldab + 1) if stride_ab is None else stride_ab
    return BandLayout(n, lo, hi, hu, ldab, stride_ab)


def _check(t: torch.Tensor, dtype: torch.dtype, what: str) -> None:
    if t.dtype != dtype or not t.is_cuda or not t.is_contiguous():
        raise TypeError(f"{what}: expected a contiguous {dtype} CUDA tensor")


def _algo(algo: str) -> int:
    try:
        return ALGOS[algo]
    except KeyError:
        raise ValueError(f"algo must be one of {sorted(ALGOS)}") from None


def band_lu_decompose(ab: torch.Tensor, count: int, lay: BandLayout, P: torch.Tensor,
                      stride_p: int | None = None, algo: str = "general") -> None:
    """Factor every system of ab in place; P (int64) receives the
    interchanges, system s's at P[s*stride_p ...]."""
    _check(ab, torch.float64, "ab")
    _check(P, torch.int64, "P")
    h = handle(ab.device.index)
    h.check(h.lib.tmvg_band_lu_decompose_batched_f64(
        h.h, count, lay.n, lay.lo, lay.hi, _algo(algo), _ptr(ab), lay.ldab, lay.stride_ab,
        _ptr(P), lay.n if stride_p is None else stride_p), "band_lu_decompose")


def band_lu_ldiveq(ab: torch.Tensor, count: int, lay: BandLayout, P: torch.Tensor,
                   B: torch.Tensor, nrhs: int, ldb: int | None = None, stride_b: int | None = None,
                   stride_p: int | None = None, algo: str = "general",
                   status: torch.Tensor | None = None) -> torch.Tensor:
    """B := (P L U)^-1 B for every system from its band factors; B holds
    system s's n x nrhs column-major block at B[s*stride_b ...].  Returns the
    per-system status (int32: 0, 1 singular, 2 interchange outside the band)."""
    _check(ab, torch.float64, "ab")
    _check(P, torch.int64, "P")
    _check(B, torch.float64, "B")
    ldb = lay.n if ldb is None else ldb
    stride_b = ldb * nrhs if stride_b is None else stride_b
    if status is None:
        status = torch.empty(count, dtype=torch.int32, device=ab.device)
    h = handle(ab.device.index)
    h.check(h.lib.tmvg_band_lu_ldiveq_batched_f64(
        h.h, count, lay.n, lay.lo, lay.hi, _algo(algo), _ptr(ab), lay.ldab, lay.stride_ab,
        _ptr(P), lay.n if stride_p is None else stride_p, nrhs, _ptr(B), ldb, stride_b,
        _ptr(status)), "band_lu_ldiveq")
    return status


def band_lu_rdiveq(ab: torch.Tensor, count: int, lay: BandLayout, P: torch.Tensor,
                   M: torch.Tensor, nrhs: int, ldb: int | None = None, stride_b: int | None = None,
                   stride_p: int | None = None, algo: str = "general",
                   status: torch.Tensor | None = None) -> torch.Tensor:
    """M := M (P L U)^-1 for every system from its band factors (x A = m,
    TMV's LU_RDivEq); M holds system s's nrhs x n block with row q at
    M[s*stride_b + q*ldb ...] (each row contiguous).  Returns the per-system
    status as band_lu_ldiveq does."""
    _check(ab, torch.float64, "ab")
    _check(P, torch.int64, "P")
    _check(M, torch.float64, "M")
    ldb = lay.n if ldb is None else ldb
    stride_b = ldb * nrhs if stride_b is None else stride_b
    if status is None:
        status = torch.empty(count, dtype=torch.int32, device=ab.device)
    h = handle(ab.device.index)
    h.check(h.lib.tmvg_band_lu_rdiveq_batched_f64(
        h.h, count, lay.n, lay.lo, lay.hi, _algo(algo), _ptr(ab), lay.ldab, lay.stride_ab,
        _ptr(P), lay.n if stride_p is None else stride_p, nrhs, _ptr(M), ldb, stride_b,
        _ptr(status)), "band_lu_rdiveq")
    return status


def band_lu_solve(ab: torch.Tensor, count: int, lay: BandLayout, B: torch.Tensor, nrhs: int,
                  ldb: int | None = None, stride_b: int | None = None, algo: str = "general",
                  P: torch.Tensor | None = None,
                  status: torch.Tensor | None = None) -> tuple[torch.Tensor, torch.Tensor]:
    """Factor and solve in one launch (x = b / A per system).  ab receives
    the factors, B the solutions; returns (P, status)."""
    _check(ab, torch.float64, "ab")
    _check(B, torch.float64, "B")
    ldb = lay.n if ldb is None else ldb
    stride_b = ldb * nrhs if stride_b is None else stride_b
    if P is None:
        P = torch.empty(count * max(lay.n, 1), dtype=torch.int64, device=ab.device)
    if status is None:
        status = torch.empty(count, dtype=torch.int32, device=ab.device)
    h = handle(ab.device.index)
    h.check(h.lib.tmvg_band_lu_solve_batched_f64(
        h.h, count, lay.n, lay.lo, lay.hi, _algo(algo), _ptr(ab), lay.ldab, lay.stride_ab,
        _ptr(P), lay.n, nrhs, _ptr(B), ldb, stride_b, _ptr(status)), "band_lu_solve")
    return P, status


def band_divide(ab: torch.Tensor, count: int, lay: BandLayout, B: torch.Tensor, nrhs: int,
                ldb: int | None = None, stride_b: int | None = None, lu: torch.Tensor | None = None,
                P: torch.Tensor | None = None, status: torch.Tensor | None = None):
    """X = A^-1 B per system as TMV's BandLUDiv computes it (B /= A for a
    tmv::BandMatrix): the tridiagonal algorithm for lo == hi == 1, A's
    transpose factored and the columns of B solved as rows (LU_RDivEq) when
    hi < lo.  ab holds A's band in lay (only diagonals -lo..hi are read; ab
    is not modified); B is solved in place.  Returns (lu, lu_layout, P,
    status, transposed): the factors (of A^T when transposed)."""
    _check(ab, torch.float64, "ab")
    _check(B, torch.float64, "B")
    n, lo, hi = lay.n, lay.lo, lay.hi
    trans = hi < lo
    lay_lu = band_layout(n, min(lo, hi), lo if trans else hi)
    if lu is None:
        lu = torch.empty(max(count * lay_lu.stride_ab, 1), dtype=torch.float64, device=ab.device)
    _check(lu, torch.float64, "lu")
    ldb = n if ldb is None else ldb
    stride_b = ldb * nrhs if stride_b is None else stride_b
    if P is None:
        P = torch.empty(count * max(n, 1), dtype=torch.int64, device=ab.device)
    if status is None:
        status = torch.empty(count, dtype=torch.int32, device=ab.device)
    h = handle(ab.device.index)
    h.check(h.lib.tmvg_band_divide_batched_f64(
        h.h, count, n, lo, hi, _ptr(ab), lay.ldab, lay.stride_ab, _ptr(lu), lay_lu.ldab,
        lay_lu.stride_ab, _ptr(P), n, nrhs, _ptr(B), ldb, stride_b, _ptr(status)), "band_divide")
    return lu, lay_lu, P, status, trans


def band_lu_solve_count(count: int, lay: BandLayout, nrhs: int) -> dict:
    """Algorithmic work of one band_lu_solve over the batch: FP64 operations
    of the general algorithm (per step a reciprocal, lo scalings, lo hu
    products and differences; per right-hand side and step lo + hu products
    and differences and a division) and the bytes of the band, P and B read
    or written once."""
    n, lo, hu = lay.n, lay.lo, lay.hu
    band = sum(min(lo, n - 1 - j) + 1 + min(hu, n - 1 - j) for j in range(n)) if n < 4096 else \
        n * (lo + hu + 1)
    flops = count * (n * (1 + lo + 2 * lo * hu) + nrhs * n * (2 * (lo + hu) + 1))
    byts = count * (8 * 2 * band + 8 * n + 8 * 2 * n * nrhs)
    return {"flops": float(flops), "bytes": float(byts)}


__all__ = ["BandLayout", "band_divide", "band_layout", "band_lu_decompose", "band_lu_ldiveq",
           "band_lu_rdiveq", "band_lu_solve", "band_lu_solve_count"]
