"""Differentiable X = A^-1 B over the C ABI forward/backward pair.

    X = lu_solve(A, B)            # torch.autograd.Function
    L = (W * X).sum(); L.backward()
    A.grad == -(A^-T W) X^T ;  B.grad == A^-T W

The forward factors A once (tmvg_lu_solve_fwd_f64) and saves LU, P and X;
the backward (tmvg_lu_solve_bwd_f64) reuses them: gB by the transpose solve
(TMV's LU_RDivEq, src/TMV_LUDiv.cpp:370-411), gA = -gB X^T by an FP64
outer-product GEMM.
"""
from __future__ import annotations

import torch

from .linalg import _check_f64_cuda, _ld, _ptr, colmajor, handle, is_colmajor


def solve_fwd(A: torch.Tensor, B: torch.Tensor):
    _check_f64_cuda(A, B)
    n = A.shape[0]
    if not is_colmajor(A):
        A = colmajor(A)
    if not is_colmajor(B):
        B = colmajor(B)
    nrhs = B.shape[1]
    X = torch.empty((nrhs, n), dtype=torch.float64, device=A.device).t()
    LU = torch.empty((n, n), dtype=torch.float64, device=A.device).t()
    P = torch.empty(n, dtype=torch.int64, device=A.device)
    h = handle(A.device.index)
    h.check(h.call("tmvg_lu_solve_fwd_f64", n, _ptr(A), _ld(A), nrhs, _ptr(B), _ld(B), _ptr(X),
                   max(n, 1), _ptr(LU), _ptr(P)), "lu_solve_fwd")
    return X, LU, P


def solve_bwd(LU, P, X, G, need_gA: bool = True, need_gB: bool = True):
    n, nrhs = X.shape
    if not is_colmajor(G):
        G = colmajor(G)
    gB = torch.empty((nrhs, n), dtype=torch.float64, device=X.device).t() if need_gB else None
    gA = torch.empty((n, n), dtype=torch.float64, device=X.device).t() if need_gA else None
    h = handle(X.device.index)
    h.check(h.call("tmvg_lu_solve_bwd_f64", n, _ptr(LU), _ld(LU), _ptr(P), nrhs, _ptr(X), _ld(X),
                   _ptr(G), _ld(G), _ptr(gB) if gB is not None else None, max(n, 1),
                   _ptr(gA) if gA is not None else None, max(n, 1)), "lu_solve_bwd")
    return gA, gB


class LUSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, B):
        squeeze = B.dim() == 1
        B2 = B.view(-1, 1) if squeeze else B
        X, LU, P = solve_fwd(A.detach(), B2.detach())
        ctx.save_for_backward(LU, P, X)
        ctx.squeeze = squeeze
        return X.view(-1) if squeeze else X

    @staticmethod
    def backward(ctx, G):
        LU, P, X = ctx.saved_tensors
        G2 = G.reshape(-1, 1) if ctx.squeeze else G
        gA, gB = solve_bwd(LU, P, X, G2.to(torch.float64), ctx.needs_input_grad[0],
                           ctx.needs_input_grad[1] or ctx.needs_input_grad[0])
        if gB is not None and ctx.squeeze:
            gB = gB.view(-1)
        return gA, (gB if ctx.needs_input_grad[1] else None)


def lu_solve(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    return LUSolve.apply(A, B)
