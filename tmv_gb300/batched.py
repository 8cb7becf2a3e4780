"""Batched uneven LU solves over the C ABI (tmvg_batch_plan_*).

    plan = BatchPlan(n, nrhs)               # host int arrays; packed layout
    A, B = plan.alloc()                     # device buffers of the right size
    ... fill A (A_s column-major at plan.a_off[s]) and B ...
    P, status = plan.solve(A, B)            # one graph launch: X_s over B_s
    P, status, iters, berr = plan.solve_mixed(A, B)   # FP32 factors + FP64 refinement

Mirrors a loop of TMV's B_s / A_s (LUDiv<double>, src/TMV_LUD.cpp:74-120)
over independent systems.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .linalg import handle


class BatchPlan:
    def __init__(self, n, nrhs, a_off=None, b_off=None, tune: bool = True, device=None):
        self.h = handle(device)
        self.n = np.ascontiguousarray(n, dtype=np.int64)
        self.nrhs = np.ascontiguousarray(nrhs, dtype=np.int64)
        self.count = len(self.n)
        ao = None if a_off is None else np.ascontiguousarray(a_off, dtype=np.int64)
        bo = None if b_off is None else np.ascontiguousarray(b_off, dtype=np.int64)
        self.a_off = ao if ao is not None else np.concatenate(
            [[0], np.cumsum(self.n * self.n)[:-1]]).astype(np.int64)
        self.b_off = bo if bo is not None else np.concatenate(
            [[0], np.cumsum(self.n * self.nrhs)[:-1]]).astype(np.int64)
        self.p_off = np.concatenate([[0], np.cumsum(self.n)[:-1]]).astype(np.int64)
        plan = C.c_void_p()
        self.h.check(self.h.call(
            "tmvg_batch_plan_create", self.count, C.c_void_p(self.n.ctypes.data),
            C.c_void_p(self.nrhs.ctypes.data),
            None if ao is None else C.c_void_p(ao.ctypes.data),
            None if bo is None else C.c_void_p(bo.ctypes.data), int(bool(tune)), C.byref(plan)),
            "batch plan")
        self.plan = plan
        ae, be, pe, fl = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        pw = (C.c_int * 4)()
        self.h.check(self.h.lib.tmvg_batch_plan_info(plan, C.byref(ae), C.byref(be), C.byref(pe),
                                                     C.byref(fl), pw))
        self.a_elems, self.b_elems, self.p_elems = ae.value, be.value, pe.value
        self.flops = fl.value
        self.panel_widths = list(pw)

    def set_tiles(self, widths) -> None:
        pw = (C.c_int * 4)(*widths)
        self.h.check(self.h.lib.tmvg_batch_plan_set_tiles(self.plan, pw))
        self.panel_widths = list(widths)

    def alloc(self, device=None):
        dev = device or torch.device("cuda", self.h.device)
        A = torch.empty(max(self.a_elems, 1), dtype=torch.float64, device=dev)
        B = torch.empty(max(self.b_elems, 1), dtype=torch.float64, device=dev)
        return A, B

    def solve(self, A: torch.Tensor, B: torch.Tensor, P: torch.Tensor | None = None,
              status: torch.Tensor | None = None):
        if P is None:
            P = torch.empty(max(self.p_elems, 1), dtype=torch.int64, device=A.device)
        if status is None:
            status = torch.empty(max(self.count, 1), dtype=torch.int32, device=A.device)
        self.h.set_stream(torch.cuda.current_stream(A.device).cuda_stream)
        self.h.check(self.h.lib.tmvg_batched_lu_solve_f64(
            self.plan, C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
            C.c_void_p(P.data_ptr()), C.c_void_p(status.data_ptr())), "batched solve")
        return P, status

    def solve_mixed(self, A: torch.Tensor, B: torch.Tensor, max_iter: int = 10, tol: float = 1e-12,
                    P: torch.Tensor | None = None, status: torch.Tensor | None = None):
        """X_s = A_s^-1 B_s with FP32 factors and FP64 refinement, one graph
        launch (tmvg_batched_lu_solve_mixed_f64).  A is left unchanged; B
        receives X.  Returns (P, status, iters, berr): status 0 converged, 1
        singular FP32 factors, 2 not converged."""
        dev = A.device
        if P is None:
            P = torch.empty(max(self.p_elems, 1), dtype=torch.int64, device=dev)
        if status is None:
            status = torch.empty(max(self.count, 1), dtype=torch.int32, device=dev)
        iters = torch.empty(max(self.count, 1), dtype=torch.int32, device=dev)
        berr = torch.empty(max(self.count, 1), dtype=torch.float64, device=dev)
        self.h.set_stream(torch.cuda.current_stream(dev).cuda_stream)
        self.h.check(self.h.lib.tmvg_batched_lu_solve_mixed_f64(
            self.plan, C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), C.c_void_p(P.data_ptr()),
            C.c_void_p(status.data_ptr()), int(max_iter), float(tol), C.c_void_p(iters.data_ptr()),
            C.c_void_p(berr.data_ptr())), "batched mixed solve")
        return P, status, iters, berr

    def close(self) -> None:
        if getattr(self, "plan", None):
            self.h.lib.tmvg_batch_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
