// mixed.cuh -- mixed-precision LU solve with FP64 iterative refinement.
#pragma once

#include "common.cuh"

namespace tmvg {

// X = A^-1 B for column-major FP64 A (n x n) and B (n x nrhs) on the device:
// FP32 factorisation, FP64 residuals and updates, at most max_iter
// refinement steps per column until the normwise backward error <= tol.
tmvg_status lu_solve_mixed(Context* c, int64_t n, const double* A, int64_t lda, int64_t nrhs,
                           const double* B, int64_t ldb, double* X, int64_t ldx, int max_iter,
                           double tol, tmvg_ir_info* info);

}  // namespace tmvg
