// gemm.cuh -- host entry of the dense products used by MultMM, the LU
// trailing updates and the blocked triangular solves.
#pragma once

#include "common.cuh"

namespace tmvg {

// A strided operand: element (i, j) at p[i*si + j*sj].
template <typename T>
struct Mat {
    T* p;
    int64_t si, sj;
};

// C (+)= alpha * A * B with A m x k, B k x n, C m x n; each operand column- or
// row-major (si == 1 or sj == 1).  beta is 0 (overwrite) or 1 (accumulate).
// Returns TMVG_BAD_ARG for any other stride pattern.
template <typename T>
tmvg_status gemm(Context* c, int64_t m, int64_t n, int64_t k, T alpha,
                 Mat<const T> A, Mat<const T> B, T beta, Mat<T> C);

}  // namespace tmvg
