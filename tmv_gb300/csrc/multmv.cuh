// multmv.cuh -- y (+)= alpha A x (tmv::MultMV<add>).
#pragma once

#include "common.cuh"

namespace tmvg {

// y (+)= alpha A x, A m x n with strides (sAi, sAj), x and y with increments;
// x may share storage with y.
tmvg_status multmv(Context* c, bool add, double alpha, int64_t m, int64_t n, const double* A, int64_t sAi,
                   int64_t sAj, const double* x, int64_t incx, double* y, int64_t incy);

}  // namespace tmvg
