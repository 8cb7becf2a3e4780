// zlu.cuh -- LU_Decompose / LU_LDivEq for std::complex<double> (entries as
// double2: real, imaginary; column-major).
#pragma once

#include "common.cuh"

#include <cfloat>
#include <cmath>
#include <cstdint>

namespace tmvg {

tmvg_status zlu_factor(Context* c, int64_t n, double2* A, int64_t lda, int64_t* P);
tmvg_status zlu_ldiveq(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, int64_t nrhs,
                       double2* B, int64_t ldb);
tmvg_status zlu_rdiveq(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, int64_t nrows,
                       double2* B, int64_t ldb);
tmvg_status zlu_inverse(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, double2* M,
                        int64_t ldm);

}  // namespace tmvg
