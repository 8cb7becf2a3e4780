// lu.cuh -- blocked LU factorisation and LU solves (host entry points).
#pragma once

#include "gemm.cuh"

namespace tmvg {

// In-place P A = L U of an n x n column-major matrix; P (device, n int64).
template <typename T>
tmvg_status lu_factor(Context* c, int64_t n, T* A, int64_t lda, int64_t* P);

// B := T^-1 B for T = the unit-lower (upper = false) or non-unit upper
// (upper = true) triangle stored in (tri, tsi, tsj); B n x nrhs with strides.
// skip_zero: TMV's vector semantics (a zero U(j,j) only matters where the
// entry it divides is nonzero); otherwise every zero U(j,j) is singular.
template <typename T>
tmvg_status tri_solve(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                      bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi,
                      int64_t bsj, bool skip_zero);

// Apply interchanges P[i1..i2) to the rows of B (n x ncols, strides): forward
// (permuteRows) or reverse order (reversePermuteRows).
template <typename T>
tmvg_status apply_pivots(Context* c, int64_t ncols, T* B, int64_t bsi, int64_t bsj,
                         const int64_t* P, int64_t i1, int64_t i2, bool reverse);

// out(i, j) = in(i, j) for strided m x n matrices.
template <typename T>
tmvg_status copy_matrix(Context* c, int64_t m, int64_t n, const T* in, int64_t isi, int64_t isj,
                        T* out, int64_t osi, int64_t osj);

// LU_LDivEq / LU_RDivEq on device data.
template <typename T>
tmvg_status lu_ldiveq(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                      int64_t nrhs, T* B, int64_t bsi, int64_t bsj);
template <typename T>
tmvg_status lu_rdiveq(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                      int64_t nrows, T* B, int64_t bsi, int64_t bsj);

// m /= T for a standalone unit-lower / lower / upper triangle (TriLDivEq).
template <typename T>
tmvg_status tri_ldiveq(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj, bool upper, bool unit,
                       int64_t nrhs, T* B, int64_t bsi, int64_t bsj);

// LU_Inverse: M = A^-1 from the factors (n x n, leading dimension ldm);
// LUDiv::makeInverseATA: M = (A^T A)^-1.
template <typename T>
tmvg_status lu_inverse(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P, T* M, int64_t ldm);
template <typename T>
tmvg_status lu_inverse_ata(Context* c, int64_t n, const T* LU, int64_t lda, T* M, int64_t ldm);

}  // namespace tmvg
