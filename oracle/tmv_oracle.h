/* tmv_oracle.h -- CPU restatement of TMV 0.76's dense hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load
 * it; the product (tmv_gb300/) never does.
 *
 * Every routine follows the reference algorithm step for step (same recursion
 * splits, same pivot rule, same dispatch thresholds); each definition in
 * tmv_oracle.c cites the reference file:line it restates.  Matrices are
 * double precision, addressed by (stepi, stepj) strides like tmv::MatrixView,
 * indices and pivots are ptrdiff_t (0-based LAPACK-style interchanges).
 */
#ifndef TMV_ORACLE_H
#define TMV_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes shared by all routines. */
#define ORACLE_OK 0
#define ORACLE_SINGULAR 1 /* TMV would throw SingularUpper/LowerTriMatrix */
#define ORACLE_BAD_ARG 2
#define ORACLE_NOMEM 3

void oracle_set_threads(int nthreads);
int oracle_max_threads(void);

/* C (+)= alpha * A * B  (MultMM<add>).  A m x k, B k x n, C m x n. */
int oracle_multmm(int add, double alpha, ptrdiff_t m, ptrdiff_t n, ptrdiff_t k,
                  const double* A, ptrdiff_t sAi, ptrdiff_t sAj,
                  const double* B, ptrdiff_t sBi, ptrdiff_t sBj,
                  double* C, ptrdiff_t sCi, ptrdiff_t sCj);

/* In-place PA = LU of an m x n matrix (LU_Decompose).  P has min(m,n)
 * entries.  Never fails (underflowed pivots zero their column). */
int oracle_lu_decompose(ptrdiff_t m, ptrdiff_t n, double* A, ptrdiff_t sAi,
                        ptrdiff_t sAj, ptrdiff_t* P);

/* B := (unit-lower L)^-1 B  or  B := U^-1 B with L/U stored in LU
 * (column-major n x n, leading dimension lda); B n x nrhs with strides. */
int oracle_tri_ldiveq(int upper, int unitdiag, ptrdiff_t n, const double* LU,
                      ptrdiff_t lda, ptrdiff_t nrhs, double* B, ptrdiff_t sBi,
                      ptrdiff_t sBj);

/* LU_LDivEq: B := (P L U)^-1 B, B n x nrhs. */
int oracle_lu_ldiveq(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                     const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                     ptrdiff_t sBi, ptrdiff_t sBj);

/* LU_RDivEq: B := B (P L U)^-1, B nrows x n. */
int oracle_lu_rdiveq(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                     const ptrdiff_t* P, ptrdiff_t nrows, double* B,
                     ptrdiff_t sBi, ptrdiff_t sBj);

/* The user-level X = B / A for a column-major A (copied, as LUDiv does).
 * LU_out / P_out may be NULL. */
int oracle_divide(ptrdiff_t n, const double* A, ptrdiff_t nrhs,
                  const double* B, double* X, double* LU_out, ptrdiff_t* P_out);

/* det and logDet of LU factors (LUDiv::det / logDet). */
void oracle_lu_det(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                   const ptrdiff_t* P, double* det, double* logdet,
                   double* sign);

/* LU_Inverse: M = A^-1 from the factors (U^-1 L^-1, columns reverse-
 * permuted).  ORACLE_SINGULAR for a zero U_jj. */
int oracle_lu_inverse(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                      const ptrdiff_t* P, double* M, ptrdiff_t ldm);

/* LUDiv::makeInverseATA: M = (A^T A)^-1 from the factors. */
int oracle_lu_inverse_ata(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                          double* M, ptrdiff_t ldm);

/* LUDiv::isSingular: 1 when min |U_jj| <= epsilon * max |U_jj|. */
int oracle_lu_is_singular(ptrdiff_t n, const double* LU, ptrdiff_t lda);

/* MultMV<add>: y (+)= alpha A x (A m x n, strides; x, y increments). */
int oracle_multmv(int add, double alpha, ptrdiff_t m, ptrdiff_t n, const double* A,
                  ptrdiff_t sAi, ptrdiff_t sAj, const double* x, ptrdiff_t incx,
                  double* y, ptrdiff_t incy);

/* Ragged batch of X_i = B_i / A_i (B_i overwritten), OpenMP over systems. */
int oracle_batched_divide(ptrdiff_t count, const ptrdiff_t* n,
                          const ptrdiff_t* nrhs, const ptrdiff_t* a_off,
                          const ptrdiff_t* b_off, const double* A, double* B,
                          int* status);

/* Band LU (tmv_oracle_band.c): TMV's column-major band storage, element
 * (i,j) at a[i + j*ldab] for j-hu <= i <= j+lo, hu = min(lo+hi, n-1)
 * superdiagonals (the interchanges fill them; ldab >= lo + hu).
 * LU_Decompose(BandMatrixView) in place, P[0..n); and LU_LDivEq on the
 * factors for B (n x nrhs, leading dimension ldb).  algo picks TMV's general
 * band algorithm or its tridiagonal one (lo = hi = 1). */
#define ORACLE_BAND_GENERAL 0
#define ORACLE_BAND_TRIDIAG 1
int oracle_band_lu_decompose(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, double* a,
                             ptrdiff_t ldab, ptrdiff_t* P);
int oracle_band_lu_ldiveq(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, const double* lu,
                          ptrdiff_t ldab, const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                          ptrdiff_t ldb);
/* x P L U = m for the nrhs rows of m (row q at B + q*ldb), in place. */
int oracle_band_lu_rdiveq(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, const double* lu,
                          ptrdiff_t ldab, const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                          ptrdiff_t ldb);
/* count systems of one shape, OpenMP over systems (system s at ab + s*sab,
 * P + s*sp, B + s*sb); status[s] per system. */
int oracle_band_batched_solve(ptrdiff_t count, ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo,
                              double* ab, ptrdiff_t ldab, ptrdiff_t sab, ptrdiff_t* P, ptrdiff_t sp,
                              ptrdiff_t nrhs, double* B, ptrdiff_t ldb, ptrdiff_t sb, int* status);

/* complex<double> (tmv_oracle_z.c): column-major, entries interleaved
 * (re, im), leading dimensions in complex elements. */
int oracle_lu_decompose_z(ptrdiff_t n, double* A, ptrdiff_t lda, ptrdiff_t* P);
int oracle_lu_ldiveq_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                       ptrdiff_t nrhs, double* B, ptrdiff_t ldb);
/* B (nrows x n, column-major) := B (P L U)^-1, row by row */
int oracle_lu_rdiveq_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                       ptrdiff_t nrows, double* B, ptrdiff_t ldb);
/* C (+)= alpha A B, strided complex views; alpha as (re, im) */
int oracle_multmm_z(int add, const double* alpha, ptrdiff_t m, ptrdiff_t n, ptrdiff_t k,
                    const double* A, ptrdiff_t sAi, ptrdiff_t sAj, const double* B, ptrdiff_t sBi,
                    ptrdiff_t sBj, double* C, ptrdiff_t sCi, ptrdiff_t sCj);
/* det and sign as (re, im) pairs */
void oracle_lu_det_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                     double* det, double* logdet, double* sign);

#ifdef __cplusplus
}
#endif

#endif
