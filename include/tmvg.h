/* tmvg.h -- C ABI of the GB300 (sm_103a) implementation of TMV's dense hot
 * path: the blocked matrix product and the partial-pivoting LU factor/solve.
 *
 * Plain pointers and sizes only.  Matrices are IEEE double (or float where a
 * name says f32), addressed like a tmv::MatrixView by (stepi, stepj) strides
 * in elements; "lda"/"ldb" name the stride between columns of a column-major
 * matrix.  Pivots are int64 (ptrdiff_t on LP64), 0-based, in TMV's (and
 * LAPACK's) interchange form: at step j row j was swapped with row P[j].
 *
 * Functions without "_host" take DEVICE pointers and are stream-ordered on the
 * handle's stream; they return once the work is enqueued unless stated.
 * Functions with "_host" take HOST pointers and are synchronous, like the TMV
 * calls they replace; they copy inputs to the device and results back.
 *
 * Each entry point names the TMV 0.76 routine it replaces (file:line in the
 * TMV source tree).  The drop-in shim (tmv_gb300/shim/tmv_gpu_shim.cpp)
 * defines those routines' explicit instantiations over this ABI.
 */
#ifndef TMVG_H
#define TMVG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef enum tmvg_status {
    TMVG_OK = 0,
    TMVG_SINGULAR = 1,       /* a zero U(j,j) was met while solving (TMV throws
                                SingularUpperTriMatrix, src/TMV_TriDiv_M.cpp:78-84) */
    TMVG_NOT_CONVERGED = 2,  /* iterative refinement missed its tolerance */
    TMVG_BAD_ARG = 3,
    TMVG_OOM = 4,            /* TMV: std::bad_alloc */
    TMVG_TIMEOUT = 5,        /* a bounded device-side wait gave up */
    TMVG_CUDA_ERROR = 6,
    TMVG_NO_DEVICE = 7,
    TMVG_UNSUPPORTED = 8
} tmvg_status;

typedef struct tmvg_context* tmvg_handle;

/* ---- context -------------------------------------------------------- */
int tmvg_version(void);
const char* tmvg_status_string(tmvg_status s);
/* Create a context on `device` (its current CUDA context, default stream). */
tmvg_status tmvg_create(tmvg_handle* h, int device);
tmvg_status tmvg_destroy(tmvg_handle h);

/* Kernel-class timing, a measurement hook with no counterpart in TMV.  While
 * enabled, the library records CUDA events on the handle's stream around
 * the launches of each class below and adds up, per class, the spans, their
 * elapsed time and the algorithmic work they do:
 *   TRAILING_UPDATE  A22 -= L21 U12 of each LU panel step (with the operand
 *                    split of the tensor-core path); bytes = sizeof(T) x
 *                    (2 m n + m k + k n), flops = 2 m n k
 *   PANEL            one panel factorisation; bytes = 2 sizeof(T) m nb,
 *                    flops = the panel's multiply-adds x 2
 *   TRI_SOLVE        one triangular solve of the mixed solve; bytes = the
 *                    triangle read once plus right-hand side in and out
 *   RESIDUAL         one FP64 residual b - A x; bytes = 8 n^2 + vectors
 * Enabling (or disabling) clears the sums; reading synchronises the stream.
 * Do not enable it while the stream is being captured into a CUDA graph. */
#define TMVG_KCLASS_TRAILING_UPDATE 0
#define TMVG_KCLASS_PANEL 1
#define TMVG_KCLASS_TRI_SOLVE 2
#define TMVG_KCLASS_RESIDUAL 3

typedef struct tmvg_kernel_timing {
    int64_t spans;   /* timed spans (one per panel step, solve, residual) */
    double total_ms; /* summed event time */
    double bytes;    /* summed algorithmic bytes */
    double flops;    /* summed algorithmic flops */
} tmvg_kernel_timing;

tmvg_status tmvg_timing_enable(tmvg_handle h, int on);
tmvg_status tmvg_timing_read(tmvg_handle h, int kclass, tmvg_kernel_timing* out);
/* Use this cudaStream_t for all later calls (NULL = legacy default stream). */
tmvg_status tmvg_set_stream(tmvg_handle h, void* cuda_stream);
tmvg_status tmvg_synchronize(tmvg_handle h);
/* Text of the last error on this handle ("" if none). */
const char* tmvg_last_error(tmvg_handle h);
/* Number of kernels this handle has launched since creation. */
int64_t tmvg_launch_count(tmvg_handle h);
/* FP64 FMA rate of the handle's device, a measurement hook with no
 * counterpart in TMV: a throughput kernel of independent DFMA chains on every
 * SM, timed with CUDA events on the handle's stream (best of three launches
 * after one warm-up), returned as TFLOP/s (2 flops per FMA).  The FP64-bound
 * roofline fractions of the benchmark use it, measured in the same process
 * and under the same clocks as the work.  Synchronises the stream. */
tmvg_status tmvg_probe_fp64_rate(tmvg_handle h, double* tflops);
/* Failure-path test hook, no counterpart in TMV.  poll_limit sets how many
 * polls the block-flag waits of the sync-free triangular solve (the solve of
 * up to 8 right-hand sides behind tmvg_tri_ldiveq_f64, tmvg_lu_ldiveq_f64 and
 * the FP64 solves) and of the mixed solve's streamed FP32 triangular solve
 * (n a multiple of 128) make before they give up (0 restores the default,
 * 2^24 polls with back-off).  skip_blocks > 0 makes the next such solve hand
 * its blocks out from ticket skip_blocks on, so the first blocks are never
 * solved and their results never published: the first block that waits on
 * one gives up after poll_limit polls, the others stop in turn, and the call
 * returns TMVG_TIMEOUT with the handle still usable (the hook resets itself
 * after that one launch).  Nothing traps or hangs. */
tmvg_status tmvg_test_set_wait(tmvg_handle h, uint32_t poll_limit, int32_t skip_blocks);

/* ---- MultMM ----------------------------------------------------------
 * C (+)= alpha * A * B;  A m x k, B k x n, C m x n.  add = 0: C = alpha*A*B,
 * add = 1: C += alpha*A*B.  A and B may each be column-major (stepi == 1) or
 * row-major (stepj == 1): the CCC, CRC, RCC (and RRC) layouts; a row-major C
 * is computed as C^T = B^T A^T.  Operands must not overlap C.
 * Replaces: template void tmv::MultMM<add,double,double,double>
 *           (src/TMV_MultMM.cpp:405-477; declared
 *            include/tmv/TMV_MatrixArithFunc.h:55-58). */
tmvg_status tmvg_multmm_f64(tmvg_handle h, int add, double alpha,
                            int64_t m, int64_t n, int64_t k,
                            const double* A, int64_t sAi, int64_t sAj,
                            const double* B, int64_t sBi, int64_t sBj,
                            double* C, int64_t sCi, int64_t sCj);
tmvg_status tmvg_multmm_f64_host(tmvg_handle h, int add, double alpha,
                                 int64_t m, int64_t n, int64_t k,
                                 const double* A, int64_t sAi, int64_t sAj,
                                 const double* B, int64_t sBi, int64_t sBj,
                                 double* C, int64_t sCi, int64_t sCj);

/* ---- FP32-accurate product on the tensor cores -----------------------
 * C -= A * B for FP32 column-major device data, A m x k, B k x n, with k a
 * multiple of 32 up to 128: the trailing-update shape of the mixed-precision
 * LU.  Runs on tcgen05 tensor cores with TF32 operands split as hi + lo
 * (three products per step, FP32 accumulation), so the result has FP32
 * accuracy.  Synchronous.  No TMV counterpart (TMV's float MultMM is
 * src/TMV_MultMM.cpp:405 on the CPU). */
tmvg_status tmvg_gemm_f32_tf32x3(tmvg_handle h, int64_t m, int64_t n, int64_t k,
                                 const float* A, int64_t lda, const float* B,
                                 int64_t ldb, float* C, int64_t ldc);

/* ---- LU_Decompose ----------------------------------------------------
 * In-place P A = L U of an n x n column-major matrix (leading dim lda):
 * L unit lower below the diagonal, U on and above it, P[0..n) interchanges.
 * Pivot rule as TMV: first index of the strict maximum |a|; a column whose
 * largest |a| is below DBL_MIN is zeroed with P[j] = j.  Never fails on
 * singular input.
 * Replaces: template void tmv::LU_Decompose(MatrixView<double>, ptrdiff_t*)
 *           (src/TMV_LUDecompose.cpp:514-559). */
tmvg_status tmvg_lu_decompose_f64(tmvg_handle h, int64_t n, double* A,
                                  int64_t lda, int64_t* P);
/* Host variant; A may be column- or row-major (stepi/stepj), as TMV allows. */
tmvg_status tmvg_lu_decompose_f64_host(tmvg_handle h, int64_t n, double* A,
                                       int64_t sAi, int64_t sAj, int64_t* P);

/* ---- LU_Decompose without device allocation --------------------------
 * No counterpart in TMV: an extra entry point for callers that cannot
 * allocate device memory (their device memory belongs to another allocator,
 * such as a framework's caching allocator or a fixed arena, or an allocation
 * is not acceptable on their code path).  For a column-major n x n device
 * matrix A and device pivots P it applies the pivot rule of
 * tmvg_lu_decompose_f64 and gives the same factors to rounding (it runs the
 * simplest schedule: the grid-barrier panel kernel, no look-ahead), but it
 * calls no cudaMalloc/cudaFree and needs no tmvg_handle: all scratch lives in
 * one static device array of 353,540 bytes (345 KiB) that every GPU loading
 * this library holds until the process exits; each call looks up the array's
 * device address in the current context.  Runs on the current device and
 * the given cudaStream_t (NULL: legacy default stream) and synchronises that
 * stream before it returns (so it cannot be called while the stream is being
 * captured into a CUDA graph).  Limit: n <= 16384, and a panel CTA's rows must
 * fit in 200 KiB of shared memory (every n <= 16384 does on a GPU with at
 * least 40 SMs); other sizes return TMVG_UNSUPPORTED before any device work.
 * Calls share the array, so calls that overlap on the GPU (other threads or
 * streams) race: serialise them. */
tmvg_status tmvg_lu_decompose_f64_noalloc(int64_t n, double* A, int64_t lda,
                                          int64_t* P, void* cuda_stream);

/* ---- LU_LDivEq / LU_RDivEq -------------------------------------------
 * LDivEq: B := (P L U)^-1 B, B n x nrhs column-major (ldb).
 * RDivEq: B := B (P L U)^-1, B nrows x n column-major (ldb).
 * Return TMVG_SINGULAR when a zero U(j,j) divides a nonzero entry.
 * Replace: template void tmv::LU_LDivEq / LU_RDivEq<double,double>
 *          (src/TMV_LUDiv.cpp:186-226, 370-411; declared src/TMV_LUDiv.h:30-35). */
tmvg_status tmvg_lu_ldiveq_f64(tmvg_handle h, int64_t n, const double* LU,
                               int64_t lda, const int64_t* P, int64_t nrhs,
                               double* B, int64_t ldb);
tmvg_status tmvg_lu_rdiveq_f64(tmvg_handle h, int64_t n, const double* LU,
                               int64_t lda, const int64_t* P, int64_t nrows,
                               double* B, int64_t ldb);
tmvg_status tmvg_lu_ldiveq_f64_host(tmvg_handle h, int64_t n, const double* LU,
                                    int64_t lda, const int64_t* P, int64_t nrhs,
                                    double* B, int64_t sBi, int64_t sBj);
tmvg_status tmvg_lu_rdiveq_f64_host(tmvg_handle h, int64_t n, const double* LU,
                                    int64_t lda, const int64_t* P, int64_t nrows,
                                    double* B, int64_t sBi, int64_t sBj);

/* ---- m.divideUsing(tmv::LU); X = B/m --------------------------------
 * Factor a copy of A (column-major n x n) and solve X = A^-1 B (n x nrhs).
 * LU and P receive the factors (kept by the caller for later solves, the
 * saveDiv() behaviour).  Replaces the LUDiv<double> construction + doLDiv
 * (src/TMV_LUD.cpp:74-120). */
tmvg_status tmvg_divide_f64(tmvg_handle h, int64_t n, const double* A,
                            int64_t lda, int64_t nrhs, const double* B,
                            int64_t ldb, double* X, int64_t ldx, double* LU,
                            int64_t* P);
tmvg_status tmvg_divide_f64_host(tmvg_handle h, int64_t n, const double* A,
                                 int64_t nrhs, const double* B, double* X,
                                 double* LU, int64_t* P);

/* det / logDet of stored factors (LUDiv::det, logDet: src/TMV_LUD.cpp:132-156). */
tmvg_status tmvg_lu_det_f64(tmvg_handle h, int64_t n, const double* LU,
                            int64_t lda, const int64_t* P, double* det,
                            double* logdet, double* sign);

/* m.inverse(): A^-1 from stored factors, U^-1 L^-1 with its columns
 * reverse-permuted by P.  Replaces LU_Inverse<double,double>
 * (src/TMV_LUInverse.cpp:236-299), reached through LUDiv::doMakeInverse
 * (src/TMV_LUD.cpp:158-170).  Minv: n x n column-major (ldm), or a host view
 * with strides (msi, msj) for the _host form.  TMVG_SINGULAR for a zero
 * U(j,j), where TMV throws SingularUpperTriMatrix (src/TMV_TriInverse.cpp:58-68). */
tmvg_status tmvg_lu_inverse_f64(tmvg_handle h, int64_t n, const double* LU,
                                int64_t lda, const int64_t* P, double* Minv,
                                int64_t ldm);
tmvg_status tmvg_lu_inverse_f64_host(tmvg_handle h, int64_t n,
                                     const double* LU, int64_t lda,
                                     const int64_t* P, double* Minv,
                                     int64_t msi, int64_t msj);

/* m.makeInverseATA(ata): (A^T A)^-1 from stored factors (the permutation
 * cancels).  Replaces LUDiv::doMakeInverseATA (src/TMV_LUD.cpp:172-200). */
tmvg_status tmvg_lu_inverse_ata_f64(tmvg_handle h, int64_t n, const double* LU,
                                    int64_t lda, double* ATA, int64_t ldata);

/* m.isSingular(): *singular = 1 when min |U(j,j)| <= epsilon * max |U(j,j)|.
 * Replaces LUDiv::isSingular (src/TMV_LUD.cpp:204-209). */
tmvg_status tmvg_lu_is_singular_f64(tmvg_handle h, int64_t n, const double* LU,
                                    int64_t lda, int* singular);

/* m /= T for a standalone triangle: B := T^-1 B, T the upper (upper = 1) or
 * lower triangle at (T, tsi, tsj), unit diagonal not read when unitdiag; B
 * n x nrhs with strides.  Replaces TriLDivEq<double,double> for
 * UpperTriMatrix / LowerTriMatrix (src/TMV_TriDiv_M.cpp:583-710), reached
 * through m /= U, x = b/U.  TMVG_SINGULAR as TMV throws SingularUpper/
 * LowerTriMatrix (one column or a column-major B: a zero T(j,j) that divides
 * a nonzero entry; otherwise any zero T(j,j)). */
tmvg_status tmvg_tri_ldiveq_f64(tmvg_handle h, int upper, int unitdiag, int64_t n,
                                const double* T, int64_t tsi, int64_t tsj,
                                int64_t nrhs, double* B, int64_t bsi, int64_t bsj);

/* m %= T: B := B T^-1 (B nrows x n), through T^T.LDivEq(m^T) as TMV does
 * (include/tmv/TMV_TriMatrix.h:945-946). */
tmvg_status tmvg_tri_rdiveq_f64(tmvg_handle h, int upper, int unitdiag, int64_t n,
                                const double* T, int64_t tsi, int64_t tsj,
                                int64_t nrows, double* B, int64_t bsi, int64_t bsj);

/* y (+)= alpha A x: A m x n with strides, x (n) and y (m) with increments; x
 * may share storage with y.  alpha = 0 or n = 0 leaves A unread.  Replaces
 * MultMV<add,double,double,double> (src/TMV_MultMV.cpp:1134-1175), reached
 * through y = A*x, y += alpha*A*x. */
tmvg_status tmvg_multmv_f64(tmvg_handle h, int add, double alpha, int64_t m,
                            int64_t n, const double* A, int64_t sAi, int64_t sAj,
                            const double* x, int64_t incx, double* y,
                            int64_t incy);

/* ---- complex<double> LU ------------------------------------------------
 * Device pointers; A, LU, B column-major with entries interleaved (real,
 * imaginary), leading dimensions in complex elements.
 * tmvg_lu_decompose_z64: A := P L U in place, P[0..n) interchanges.  Pivot
 * rule as TMV's complex instantiation: first index of the strict maximum of
 * TMV's modulus (TMV_ABS, include/tmv/TMV_Base.h:312-325); a column whose
 * largest modulus is below DBL_MIN is zeroed with P[j] = j; the column is
 * scaled by TMV_InverseOf of the pivot.  Never fails on singular input.
 * Replaces: template void tmv::LU_Decompose(MatrixView<std::complex<double> >,
 *           ptrdiff_t*) (src/TMV_LUDecompose.cpp:514-559).
 * tmvg_lu_ldiveq_z64: B := (P L U)^-1 B, each column with TMV's vector
 * solves (zero entries skipped; a division by U(j,j) as TMV_Divide);
 * TMVG_SINGULAR when a zero U(j,j) meets a nonzero entry.  Synchronises.
 * Replaces: template void tmv::LU_LDivEq(const GenMatrix<std::complex<double> >&,
 *           const ptrdiff_t*, MatrixView<std::complex<double> >)
 *           (src/TMV_LUDiv.cpp:186). */
tmvg_status tmvg_lu_decompose_z64(tmvg_handle h, int64_t n, double* A, int64_t lda,
                                  int64_t* P);
tmvg_status tmvg_lu_ldiveq_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                               const int64_t* P, int64_t nrhs, double* B, int64_t ldb);
/* B (nrows x n, column-major, leading dimension ldb) := B (P L U)^-1 with
 * TMV's row-oriented solves of the transposed factors (leading / trailing
 * zeros trimmed, a zero U(i,i) then TMVG_SINGULAR).  Synchronises.
 * Replaces: template void tmv::LU_RDivEq(const GenMatrix<std::complex<double> >&,
 *           const ptrdiff_t*, MatrixView<std::complex<double> >)
 *           (src/TMV_LUDiv.cpp:370). */
tmvg_status tmvg_lu_rdiveq_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                               const int64_t* P, int64_t nrows, double* B, int64_t ldb);
/* Minv (n x n, column-major) := (P L U)^-1, TMV's m.inverse() up to
 * rounding; TMVG_SINGULAR for a zero U(j,j).  Synchronises.
 * Replaces: template void tmv::LU_Inverse(const GenMatrix<std::complex<double> >&,
 *           const ptrdiff_t*, MatrixView<std::complex<double> >)
 *           (src/TMV_LUInverse.cpp:236). */
tmvg_status tmvg_lu_inverse_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                const int64_t* P, double* Minv, int64_t ldm);
/* Host-view variants of the four complex<double> entries above, as the
 * link-time drop-in calls them: A, B and Minv are host views with TMV's
 * (stepi, stepj) in complex elements (column- or row-major), LU is a
 * column-major host matrix with leading dimension lda, P a host vector.
 * Each copies its operands to the device, runs the entry above and copies
 * the results back; synchronous, as TMV's calls are. */
tmvg_status tmvg_lu_decompose_z64_host(tmvg_handle h, int64_t n, double* A, int64_t sAi,
                                       int64_t sAj, int64_t* P);
tmvg_status tmvg_lu_ldiveq_z64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                    const int64_t* P, int64_t nrhs, double* B, int64_t sBi,
                                    int64_t sBj);
tmvg_status tmvg_lu_rdiveq_z64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                    const int64_t* P, int64_t nrows, double* B, int64_t sBi,
                                    int64_t sBj);
tmvg_status tmvg_lu_inverse_z64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                     const int64_t* P, double* Minv, int64_t msi, int64_t msj);

/* ---- float: MultMM, LU_Decompose, LU_LDivEq / LU_RDivEq, LU_Inverse ----
 * Host views (TMV's (stepi, stepj); LU column-major with lda), synchronous,
 * with the conventions of the double entries: the product (FP32 FMA tiles)
 * C (+)= alpha A B; the factorisation P A = L U with TMV's pivot rule on FP32
 * values (its trailing updates are 3xTF32 tensor-core products, FP32-accurate
 * but not FP32-rounded step by step); B := B / (P L U) and B (P L U)^-1 with
 * TMVG_SINGULAR where TMV throws SingularUpperTriMatrix<float>; Minv :=
 * (P L U)^-1.
 * Replace: template void tmv::MultMM<add,float,float,float>
 *          (src/TMV_MultMM.cpp:405-477), tmv::LU_Decompose<float>
 *          (src/TMV_LUDecompose.cpp:514-559), tmv::LU_LDivEq / LU_RDivEq
 *          <float,float> (src/TMV_LUDiv.cpp:186-226, 370-411) and
 *          tmv::LU_Inverse<float,float> (src/TMV_LUInverse.cpp:236-299). */
tmvg_status tmvg_multmm_f32_host(tmvg_handle h, int add, float alpha, int64_t m, int64_t n,
                                 int64_t k, const float* A, int64_t sAi, int64_t sAj,
                                 const float* B, int64_t sBi, int64_t sBj, float* C,
                                 int64_t sCi, int64_t sCj);
tmvg_status tmvg_lu_decompose_f32_host(tmvg_handle h, int64_t n, float* A, int64_t sAi,
                                       int64_t sAj, int64_t* P);
tmvg_status tmvg_lu_ldiveq_f32_host(tmvg_handle h, int64_t n, const float* LU, int64_t lda,
                                    const int64_t* P, int64_t nrhs, float* B, int64_t sBi,
                                    int64_t sBj);
tmvg_status tmvg_lu_rdiveq_f32_host(tmvg_handle h, int64_t n, const float* LU, int64_t lda,
                                    const int64_t* P, int64_t nrows, float* B, int64_t sBi,
                                    int64_t sBj);
tmvg_status tmvg_lu_inverse_f32_host(tmvg_handle h, int64_t n, const float* LU, int64_t lda,
                                     const int64_t* P, float* Minv, int64_t msi, int64_t msj);
/* det (re, im), logdet = sum log|U_jj| and sign (re, im) from the factors,
 * host outputs.  Replaces: LUDiv<std::complex<double> >::det / logDet
 * (src/TMV_LUD.cpp:132-156). */
tmvg_status tmvg_lu_det_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                            const int64_t* P, double* det, double* logdet, double* sign);

/* ---- mixed-precision solve with FP64 iterative refinement ---------------
 * X = A^-1 B for a column-major FP64 A: the factorisation runs in FP32
 * (pivots chosen by comparing in FP64), then each column is refined with
 * FP64 residuals r = b - A x and FP64 updates until the normwise backward
 * error ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol, or max_iter
 * refinement steps (TMVG_NOT_CONVERGED; X then holds the last iterate).
 * TMV has no mixed-precision path; this is an alternative engine for the
 * same X = B/m of a tmv::Matrix<double> (LUDiv::doLDiv, src/TMV_LUD.cpp:112-120). */
typedef struct tmvg_ir_info {
    int32_t iterations;     /* refinement steps applied (worst column) */
    int32_t converged;      /* 1 when every column met tol */
    double backward_error;  /* worst normwise backward error at exit */
    double anorm_inf;       /* ||A||_inf */
} tmvg_ir_info;

tmvg_status tmvg_lu_solve_mixed_f64(tmvg_handle h, int64_t n, const double* A,
                                    int64_t lda, int64_t nrhs, const double* B,
                                    int64_t ldb, double* X, int64_t ldx,
                                    int max_iter, double tol, tmvg_ir_info* info);
/* Host variant: dense column-major host A (n x n), B and X (n x nrhs). */
tmvg_status tmvg_lu_solve_mixed_f64_host(tmvg_handle h, int64_t n, const double* A,
                                         int64_t nrhs, const double* B, double* X,
                                         int max_iter, double tol, tmvg_ir_info* info);

/* ---- solve adjoint (forward / backward pair) ------------------------------
 * Forward: X = A^-1 B (A column-major n x n, B n x nrhs), keeping the LU
 * factors and interchanges for the backward (same work as tmvg_divide_f64).
 * Backward, given G = dL/dX (n x nrhs) and the saved LU, P and X:
 *   gB = dL/dB = A^-T G   -- the transpose solve with the saved factors,
 *                            U^T then L^T then the reversed interchanges,
 *                            i.e. TMV's (G^T % A)^T (LU_RDivEq,
 *                            src/TMV_LUDiv.cpp:370-411);
 *   gA = dL/dA = -gB X^T  -- an FP64 outer-product GEMM (K = nrhs).
 * gB and gA are outputs (column-major, ldgb / ldga); either may be NULL to
 * skip it (gA needs gB, which is then computed into scratch).  TMV has no
 * adjoint; this pair has the contract of an autograd backward. */
tmvg_status tmvg_lu_solve_fwd_f64(tmvg_handle h, int64_t n, const double* A, int64_t lda,
                                  int64_t nrhs, const double* B, int64_t ldb, double* X,
                                  int64_t ldx, double* LU, int64_t* P);
tmvg_status tmvg_lu_solve_bwd_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                  const int64_t* P, int64_t nrhs, const double* X,
                                  int64_t ldx, const double* G, int64_t ldg, double* gB,
                                  int64_t ldgb, double* gA, int64_t ldga);

/* ---- batched uneven LU solves ---------------------------------------------
 * Thousands of independent systems X_s = A_s^-1 B_s (1 <= n_s <= 256,
 * 0 <= nrhs_s <= 16) factored and solved in FP64 by one persistent kernel
 * launch, replayed from a CUDA graph captured when the plan is created.
 * Layout: A_s column-major n_s x n_s at A + a_off[s], B_s column-major
 * n_s x nrhs_s at B + b_off[s]; a_off/b_off NULL means packed in order.
 * A_s is overwritten by its LU factors, B_s by X_s, the interchanges go to
 * P + (n_0 + ... + n_{s-1}); status[s] = 1 where a zero U(j,j) met a
 * nonzero (TMV's SingularUpperTriMatrix), else 0.  With tune_tiles the
 * plan times the panel widths 8 and 16 on a sample of every size class
 * (n <= 32, 64, 128, 256) and keeps the fastest.
 * Replaces a loop of LUDiv<double> B_s / A_s (src/TMV_LUD.cpp:74-120). */
typedef struct tmvg_batch_plan_s* tmvg_batch_plan;

tmvg_status tmvg_batch_plan_create(tmvg_handle h, int64_t count, const int64_t* n,
                                   const int64_t* nrhs, const int64_t* a_off,
                                   const int64_t* b_off, int tune_tiles,
                                   tmvg_batch_plan* plan);
/* Buffer extents (elements), total algorithmic FLOPs
 * (sum 2n^3/3 + 2n^2 nrhs) and the panel width per size class (4 ints). */
tmvg_status tmvg_batch_plan_info(tmvg_batch_plan plan, int64_t* a_elems,
                                 int64_t* b_elems, int64_t* p_elems, double* flops,
                                 int* panel_widths);
tmvg_status tmvg_batch_plan_set_tiles(tmvg_batch_plan plan, const int* panel_widths);
/* Device pointers; synchronous. */
tmvg_status tmvg_batched_lu_solve_f64(tmvg_batch_plan plan, double* A, double* B,
                                      int64_t* P, int32_t* status);
/* The same batch with FP32 factors and FP64 refinement (the systems the
 * batched workload calls FP32-refined): per system, an FP32 copy of A is
 * factored with pivots chosen by comparing in FP64 (P receives them), then
 * x = 0 and, until every column's normwise backward error
 * ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol, r = b - A x in
 * FP64, d = A^-1 r with the FP32 factors, x += d in FP64, at most max_iter
 * corrections, all in the same persistent launch (a captured CUDA graph).  A
 * and the right-hand sides are read, not modified; B receives X.
 * status[s]: 0 converged, 1 a zero U(j,j) of the FP32 factors met a nonzero
 * (TMV's SingularUpperTriMatrix), 2 not converged (B holds the last iterate).
 * iters[s] (corrections applied) and berr[s] (worst column's backward error
 * at exit) are optional.  TMV has no mixed-precision path; this is another
 * engine for the same X_i = B_i / A_i (LUDiv::doLDiv, src/TMV_LUD.cpp:112-120). */
tmvg_status tmvg_batched_lu_solve_mixed_f64(tmvg_batch_plan plan, const double* A,
                                            double* B, int64_t* P, int32_t* status,
                                            int max_iter, double tol,
                                            int32_t* iters, double* berr);
tmvg_status tmvg_batch_plan_destroy(tmvg_batch_plan plan);

/* ---------------------------------------------------------------------
 * Batched band LU: count n x n band systems of one shape (lo subdiagonals,
 * hi superdiagonals), one GPU thread per system.  Replaces, per system,
 * tmv::LU_Decompose(BandMatrixView<double>, ptrdiff_t* P, ptrdiff_t Anhi)
 * (include/tmv/TMV_BandLUD.h:61, src/TMV_BandLUDecompose.cpp:383-425) and
 * tmv::LU_LDivEq(const GenBandMatrix<double>&, const ptrdiff_t*,
 * MatrixView<double>) (src/TMV_BandLUDiv.h:52, src/TMV_BandLUDiv.cpp:811),
 * the two steps of BandLUDiv (x = b / A for a tmv::BandMatrix); results are
 * TMV's bit for bit.
 *
 * Storage is TMV's column-major band layout: system s's element (i,j) at
 * AB[s*stride_ab + i + j*ldab] for j-hu <= i <= j+lo, hu = min(lo+hi, n-1)
 * (the superdiagonals the interchanges fill), ldab >= lo + hu, stride_ab >=
 * (n-1)(ldab+1)+1.  The factors replace A in those slots (the fill diagonals
 * hi+1..hu are written, never read); P[s*stride_p + j] receives the row
 * interchanged with row j (TMV's ptrdiff_t P).  B is n x nrhs column-major
 * per system at B[s*stride_b + i + q*ldb], ldb >= n.
 *
 * algo: TMVG_BAND_GENERAL, TMV's general band algorithm (the column-major
 * BandMatrixView above), or TMVG_BAND_TRIDIAG (lo == hi == 1), the
 * tridiagonal algorithm BandLUDiv runs on its diagonal-major copy of a
 * tridiagonal matrix (src/TMV_BandLUDecompose.cpp:144-200,
 * src/TMV_BandTriDiv_V.cpp:63-135), here on the same column-major storage.
 *
 * status[s] (solves): 0; 1 a zero U(j,j) met where TMV throws
 * SingularBandLU (B then holds a partial result); 2 an interchange P[j]
 * outside rows j..min(j+lo, n-1), not applied (factors not made by this
 * factorisation).  Device pointers, stream-ordered on the handle's stream;
 * no synchronisation.
 * --------------------------------------------------------------------- */
#define TMVG_BAND_GENERAL 0
#define TMVG_BAND_TRIDIAG 1
tmvg_status tmvg_band_lu_decompose_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo,
                                               int64_t hi, int algo, double* AB, int64_t ldab,
                                               int64_t stride_ab, int64_t* P, int64_t stride_p);
tmvg_status tmvg_band_lu_ldiveq_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo,
                                            int64_t hi, int algo, const double* AB, int64_t ldab,
                                            int64_t stride_ab, const int64_t* P, int64_t stride_p,
                                            int64_t nrhs, double* B, int64_t ldb, int64_t stride_b,
                                            int32_t* status);
/* x P L U = m for every system from its band factors: replaces
 * tmv::LU_RDivEq(const GenBandMatrix<double>&, const ptrdiff_t*,
 * MatrixView<double>) (src/TMV_BandLUDiv.h:55, src/TMV_BandLUDiv.cpp:834-851),
 * the step of BandLUDiv behind m %= A (and behind b / A when BandLUDiv
 * factors the transpose), bit for bit.  m is nrhs x n per system, row q at
 * B[s*stride_b + q*ldb] (unit step, ldb >= n: a row-major m to TMV); the
 * memory layout is ldiveq's B.  Same status values. */
tmvg_status tmvg_band_lu_rdiveq_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo,
                                            int64_t hi, int algo, const double* AB, int64_t ldab,
                                            int64_t stride_ab, const int64_t* P, int64_t stride_p,
                                            int64_t nrhs, double* B, int64_t ldb, int64_t stride_b,
                                            int32_t* status);
/* X = A^-1 B for every system as tmv::BandLUDiv computes it (B /= A for a
 * column-major tmv::BandMatrix, src/TMV_BandLUD.cpp:60-146, 217-222), bit for
 * bit: A's band (lo, hi) at AB[s*stride_ab + i + j*ldab], j-hi <= i <= j+lo,
 * ldab >= lo + hi (not modified) is copied into LU (min(lo,hi)
 * subdiagonals, hu = min(lo+hi, n-1) superdiagonals, ldlu >= min(lo,hi) +
 * hu; must not overlap AB), transposed when hi < lo, and factored with the
 * tridiagonal algorithm when lo == hi == 1; B (n x nrhs column-major, as for
 * ldiveq) is then solved with LU_LDivEq, or with LU_RDivEq on the
 * transpose's factors (its rows are B's columns).  LU and P keep the
 * factors (of A^T when hi < lo).  Same status values. */
tmvg_status tmvg_band_divide_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo, int64_t hi,
                                         const double* AB, int64_t ldab, int64_t stride_ab, double* LU,
                                         int64_t ldlu, int64_t stride_lu, int64_t* P, int64_t stride_p,
                                         int64_t nrhs, double* B, int64_t ldb, int64_t stride_b,
                                         int32_t* status);
/* Both in one launch (the factors and P are written as by the decompose). */
tmvg_status tmvg_band_lu_solve_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo,
                                           int64_t hi, int algo, double* AB, int64_t ldab,
                                           int64_t stride_ab, int64_t* P, int64_t stride_p,
                                           int64_t nrhs, double* B, int64_t ldb, int64_t stride_b,
                                           int32_t* status);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* TMVG_H */
