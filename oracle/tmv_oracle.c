/* tmv_oracle.c -- CPU restatement of TMV 0.76's dense hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see tmv_oracle.h).  It is the checker the GPU
 * kernels are compared against and the "port" CPU baseline; it is pinned
 * against TMV itself (oracle/_ref, built from the reference sources) by
 * tests/test_oracle_vs_ref.py and against golden vectors by
 * tests/test_oracle_golden.py.
 *
 * Restated (file:line are in the TMV 0.76 tree):
 *   MultMM normalisation ......... src/TMV_MultMM.cpp:405-454
 *   NonBlasMultMM dispatch ....... src/TMV_MultMM.cpp:47-100
 *   OpenMPMultMM ................. src/TMV_MultMM_OpenMP.cpp:31-66
 *   Block product (16x16 tiles, KB-deep panels, per-panel partial sums added
 *     into a zeroed 16x16 scratch, then C (+)= x*scratch)
 *                                  src/TMV_MultMM_Block.cpp:35-94,173-332
 *                                  src/TMV_MultMM_Kernel.h:41 (generic, KB=16)
 *   Simple CCC/CRC/RCC products .. src/TMV_MultMM_CCC.cpp:33-122 (+CRC, RCC)
 *   maxAbsElement ................ src/TMV_Vector.cpp:474-503
 *   TMV_Underflow ................ include/tmv/TMV_Base.h:692-696
 *   permuteRows .................. src/TMV_Matrix.cpp:866-900
 *   RecursiveLUDecompose ......... src/TMV_LUDecompose.cpp:217-407
 *   LU_Decompose ................. src/TMV_LUDecompose.cpp:514-540
 *   NonBlasTriLDivEq (matrix) .... src/TMV_TriDiv_M.cpp:58-266
 *   TriLDivEq (vector) ........... src/TMV_TriDiv_V.cpp:148-462
 *   LU_LDivEq / LU_RDivEq ........ src/TMV_LUDiv.cpp:46-55,186-226,232-242,370-411
 *   LUDiv::det / logDet .......... src/TMV_LUD.cpp:132-190
 *   LU_Inverse ................... src/TMV_LUInverse.cpp:38-52,236-299
 *   RecursiveInverse (upper tri) . src/TMV_TriInverse.cpp:49-88
 *   LUDiv::makeInverseATA ........ src/TMV_LUD.cpp:172-200
 *   MultMV ....................... src/TMV_MultMV.cpp:80-215,298-380,1134-1175
 *   LUDiv::isSingular ............ src/TMV_LUD.cpp:204-209,
 *                                  src/TMV_Vector.cpp:539-600
 *
 * Built with -ffp-contract=off so that a*b+c is never fused, as in the
 * reference's x86 build.
 */
#include "tmv_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef ptrdiff_t idx;

/* A strided matrix view (tmv::MatrixView without conj). */
typedef struct {
    double* p;
    idx m, n;   /* colsize, rowsize */
    idx si, sj; /* stepi, stepj */
} view;

#define AT(v, i, j) ((v).p[(i) * (v).si + (j) * (v).sj])

static view mkview(double* p, idx m, idx n, idx si, idx sj)
{
    view v = {p, m, n, si, sj};
    return v;
}
static view sub(view v, idx i1, idx i2, idx j1, idx j2)
{
    return mkview(v.p + i1 * v.si + j1 * v.sj, i2 - i1, j2 - j1, v.si, v.sj);
}
static view transp(view v) { return mkview(v.p, v.n, v.m, v.sj, v.si); }
static int iscm(view v) { return v.si == 1; }
static int isrm(view v) { return v.sj == 1; }

void oracle_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int in_parallel(void)
{
#ifdef _OPENMP
    return omp_in_parallel();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* MultMM                                                              */
/* ------------------------------------------------------------------ */

/* C (+)= x * T, T a dense column-major m x n scratch. */
static void add_scaled(int add, double x, const double* T, idx ldt, view C)
{
    for (idx j = 0; j < C.n; ++j)
        for (idx i = 0; i < C.m; ++i) {
            double t = T[i + j * ldt];
            if (x != 1.0) t = x * t;
            if (add) AT(C, i, j) += t;
            else AT(C, i, j) = t;
        }
}

/* Small products (src/TMV_MultMM_CCC.cpp:87-122 and the CRC/RCC twins):
 * accumulate A*B into a zeroed temporary, each C(i,j) summed over k in
 * increasing order, then scale and store/add. */
static int simple_multmm(int add, double alpha, view A, view B, view C)
{
    const idx M = C.m, N = C.n, K = A.n;
    double* T = (double*)calloc((size_t)(M * N), sizeof(double));
    if (!T) return ORACLE_NOMEM;
    if (iscm(A)) {
        for (idx j = 0; j < N; ++j)
            for (idx k = 0; k < K; ++k) {
                const double b = AT(B, k, j);
                for (idx i = 0; i < M; ++i) T[i + j * M] += AT(A, i, k) * b;
            }
    } else {
        for (idx j = 0; j < N; ++j)
            for (idx i = 0; i < M; ++i) {
                double s = 0.0;
                for (idx k = 0; k < K; ++k) s += AT(A, i, k) * AT(B, k, j);
                T[i + j * M] = s;
            }
    }
    if (alpha != 1.0)
        for (idx t = 0; t < M * N; ++t) T[t] *= alpha;
    add_scaled(add, 1.0, T, M, C);
    free(T);
    return ORACLE_OK;
}

/* Block product (the generic BlockHelper, KB = 16,
 * src/TMV_MultMM_Block.cpp:96-116, 173-332).  A is packed once into 16-row
 * panels of KB x 16 row-major blocks ("Ax", stepi = KB), B one 16-column
 * panel at a time into column-major KB x 16 blocks ("Bx"); for every 16x16
 * tile of C and every KB-deep block the micro-kernel sums its KB products
 * from zero in 2x2 register blocks and adds the partial sums into a zeroed
 * 16x16 scratch (src/TMV_MultMM_Kernel.h:41-260, 1038-1200); the scratch is
 * then stored as C (+)= x*scratch (src/TMV_MultMM_Block.cpp:84-93). */
#define KB 16
static void micro_kernel(idx mb, idx nb, idx kb, const double* Ap, const double* Bp, double* Ct)
{
    /* Ap: mb rows, row i at Ap + i*KB (k contiguous); Bp: nb columns, column
     * j at Bp + j*KB.  Ct: 16 x 16 column-major. */
    idx i, j;
    for (j = 0; j + 1 < nb; j += 2) {
        const double* b0 = Bp + j * KB;
        const double* b1 = b0 + KB;
        for (i = 0; i + 1 < mb; i += 2) {
            const double* a0 = Ap + i * KB;
            const double* a1 = a0 + KB;
            double c00 = 0, c01 = 0, c10 = 0, c11 = 0;
            for (idx k = 0; k < kb; ++k) {
                c00 += a0[k] * b0[k];
                c10 += a1[k] * b0[k];
                c01 += a0[k] * b1[k];
                c11 += a1[k] * b1[k];
            }
            Ct[i + 16 * j] += c00;
            Ct[i + 1 + 16 * j] += c10;
            Ct[i + 16 * (j + 1)] += c01;
            Ct[i + 1 + 16 * (j + 1)] += c11;
        }
        if (i < mb) {
            const double* a0 = Ap + i * KB;
            double c00 = 0, c01 = 0;
            for (idx k = 0; k < kb; ++k) {
                c00 += a0[k] * b0[k];
                c01 += a0[k] * b1[k];
            }
            Ct[i + 16 * j] += c00;
            Ct[i + 16 * (j + 1)] += c01;
        }
    }
    if (j < nb) {
        const double* b0 = Bp + j * KB;
        for (i = 0; i < mb; ++i) {
            const double* a0 = Ap + i * KB;
            double c00 = 0;
            for (idx k = 0; k < kb; ++k) c00 += a0[k] * b0[k];
            Ct[i + 16 * j] += c00;
        }
    }
}

static void block_multmm(int add, double x, view A, view B, view C)
{
    const idx M = C.m, N = C.n, K = A.n;
    const idx nkb = (K + KB - 1) / KB;
    const idx nmb = (M + 15) / 16;
    /* full packed copy of A: for each 16-row panel, nkb blocks of 16 x KB */
    double* Ap = (double*)calloc((size_t)(nmb * nkb * 16 * KB), sizeof(double));
    double* Bp = (double*)calloc((size_t)(nkb * 16 * KB), sizeof(double));
    double Ct[16 * 16];
    if (!Ap || !Bp) {
        /* the reference falls back to the simple product on bad_alloc
         * (src/TMV_MultMM_Block.cpp:400-439) */
        free(Ap);
        free(Bp);
        simple_multmm(add, x, A, B, C);
        return;
    }
    for (idx ib = 0; ib < nmb; ++ib)
        for (idx kb = 0; kb < nkb; ++kb) {
            double* blk = Ap + (ib * nkb + kb) * 16 * KB;
            const idx i1 = ib * 16, k1 = kb * KB;
            const idx mb = M - i1 < 16 ? M - i1 : 16, kk = K - k1 < KB ? K - k1 : KB;
            for (idx i = 0; i < mb; ++i)
                for (idx k = 0; k < kk; ++k) blk[i * KB + k] = AT(A, i1 + i, k1 + k);
        }
    for (idx j1 = 0; j1 < N; j1 += 16) {
        const idx nb = N - j1 < 16 ? N - j1 : 16;
        for (idx kb = 0; kb < nkb; ++kb) {
            double* blk = Bp + kb * 16 * KB;
            const idx k1 = kb * KB, kk = K - k1 < KB ? K - k1 : KB;
            for (idx j = 0; j < nb; ++j)
                for (idx k = 0; k < kk; ++k) blk[j * KB + k] = AT(B, k1 + k, j1 + j);
        }
        for (idx ib = 0; ib < nmb; ++ib) {
            const idx i1 = ib * 16;
            const idx mb = M - i1 < 16 ? M - i1 : 16;
            memset(Ct, 0, sizeof(Ct));
            for (idx kb = 0; kb < nkb; ++kb) {
                const idx k1 = kb * KB, kk = K - k1 < KB ? K - k1 : KB;
                micro_kernel(mb, nb, kk, Ap + (ib * nkb + kb) * 16 * KB, Bp + kb * 16 * KB, Ct);
            }
            add_scaled(add, x, Ct, 16, sub(C, i1, i1 + mb, j1, j1 + nb));
        }
    }
    free(Ap);
    free(Bp);
}

/* src/TMV_MultMM_OpenMP.cpp:31-66: split C into 16-aligned row slices
 * (M > N) or column slices, one BlockMultMM per thread. */
static void openmp_multmm(int add, double x, view A, view B, view C)
{
#ifdef _OPENMP
    const idx M = C.m, N = C.n;
#pragma omp parallel
    {
        const idx nt = omp_get_num_threads();
        const idx me = omp_get_thread_num();
        if (nt == 1) {
            block_multmm(add, x, A, B, C);
        } else if (M > N) {
            idx Mx = M / nt;
            Mx = (((Mx - 1) >> 4) + 1) << 4;
            idx i1 = me * Mx, i2 = (me + 1) * Mx;
            if (i2 > M || me == nt - 1) i2 = M;
            if (i1 < M)
                block_multmm(add, x, sub(A, i1, i2, 0, A.n), B,
                             sub(C, i1, i2, 0, N));
        } else {
            idx Nx = N / nt;
            Nx = (((Nx - 1) >> 4) + 1) << 4;
            idx j1 = me * Nx, j2 = (me + 1) * Nx;
            if (j2 > N || me == nt - 1) j2 = N;
            if (j1 < N)
                block_multmm(add, x, A, sub(B, 0, B.m, j1, j2),
                             sub(C, 0, M, j1, j2));
        }
    }
#else
    block_multmm(add, x, A, B, C);
#endif
}

/* src/TMV_MultMM.cpp:47-100 */
static int nonblas_multmm(int add, double alpha, view A, view B, view C)
{
    const idx M = C.m, N = C.n, K = A.n;
    const idx Mb = M >> 6, Nb = N >> 6, Kb = K >> 6;
    const idx Mc = M < 16 ? 1 : (M >> 4);
    const idx Nc = N < 16 ? 1 : (N >> 4);
    const idx Kc = K < 16 ? 1 : (K >> 4);
    const int twobig = (Mb && Nb) || (Mb && Kb) || (Nb && Kb);
    if ((M < 16 && N < 16 && K < 16) || (M <= 3 || N <= 3 || K <= 3) ||
        ((M < 16 || N < 16 || K < 16) && (!twobig || (Mc * Nc * Kc < 4)))) {
        return simple_multmm(add, alpha, A, B, C);
    } else if (!in_parallel() && (Mb || Nb) && (Mc * Nc * Kc >= 64)) {
        openmp_multmm(add, alpha, A, B, C);
    } else {
        block_multmm(add, alpha, A, B, C);
    }
    return ORACLE_OK;
}

static double* dense_copy(view v)
{
    double* t = (double*)malloc(sizeof(double) * (size_t)(v.m * v.n > 0 ? v.m * v.n : 1));
    if (!t) return NULL;
    for (idx j = 0; j < v.n; ++j)
        for (idx i = 0; i < v.m; ++i) t[i + j * v.m] = AT(v, i, j);
    return t;
}

/* src/TMV_MultMM.cpp:405-454 (no conjugation for real T; operands are
 * assumed not to alias C, as for distinct tmv::Matrix objects). */
static int multmm_view(int add, double alpha, view A, view B, view C)
{
    if (C.m <= 0 || C.n <= 0) return ORACLE_OK;
    if (A.n == 0 || alpha == 0.0) {
        if (!add)
            for (idx j = 0; j < C.n; ++j)
                for (idx i = 0; i < C.m; ++i) AT(C, i, j) = 0.0;
        return ORACLE_OK;
    }
    if (iscm(C)) {
        int rc;
        double *ta = NULL, *tb = NULL;
        if (!(iscm(A) || isrm(A))) {
            ta = dense_copy(A);
            if (!ta) return ORACLE_NOMEM;
            A = mkview(ta, A.m, A.n, 1, A.m);
        }
        if (!(iscm(B) || isrm(B))) {
            tb = dense_copy(B);
            if (!tb) { free(ta); return ORACLE_NOMEM; }
            B = mkview(tb, B.m, B.n, 1, B.m);
        }
        rc = nonblas_multmm(add, alpha, A, B, C);
        free(ta);
        free(tb);
        return rc;
    } else if (isrm(C)) {
        return multmm_view(add, alpha, transp(B), transp(A), transp(C));
    } else {
        double* t = (double*)malloc(sizeof(double) * (size_t)(C.m * C.n));
        int rc;
        if (!t) return ORACLE_NOMEM;
        rc = multmm_view(0, 1.0, A, B, mkview(t, C.m, C.n, 1, C.m));
        if (rc == ORACLE_OK) add_scaled(add, alpha, t, C.m, C);
        free(t);
        return rc;
    }
}

int oracle_multmm(int add, double alpha, ptrdiff_t m, ptrdiff_t n, ptrdiff_t k,
                  const double* A, ptrdiff_t sAi, ptrdiff_t sAj,
                  const double* B, ptrdiff_t sBi, ptrdiff_t sBj,
                  double* C, ptrdiff_t sCi, ptrdiff_t sCj)
{
    if (m < 0 || n < 0 || k < 0) return ORACLE_BAD_ARG;
    return multmm_view(add, alpha, mkview((double*)A, m, k, sAi, sAj),
                       mkview((double*)B, k, n, sBi, sBj),
                       mkview(C, m, n, sCi, sCj));
}

/* ------------------------------------------------------------------ */
/* Pivot search, permutations                                          */
/* ------------------------------------------------------------------ */

/* src/TMV_Vector.cpp:474-503: first index of the strict maximum of |v|;
 * a NaN is only ever chosen when it is v[0]. */
static double max_abs_element(const double* p, idx len, idx step, idx* imax)
{
    double mx = fabs(p[0]);
    *imax = 0;
    for (idx i = 1; i < len; ++i) {
        const double a = fabs(p[i * step]);
        if (a > mx) {
            mx = a;
            *imax = i;
        }
    }
    return mx;
}

/* include/tmv/TMV_Base.h:692-696 with TMV_ABS2(x) = std::abs(x) for a real
 * x (include/tmv/TMV_Base.h:330-331): |x| < DBL_MIN. */
static int underflow(double x) { return fabs(x) < DBL_MIN; }

static void swap_rows(view A, idx i1, idx i2)
{
    if (i1 == i2) return;
    for (idx j = 0; j < A.n; ++j) {
        const double t = AT(A, i1, j);
        AT(A, i1, j) = AT(A, i2, j);
        AT(A, i2, j) = t;
    }
}

/* src/TMV_Matrix.cpp:866-900 (the 32-column strips change no value). */
static void permute_rows(view A, const idx* P, idx i1, idx i2)
{
    for (idx i = i1; i < i2; ++i) swap_rows(A, i, P[i]);
}

static void reverse_permute_rows(view A, const idx* P, idx i1, idx i2)
{
    for (idx i = i2; i > i1;) {
        --i;
        swap_rows(A, i, P[i]);
    }
}

/* ------------------------------------------------------------------ */
/* Triangular solves                                                   */
/* ------------------------------------------------------------------ */

typedef struct {
    view a;    /* n x n, only one triangle is read */
    int upper; /* 1 upper, 0 lower */
    int unit;  /* unit diagonal (not read) */
} tri;

static tri tri_sub(tri t, idx i1, idx i2)
{
    tri r = {sub(t.a, i1, i2, i1, i2), t.upper, t.unit};
    return r;
}

/* Vector solves, column-oriented (A column-major): src/TMV_TriDiv_V.cpp:148-236
 * (upper) and 322-398 (lower).  Entries of b equal to 0 are skipped. */
static int col_tri_ldiveq_vec(tri t, double* b)
{
    const view A = t.a;
    const idx N = A.m;
    if (t.upper) {
        for (idx j = N - 1; j > 0; --j) {
            if (b[j] != 0.0) {
                if (!t.unit) {
                    if (AT(A, j, j) == 0.0) return ORACLE_SINGULAR;
                    b[j] = b[j] / AT(A, j, j);
                }
                for (idx i = 0; i < j; ++i) b[i] -= b[j] * AT(A, i, j);
            }
        }
        if (!t.unit && b[0] != 0.0) {
            if (AT(A, 0, 0) == 0.0) return ORACLE_SINGULAR;
            b[0] = b[0] / AT(A, 0, 0);
        }
    } else {
        for (idx j = 0; j < N - 1; ++j) {
            if (b[j] != 0.0) {
                if (!t.unit) {
                    if (AT(A, j, j) == 0.0) return ORACLE_SINGULAR;
                    b[j] = b[j] / AT(A, j, j);
                }
                for (idx i = j + 1; i < N; ++i) b[i] -= b[j] * AT(A, i, j);
            }
        }
        if (!t.unit && b[N - 1] != 0.0) {
            if (AT(A, N - 1, N - 1) == 0.0) return ORACLE_SINGULAR;
            b[N - 1] = b[N - 1] / AT(A, N - 1, N - 1);
        }
    }
    return ORACLE_OK;
}

/* Row-oriented vector solves (A row-major): src/TMV_TriDiv_V.cpp:59-146, 237-320. */
static int row_tri_ldiveq_vec(tri t, double* b)
{
    const view A = t.a;
    const idx N = A.m;
    if (t.upper) {
        for (idx i = N - 1; i >= 0; --i) {
            for (idx j = i + 1; j < N; ++j) b[i] -= b[j] * AT(A, i, j);
            if (!t.unit) {
                if (AT(A, i, i) == 0.0) return ORACLE_SINGULAR;
                b[i] = b[i] / AT(A, i, i);
            }
        }
    } else {
        for (idx i = 0; i < N; ++i) {
            for (idx j = 0; j < i; ++j) b[i] -= b[j] * AT(A, i, j);
            if (!t.unit) {
                if (AT(A, i, i) == 0.0) return ORACLE_SINGULAR;
                b[i] = b[i] / AT(A, i, i);
            }
        }
    }
    return ORACLE_OK;
}

/* src/TMV_TriDiv_V.cpp:401-462: trim the leading (lower) or trailing
 * (upper) zeros of b, then the row or column variant by A's storage. */
static int tri_ldiveq_vec(tri t, double* b, idx step)
{
    const idx N = t.a.m;
    double* bb = b;
    int rc;
    if (N <= 0) return ORACLE_OK;
    if (step != 1) {
        bb = (double*)malloc(sizeof(double) * (size_t)N);
        if (!bb) return ORACLE_NOMEM;
        for (idx i = 0; i < N; ++i) bb[i] = b[i * step];
    }
    if (t.upper) {
        idx i2 = N;
        while (i2 > 0 && bb[i2 - 1] == 0.0) --i2;
        if (i2 == 0) rc = ORACLE_OK;
        else {
            tri s = tri_sub(t, 0, i2);
            rc = isrm(s.a) ? row_tri_ldiveq_vec(s, bb)
                 : iscm(s.a) ? col_tri_ldiveq_vec(s, bb)
                             : row_tri_ldiveq_vec(s, bb);
        }
    } else {
        idx i1 = 0;
        while (i1 < N && bb[i1] == 0.0) ++i1;
        if (i1 == N) rc = ORACLE_OK;
        else {
            tri s = tri_sub(t, i1, N);
            rc = isrm(s.a) ? row_tri_ldiveq_vec(s, bb + i1)
                 : iscm(s.a) ? col_tri_ldiveq_vec(s, bb + i1)
                             : row_tri_ldiveq_vec(s, bb + i1);
        }
    }
    if (step != 1) {
        for (idx i = 0; i < N; ++i) b[i * step] = bb[i];
        free(bb);
    }
    return rc;
}

/* Leaf solves with a row-major B: src/TMV_TriDiv_M.cpp:58-188. */
static int leaf_tri_ldiveq_rm(tri t, view B)
{
    const view A = t.a;
    const idx N = A.m, K = B.n;
    if (isrm(A)) {
        /* RowTriLDivEq: B.row(i) -= A.row(i,..) * B.rowRange(..); B.row(i) /= Aii */
        if (t.upper) {
            for (idx i = N - 1; i >= 0; --i) {
                for (idx c = 0; c < K; ++c) {
                    double s = 0.0;
                    for (idx j = i + 1; j < N; ++j) s += AT(A, i, j) * AT(B, j, c);
                    AT(B, i, c) -= s;
                }
                if (!t.unit) {
                    if (AT(A, i, i) == 0.0) return ORACLE_SINGULAR;
                    const double inv = 1.0 / AT(A, i, i);
                    for (idx c = 0; c < K; ++c) AT(B, i, c) *= inv;
                }
            }
        } else {
            for (idx i = 0; i < N; ++i) {
                for (idx c = 0; c < K; ++c) {
                    double s = 0.0;
                    for (idx j = 0; j < i; ++j) s += AT(A, i, j) * AT(B, j, c);
                    AT(B, i, c) -= s;
                }
                if (!t.unit) {
                    if (AT(A, i, i) == 0.0) return ORACLE_SINGULAR;
                    const double inv = 1.0 / AT(A, i, i);
                    for (idx c = 0; c < K; ++c) AT(B, i, c) *= inv;
                }
            }
        }
    } else {
        /* ColTriLDivEq: B.row(j) /= Ajj; B.rowRange(..) -= A.col(j,..) ^ B.row(j) */
        if (t.upper) {
            for (idx j = N - 1; j >= 0; --j) {
                if (!t.unit) {
                    if (AT(A, j, j) == 0.0) return ORACLE_SINGULAR;
                    const double inv = 1.0 / AT(A, j, j);
                    for (idx c = 0; c < K; ++c) AT(B, j, c) *= inv;
                }
                for (idx i = 0; i < j; ++i)
                    for (idx c = 0; c < K; ++c) AT(B, i, c) -= AT(A, i, j) * AT(B, j, c);
            }
        } else {
            for (idx j = 0; j < N; ++j) {
                if (!t.unit) {
                    if (AT(A, j, j) == 0.0) return ORACLE_SINGULAR;
                    const double inv = 1.0 / AT(A, j, j);
                    for (idx c = 0; c < K; ++c) AT(B, j, c) *= inv;
                }
                for (idx i = j + 1; i < N; ++i)
                    for (idx c = 0; c < K; ++c) AT(B, i, c) -= AT(A, i, j) * AT(B, j, c);
            }
        }
    }
    return ORACLE_OK;
}

#define TRI_DIV_BLOCKSIZE 64
#define TRI_DIV_BLOCKSIZE2 32

/* src/TMV_TriDiv_M.cpp:190-266: split at k = N/2 (rounded down to a
 * multiple of 64 when above 64) with a MultMM off-diagonal update; leaves
 * of <= 32 rows. */
static int nonblas_tri_ldiveq(tri t, view B)
{
    const idx N = t.a.m;
    int rc;
    if (N <= TRI_DIV_BLOCKSIZE2) {
        if (isrm(B)) return leaf_tri_ldiveq_rm(t, B);
        for (idx j = 0; j < B.n; ++j) {
            rc = tri_ldiveq_vec(t, &AT(B, 0, j), B.si);
            if (rc) return rc;
        }
        return ORACLE_OK;
    }
    idx k = N / 2;
    if (k > TRI_DIV_BLOCKSIZE) k = k / TRI_DIV_BLOCKSIZE * TRI_DIV_BLOCKSIZE;
    view B0 = sub(B, 0, k, 0, B.n), B1 = sub(B, k, N, 0, B.n);
    if (t.upper) {
        rc = nonblas_tri_ldiveq(tri_sub(t, k, N), B1);
        if (rc) return rc;
        rc = multmm_view(1, -1.0, sub(t.a, 0, k, k, N), B1, B0);
        if (rc) return rc;
        return nonblas_tri_ldiveq(tri_sub(t, 0, k), B0);
    } else {
        rc = nonblas_tri_ldiveq(tri_sub(t, 0, k), B0);
        if (rc) return rc;
        rc = multmm_view(1, -1.0, sub(t.a, k, N, 0, k), B0, B1);
        if (rc) return rc;
        return nonblas_tri_ldiveq(tri_sub(t, k, N), B1);
    }
}

/* src/TMV_TriDiv_M.cpp:583-710 (matrix) -> vector path for one column. */
static int tri_ldiveq(tri t, view B)
{
    if (B.m <= 0 || B.n <= 0) return ORACLE_OK;
    if (B.n == 1) return tri_ldiveq_vec(t, B.p, B.si);
    return nonblas_tri_ldiveq(t, B);
}

int oracle_tri_ldiveq(int upper, int unitdiag, ptrdiff_t n, const double* LU,
                      ptrdiff_t lda, ptrdiff_t nrhs, double* B, ptrdiff_t sBi,
                      ptrdiff_t sBj)
{
    tri t = {mkview((double*)LU, n, n, 1, lda), upper, unitdiag};
    return tri_ldiveq(t, mkview(B, n, nrhs, sBi, sBj));
}

/* ------------------------------------------------------------------ */
/* LU decomposition                                                    */
/* ------------------------------------------------------------------ */

#define LU_BLOCKSIZE 64

/* src/TMV_LUDecompose.cpp:217-407 */
static int recursive_lu(view A, idx* P)
{
    const idx N = A.n, M = A.m;
    const idx R = M < N ? M : N;
    int rc;
    if (R > 2) {
        idx N1 = R / 2;
        if (N1 > LU_BLOCKSIZE) N1 = (N1 / LU_BLOCKSIZE) * LU_BLOCKSIZE;
        view A0 = sub(A, 0, M, 0, N1);
        view A00 = sub(A0, 0, N1, 0, N1);
        view A10 = sub(A0, N1, M, 0, N1);
        view A1 = sub(A, 0, M, N1, N);
        view A01 = sub(A1, 0, N1, 0, N - N1);
        view A11 = sub(A1, N1, M, 0, N - N1);

        rc = recursive_lu(A0, P);
        if (rc) return rc;
        permute_rows(A1, P, 0, N1);
        {
            tri L00 = {A00, 0, 1};
            rc = tri_ldiveq(L00, A01);
            if (rc) return rc;
        }
        rc = multmm_view(1, -1.0, A10, A01, A11);
        if (rc) return rc;
        rc = recursive_lu(A11, P + N1);
        if (rc) return rc;
        for (idx i = N1; i < R; ++i) P[i] += N1;
        permute_rows(A0, P, N1, R);
    } else if (R == 2) {
        /* src/TMV_LUDecompose.cpp:274-358 */
        double* a0 = &AT(A, 0, 0);
        double* a1 = &AT(A, 0, 1);
        const idx s = A.si;
        idx ip0, ip1;
        double piv = max_abs_element(a0, M, s, &ip0);
        if (underflow(piv)) {
            ip0 = 0;
            piv = 0.0;
            for (idx i = 0; i < M; ++i) a0[i * s] = 0.0;
        }
        if (piv != 0.0) {
            if (ip0 != 0) {
                double t = a0[ip0 * s]; a0[ip0 * s] = a0[0]; a0[0] = t;
                t = a1[ip0 * s]; a1[ip0 * s] = a1[0]; a1[0] = t;
            }
            const double inv00 = 1.0 / a0[0];
            const double a01 = a1[0];
            piv = 0.0;
            ip1 = 1;
            for (idx i = 1; i < M; ++i) {
                a0[i * s] *= inv00;
                a1[i * s] -= a0[i * s] * a01;
                const double ab = fabs(a1[i * s]);
                if (ab > piv) { piv = ab; ip1 = i; }
            }
        } else {
            piv = max_abs_element(a1 + s, M - 1, s, &ip1);
            ++ip1;
        }
        if (underflow(piv)) {
            piv = 0.0;
            ip1 = 1;
            for (idx i = 1; i < M; ++i) a1[i * s] = 0.0;
        }
        if (piv != 0.0 && M > 2) {
            if (ip1 != 1) {
                double t = a1[ip1 * s]; a1[ip1 * s] = a1[s]; a1[s] = t;
                t = a0[ip1 * s]; a0[ip1 * s] = a0[s]; a0[s] = t;
            }
            const double inv11 = 1.0 / a1[s];
            for (idx i = 2; i < M; ++i) a1[i * s] *= inv11;
        }
        if (N > 2) {
            /* M == 2: U(0:2, 2:N) */
            view Ar = sub(A, 0, 2, 2, N);
            if (ip0 == 1) swap_rows(Ar, 0, 1);
            const double a01 = a1[0];
            for (idx j = 0; j < Ar.n; ++j) AT(Ar, 1, j) -= a01 * AT(Ar, 0, j);
        }
        P[0] = ip0;
        P[1] = ip1;
    } else if (R == 1) {
        /* src/TMV_LUDecompose.cpp:359-383 */
        double* a0 = &AT(A, 0, 0);
        const idx s = A.si;
        double piv = max_abs_element(a0, M, s, &P[0]);
        if (underflow(piv)) {
            piv = 0.0;
            P[0] = 0;
            for (idx i = 0; i < M; ++i) a0[i * s] = 0.0;
        }
        if (piv != 0.0) {
            if (P[0] != 0) {
                const double t = a0[P[0] * s]; a0[P[0] * s] = a0[0]; a0[0] = t;
            }
            const double inv = 1.0 / a0[0];
            for (idx i = 1; i < M; ++i) a0[i * s] *= inv;
        }
    }
    return ORACLE_OK;
}

int oracle_lu_decompose(ptrdiff_t m, ptrdiff_t n, double* A, ptrdiff_t sAi,
                        ptrdiff_t sAj, ptrdiff_t* P)
{
    /* src/TMV_LUDecompose.cpp:514-540: column-major in place; row-major via
     * the transpose (transposeSelf is a value-preserving relabelling for the
     * square case); other strides through a column-major copy. */
    view v = mkview(A, m, n, sAi, sAj);
    if (m <= 0 || n <= 0) return ORACLE_OK;
    if (iscm(v)) return recursive_lu(v, P);
    {
        /* Row-major: transposeSelf; LU_Decompose(A.transpose()); transposeSelf
         * factors A's own values and stores the factor in A's layout, which
         * is what factoring a column-major copy and writing it back does. */
        double* t = dense_copy(v);
        int rc;
        if (!t) return ORACLE_NOMEM;
        rc = recursive_lu(mkview(t, m, n, 1, m), P);
        for (idx j = 0; j < n; ++j)
            for (idx i = 0; i < m; ++i) AT(v, i, j) = t[i + j * m];
        free(t);
        return rc;
    }
}

/* ------------------------------------------------------------------ */
/* LU solves                                                           */
/* ------------------------------------------------------------------ */

int oracle_lu_ldiveq(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                     const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                     ptrdiff_t sBi, ptrdiff_t sBj)
{
    /* src/TMV_LUDiv.cpp:186-226, core 47-55 */
    view Bv = mkview(B, n, nrhs, sBi, sBj);
    tri L = {mkview((double*)LU, n, n, 1, lda), 0, 1};
    tri U = {mkview((double*)LU, n, n, 1, lda), 1, 0};
    int rc;
    permute_rows(Bv, P, 0, n);
    rc = tri_ldiveq(L, Bv);
    if (rc) return rc;
    return tri_ldiveq(U, Bv);
}

int oracle_lu_rdiveq(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                     const ptrdiff_t* P, ptrdiff_t nrows, double* B,
                     ptrdiff_t sBi, ptrdiff_t sBj)
{
    /* src/TMV_LUDiv.cpp:370-411, core 233-242: m %= U; m %= L;
     * m.reversePermuteCols(P).  m %= T is T^T.LDivEq(m^T)
     * (include/tmv/TMV_TriMatrix.h:945-946). */
    view Bt = mkview(B, n, nrows, sBj, sBi); /* m^T */
    tri Ut = {mkview((double*)LU, n, n, lda, 1), 0, 0}; /* U^T: lower, row-major */
    tri Lt = {mkview((double*)LU, n, n, lda, 1), 1, 1}; /* L^T: upper unit */
    int rc = tri_ldiveq(Ut, Bt);
    if (rc) return rc;
    rc = tri_ldiveq(Lt, Bt);
    if (rc) return rc;
    reverse_permute_rows(Bt, P, 0, n);
    return ORACLE_OK;
}

int oracle_divide(ptrdiff_t n, const double* A, ptrdiff_t nrhs,
                  const double* B, double* X, double* LU_out, ptrdiff_t* P_out)
{
    /* LUDiv copies A (src/TMV_LUD.cpp:64-87), factors, then doLDiv copies
     * B into X and solves in place (src/TMV_LUD.cpp:92-120). */
    double* lu = (double*)malloc(sizeof(double) * (size_t)(n * n > 0 ? n * n : 1));
    idx* P = (idx*)malloc(sizeof(idx) * (size_t)(n > 0 ? n : 1));
    int rc;
    if (!lu || !P) { free(lu); free(P); return ORACLE_NOMEM; }
    memcpy(lu, A, sizeof(double) * (size_t)(n * n));
    rc = oracle_lu_decompose(n, n, lu, 1, n, P);
    if (rc == ORACLE_OK) {
        memcpy(X, B, sizeof(double) * (size_t)(n * nrhs));
        rc = oracle_lu_ldiveq(n, lu, n, P, nrhs, X, 1, n);
    }
    if (LU_out) memcpy(LU_out, lu, sizeof(double) * (size_t)(n * n));
    if (P_out) memcpy(P_out, P, sizeof(idx) * (size_t)n);
    free(lu);
    free(P);
    return rc;
}

void oracle_lu_det(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                   const ptrdiff_t* P, double* det, double* logdet,
                   double* sign)
{
    /* src/TMV_LUD.cpp:132-156 with GenDiagMatrix::logDet
     * (src/TMV_DiagMatrix.cpp:59-85) and Permutation::det
     * (include/tmv/TMV_Permutation.h:273-278): logdet sums log|U_jj| (a zero
     * resets it to log(0) = -inf and the sign to 0); det = sign*exp(logdet). */
    double ld = 0.0, s = 1.0;
    int pd = 1;
    for (idx j = 0; j < n; ++j) {
        const double u = LU[j + j * lda];
        if (u == 0.0) {
            ld = log(0.0);
            s = 0.0;
        } else {
            const double a = fabs(u);
            ld += log(a);
            s *= u > 0 ? 1.0 : -1.0;
        }
        if (P[j] != j) pd = -pd;
    }
    s *= (double)pd;
    *logdet = ld;
    *sign = s;
    *det = s == 0.0 ? 0.0 : s * exp(ld);
}

/* ------------------------------------------------------------------ */
/* Inverses                                                            */
/* ------------------------------------------------------------------ */

/* In-place inverse of the upper triangle of U (with unit, the diagonal is
 * taken as 1 and neither read nor written).  src/TMV_TriInverse.cpp:49-88:
 * split k = N/2, rounded down to a multiple of 64 above 64; invert U00 and
 * U11; U01 = -U00 U01; U01 *= U11.  A zero U_jj is singular (TMV throws
 * SingularUpperTriMatrix). */
static int upper_invert(view U, int unit)
{
    const idx N = U.m;
    if (N <= 0) return ORACLE_OK;
    if (N == 1) {
        if (!unit) {
            if (AT(U, 0, 0) == 0.0) return ORACLE_SINGULAR;
            AT(U, 0, 0) = 1.0 / AT(U, 0, 0);
        }
        return ORACLE_OK;
    }
    idx k = N / 2;
    if (k > 64) k = k / 64 * 64;
    view U00 = sub(U, 0, k, 0, k), U01 = sub(U, 0, k, k, N), U11 = sub(U, k, N, k, N);
    int rc = upper_invert(U00, unit);
    if (rc) return rc;
    rc = upper_invert(U11, unit);
    if (rc) return rc;
    /* U01 = -U00 U01: row i of the result reads rows i.. of U01, so rows
     * are produced top down in place */
    for (idx j = 0; j < U01.n; ++j)
        for (idx i = 0; i < k; ++i) {
            double t = unit ? AT(U01, i, j) : AT(U00, i, i) * AT(U01, i, j);
            for (idx l = i + 1; l < k; ++l) t += AT(U00, i, l) * AT(U01, l, j);
            AT(U01, i, j) = -t;
        }
    /* U01 *= U11: column j of the result reads columns ..j, produced right
     * to left in place */
    for (idx i = 0; i < k; ++i)
        for (idx j = U01.n - 1; j >= 0; --j) {
            double t = unit ? AT(U01, i, j) : AT(U01, i, j) * AT(U11, j, j);
            for (idx l = 0; l < j; ++l) t += AT(U01, i, l) * AT(U11, l, j);
            AT(U01, i, j) = t;
        }
    return ORACLE_OK;
}

int oracle_lu_inverse(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                      const ptrdiff_t* P, double* M, ptrdiff_t ldm)
{
    /* src/TMV_LUInverse.cpp:38-52 (NonLapLUInverse) and 236-299
     * (LU_Inverse): minv = LUx; U.invertSelf(); L.invertSelf();
     * minv = U*L; minv.reversePermuteCols(P).  L.invertSelf() is the upper
     * routine on the transposed view (include/tmv/TMV_TriMatrix.h:2674-2675). */
    if (n <= 0) return ORACLE_OK;
    view Mv = mkview(M, n, n, 1, ldm);
    for (idx j = 0; j < n; ++j)
        for (idx i = 0; i < n; ++i) AT(Mv, i, j) = LU[i + j * lda];
    int rc = upper_invert(Mv, 0);
    if (rc) return rc;
    rc = upper_invert(transp(Mv), 1);
    if (rc) return rc;
    /* minv = U^-1 L^-1 (U upper with its diagonal, L unit lower) */
    double* T = (double*)malloc(sizeof(double) * (size_t)(n * n));
    if (!T) return ORACLE_NOMEM;
    for (idx j = 0; j < n; ++j)
        for (idx i = 0; i < n; ++i) {
            const idx l0 = i > j ? i : j;
            double t = l0 == j ? AT(Mv, i, j) : 0.0; /* U(i,j) * L(j,j) = U(i,j) */
            for (idx l = l0 == j ? j + 1 : l0; l < n; ++l) t += AT(Mv, i, l) * AT(Mv, l, j);
            T[i + j * n] = t;
        }
    for (idx j = 0; j < n; ++j)
        for (idx i = 0; i < n; ++i) AT(Mv, i, j) = T[i + j * n];
    free(T);
    reverse_permute_rows(transp(Mv), P, 0, n);
    return ORACLE_OK;
}

int oracle_lu_inverse_ata(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                          double* M, ptrdiff_t ldm)
{
    /* LUDiv::doMakeInverseATA, non-transposed case (src/TMV_LUD.cpp:172-200):
     * linv = L.inverse(); ata = linv * linv^T; ata /= U; ata %= U^T.
     * (A^T A)^-1 = U^-1 L^-1 L^-T U^-T: the permutation cancels. */
    if (n <= 0) return ORACLE_OK;
    view Mv = mkview(M, n, n, 1, ldm);
    double* Li = (double*)malloc(sizeof(double) * (size_t)(n * n));
    if (!Li) return ORACLE_NOMEM;
    view Lv = mkview(Li, n, n, 1, n);
    for (idx j = 0; j < n; ++j)
        for (idx i = 0; i < n; ++i) AT(Lv, i, j) = i > j ? LU[i + j * lda] : (i == j ? 1.0 : 0.0);
    int rc = upper_invert(transp(Lv), 1);
    if (rc) { free(Li); return rc; }
    /* ata = linv linv^T, linv unit lower */
    for (idx j = 0; j < n; ++j)
        for (idx i = 0; i < n; ++i) {
            const idx lmax = i < j ? i : j;
            double t = 0.0;
            for (idx l = 0; l <= lmax; ++l) t += AT(Lv, i, l) * AT(Lv, j, l);
            AT(Mv, i, j) = t;
        }
    free(Li);
    tri U = {mkview((double*)LU, n, n, 1, lda), 1, 0};
    rc = tri_ldiveq(U, Mv); /* ata /= U */
    if (rc) return rc;
    return tri_ldiveq(U, transp(Mv)); /* ata %= U^T: (ata^T) /= U */
}

int oracle_lu_is_singular(ptrdiff_t n, const double* LU, ptrdiff_t lda)
{
    /* src/TMV_LUD.cpp:204-209: diag.minAbs2Element() <=
     * epsilon * diag.maxAbs2Element(), with Abs2 = |x| for a real and the
     * first-extreme scans of src/TMV_Vector.cpp:539-600 (NaN never replaces
     * the running value). */
    if (n <= 0) return 0;
    double mn = fabs(LU[0]), mx = mn;
    for (idx j = 1; j < n; ++j) {
        const double a = fabs(LU[j + j * lda]);
        if (a > mx) mx = a;
        if (a < mn) mn = a;
    }
    return mn <= DBL_EPSILON * mx;
}

/* ------------------------------------------------------------------ */
/* Matrix-vector product                                               */
/* ------------------------------------------------------------------ */

/* UnitAMultMV1 (src/TMV_MultMV.cpp:186-215) with unit-step x and y: the row
 * form (RowMultMV, :80-122) for a row-major A, the column form (ColMultMV,
 * :124-184, which skips columns with x_j == 0) for a column-major one,
 * otherwise the row form when N >= M. */
static void unit_multmv(int add, view A, const double* x, double* y)
{
    const idx M = A.m, N = A.n;
    const int row = isrm(A) ? 1 : iscm(A) ? 0 : (N >= M);
    if (row) {
        for (idx i = 0; i < M; ++i) {
            double t = 0.0;
            for (idx j = 0; j < N; ++j) t += x[j] * AT(A, i, j);
            y[i] = add ? y[i] + t : t;
        }
        return;
    }
    idx j0 = 0;
    if (!add) {
        if (x[0] == 0.0)
            for (idx i = 0; i < M; ++i) y[i] = 0.0;
        else
            for (idx i = 0; i < M; ++i) y[i] = x[0] * AT(A, i, 0);
        j0 = 1;
    }
    for (idx j = j0; j < N; ++j)
        if (x[j] != 0.0)
            for (idx i = 0; i < M; ++i) y[i] += x[j] * AT(A, i, j);
}

int oracle_multmv(int add, double alpha, ptrdiff_t m, ptrdiff_t n, const double* A,
                  ptrdiff_t sAi, ptrdiff_t sAj, const double* x, ptrdiff_t incx,
                  double* y, ptrdiff_t incy)
{
    /* MultMV (src/TMV_MultMV.cpp:1134-1175): alpha == 0 or an empty x sets y
     * to zero unless add.  NonBlasMultMV (:298-380): with a strided x, or
     * alpha != 1 with M/4 >= N and unit-step y, x is scaled by alpha into a
     * copy first; otherwise with alpha != 1 or a strided y the product goes
     * to a temporary that is scaled into y; else straight into y. */
    if (m <= 0) return ORACLE_OK;
    if (n <= 0 || alpha == 0.0) {
        if (!add)
            for (idx i = 0; i < m; ++i) y[i * incy] = 0.0;
        return ORACLE_OK;
    }
    view Av = mkview((double*)A, m, n, sAi, sAj);
    double* xx = (double*)malloc(sizeof(double) * (size_t)n);
    double* yy = (double*)malloc(sizeof(double) * (size_t)m);
    if (!xx || !yy) { free(xx); free(yy); return ORACLE_NOMEM; }
    if (incx != 1 || (alpha != 1.0 && incy == 1 && m / 4 >= n)) {
        for (idx j = 0; j < n; ++j) xx[j] = alpha * x[j * incx];
        if (incy != 1) {
            unit_multmv(0, Av, xx, yy);
            for (idx i = 0; i < m; ++i) y[i * incy] = add ? y[i * incy] + yy[i] : yy[i];
        } else {
            unit_multmv(add, Av, xx, y);
        }
    } else if (incy != 1 || alpha != 1.0) {
        unit_multmv(0, Av, x, yy);
        for (idx i = 0; i < m; ++i) y[i * incy] = add ? y[i * incy] + alpha * yy[i] : alpha * yy[i];
    } else {
        unit_multmv(add, Av, x, y);
    }
    free(xx);
    free(yy);
    return ORACLE_OK;
}

int oracle_batched_divide(ptrdiff_t count, const ptrdiff_t* n,
                          const ptrdiff_t* nrhs, const ptrdiff_t* a_off,
                          const ptrdiff_t* b_off, const double* A, double* B,
                          int* status)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (idx i = 0; i < count; ++i) {
        const idx ni = n[i], ri = nrhs[i];
        double* lu = (double*)malloc(sizeof(double) * (size_t)(ni * ni > 0 ? ni * ni : 1));
        idx* P = (idx*)malloc(sizeof(idx) * (size_t)(ni > 0 ? ni : 1));
        if (!lu || !P) {
            status[i] = ORACLE_NOMEM;
        } else {
            memcpy(lu, A + a_off[i], sizeof(double) * (size_t)(ni * ni));
            status[i] = oracle_lu_decompose(ni, ni, lu, 1, ni, P);
            if (status[i] == ORACLE_OK)
                status[i] = oracle_lu_ldiveq(ni, lu, ni, P, ri, B + b_off[i], 1, ni);
        }
        free(lu);
        free(P);
    }
    return ORACLE_OK;
}
