/* tmv_oracle_z.c -- C restatement of TMV 0.76's LU_Decompose, LU_LDivEq,
 * LU_RDivEq and LUDiv::det/logDet for std::complex<double> (TEST
 * INFRASTRUCTURE ONLY).
 *
 * The complex instantiations follow the real ones (tmv_oracle.c) step for
 * step; what changes is TMV's complex arithmetic:
 *   - the pivot is the first strict maximum of TMV_ABS, TMV's own
 *     overflow-guarded modulus (include/tmv/TMV_Base.h:312-325; the scan of
 *     src/TMV_Vector.cpp:474-503), and a pivot underflows when that real
 *     maximum is below DBL_MIN (include/tmv/TMV_Base.h:692-696);
 *   - a column is scaled by TMV_InverseOf of the pivot, TMV's guarded complex
 *     reciprocal (include/tmv/TMV_Base.h:722-742; vector /= x is
 *     MultXV(TMV_InverseOf(x), v), include/tmv/TMV_VectorArith.h:104-118);
 *   - a division by a diagonal entry in the triangular solves is
 *     TMV_Divide(b, d) = b * TMV_InverseOf(d) (include/tmv/TMV_Base.h:747-752,
 *     src/TMV_TriDiv_V.cpp:186, 216, 355, 381).
 * The recursion's block steps (A01 /= A00.lowerTri(UnitDiag), A11 -= A10 A01)
 * are plain column-oriented loops with each entry's terms in k order, not
 * TMV's blocked complex kernels: values agree with TMV's to rounding (the
 * tests pin them against TMV itself), pivots are identical unless rounding
 * decides a tie.
 *
 * Matrices are column-major, complex entries interleaved (re, im), leading
 * dimension in complex elements; pivots in TMV's form (row j swapped with
 * P[j] at step j). */
#include <complex.h>
#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

#include "tmv_oracle.h"

typedef double _Complex zc;
typedef ptrdiff_t idx;

typedef struct {
    zc* p;
    idx m, n, ld; /* column-major */
} zview;

#define ZA(v, i, j) ((v).p[(i) + (j) * (v).ld])

static zview zsub(zview v, idx i1, idx i2, idx j1, idx j2)
{
    zview r = {v.p + i1 + j1 * v.ld, i2 - i1, j2 - j1, v.ld};
    return r;
}

/* TMV_ABS(std::complex<T>), include/tmv/TMV_Base.h:312-325. */
static double tmv_abs(zc x)
{
    double xr = creal(x), xi = cimag(x);
    const double ar = fabs(xr), ai = fabs(xi);
    const double s = ar < ai ? ai : ar; /* std::max */
    if (s == 0.0) return s;
    xr /= s;
    xi /= s;
    return s * sqrt(xr * xr + xi * xi);
}

/* TMV_InverseOf(std::complex<T>), include/tmv/TMV_Base.h:722-742. */
static zc tmv_inverse_of(zc x)
{
    double xr = creal(x), xi = cimag(x);
    if (fabs(xr) > fabs(xi)) {
        xi /= xr;
        const double denom = xr * (1.0 + xi * xi);
        return CMPLX(1.0 / denom, -xi / denom);
    } else if (fabs(xi) > 0.0) {
        xr /= xi;
        const double denom = xi * (1.0 + xr * xr);
        return CMPLX(xr / denom, -1.0 / denom);
    }
    /* (0, 0): TMV divides by zero as a real and lets it happen */
    return CMPLX(1.0 / xi, 0.0);
}

/* src/TMV_Vector.cpp:474-503 with TMV_ABS: first index of the strict maximum. */
static double max_abs_element(const zc* p, idx len, idx* imax)
{
    double mx = tmv_abs(p[0]);
    *imax = 0;
    for (idx i = 1; i < len; ++i) {
        const double a = tmv_abs(p[i]);
        if (a > mx) {
            mx = a;
            *imax = i;
        }
    }
    return mx;
}

static int underflow(double piv) { return fabs(piv) < DBL_MIN; }

static void swap_rows(zview A, idx i1, idx i2)
{
    if (i1 == i2) return;
    for (idx j = 0; j < A.n; ++j) {
        const zc t = ZA(A, i1, j);
        ZA(A, i1, j) = ZA(A, i2, j);
        ZA(A, i2, j) = t;
    }
}

static void scale(zc* p, idx len, zc x)
{
    for (idx i = 0; i < len; ++i) p[i] *= x;
}

/* src/TMV_LUDecompose.cpp:217-407 (RecursiveLUDecompose), complex T. */
static void recursive_lu(zview A, idx* P)
{
    const idx N = A.n, M = A.m;
    const idx R = M < N ? M : N;
    if (R > 2) {
        idx N1 = R / 2;
        if (N1 > 64) N1 = (N1 / 64) * 64;
        zview A0 = zsub(A, 0, M, 0, N1);
        zview A10 = zsub(A0, N1, M, 0, N1);
        zview A1 = zsub(A, 0, M, N1, N);
        zview A01 = zsub(A1, 0, N1, 0, N - N1);
        zview A11 = zsub(A1, N1, M, 0, N - N1);
        recursive_lu(A0, P);
        for (idx i = 0; i < N1; ++i) swap_rows(A1, i, P[i]);
        /* A01 /= A00.lowerTri(UnitDiag) */
        for (idx c = 0; c < A01.n; ++c)
            for (idx j = 0; j < N1; ++j) {
                const zc bj = ZA(A01, j, c);
                if (bj != 0.0)
                    for (idx i = j + 1; i < N1; ++i) ZA(A01, i, c) -= bj * ZA(A0, i, j);
            }
        /* A11 -= A10 * A01 */
        for (idx c = 0; c < A11.n; ++c)
            for (idx k = 0; k < N1; ++k) {
                const zc b = ZA(A01, k, c);
                for (idx i = 0; i < A11.m; ++i) ZA(A11, i, c) -= ZA(A10, i, k) * b;
            }
        recursive_lu(A11, P + N1);
        for (idx i = N1; i < R; ++i) P[i] += N1;
        for (idx i = N1; i < R; ++i) swap_rows(A0, i, P[i]);
    } else if (R == 2) {
        /* src/TMV_LUDecompose.cpp:274-358 */
        zc* a0 = &ZA(A, 0, 0);
        zc* a1 = &ZA(A, 0, 1);
        idx ip0, ip1;
        double piv = max_abs_element(a0, M, &ip0);
        if (underflow(piv)) {
            ip0 = 0;
            piv = 0.0;
            for (idx i = 0; i < M; ++i) a0[i] = 0.0;
        }
        if (piv != 0.0) {
            if (ip0 != 0) {
                zc t = a0[ip0]; a0[ip0] = a0[0]; a0[0] = t;
                t = a1[ip0]; a1[ip0] = a1[0]; a1[0] = t;
            }
            const zc inv00 = tmv_inverse_of(a0[0]);
            const zc a01 = a1[0];
            piv = 0.0;
            ip1 = 1;
            for (idx i = 1; i < M; ++i) {
                a0[i] *= inv00;
                a1[i] -= a0[i] * a01;
                const double ab = tmv_abs(a1[i]);
                if (ab > piv) { piv = ab; ip1 = i; }
            }
        } else {
            piv = max_abs_element(a1 + 1, M - 1, &ip1);
            ++ip1;
        }
        if (underflow(piv)) {
            piv = 0.0;
            ip1 = 1;
            for (idx i = 1; i < M; ++i) a1[i] = 0.0;
        }
        if (piv != 0.0 && M > 2) {
            if (ip1 != 1) {
                zc t = a1[ip1]; a1[ip1] = a1[1]; a1[1] = t;
                t = a0[ip1]; a0[ip1] = a0[1]; a0[1] = t;
            }
            scale(a1 + 2, M - 2, tmv_inverse_of(a1[1]));
        }
        if (N > 2) {
            /* M == 2: U(0:2, 2:N) */
            zview Ar = zsub(A, 0, 2, 2, N);
            if (ip0 == 1) swap_rows(Ar, 0, 1);
            const zc a01 = a1[0];
            for (idx j = 0; j < Ar.n; ++j) ZA(Ar, 1, j) -= a01 * ZA(Ar, 0, j);
        }
        P[0] = ip0;
        P[1] = ip1;
    } else if (R == 1) {
        /* src/TMV_LUDecompose.cpp:359-383 */
        zc* a0 = &ZA(A, 0, 0);
        double piv = max_abs_element(a0, M, &P[0]);
        if (underflow(piv)) {
            piv = 0.0;
            P[0] = 0;
            for (idx i = 0; i < M; ++i) a0[i] = 0.0;
        }
        if (piv != 0.0) {
            if (P[0] != 0) {
                const zc t = a0[P[0]]; a0[P[0]] = a0[0]; a0[0] = t;
            }
            scale(a0 + 1, M - 1, tmv_inverse_of(a0[0]));
        }
    }
}

int oracle_lu_decompose_z(ptrdiff_t n, double* A, ptrdiff_t lda, ptrdiff_t* P)
{
    if (n <= 0) return ORACLE_OK;
    zview v = {(zc*)A, n, n, lda};
    recursive_lu(v, P);
    return ORACLE_OK;
}

/* LU_LDivEq (src/TMV_LUDiv.cpp:186) for one column b: permuteRows(P), then
 * the column-oriented vector solves of src/TMV_TriDiv_V.cpp:322-398 (unit
 * lower L) and 148-236 (upper U), zero entries of b skipped, a division by
 * U(j,j) as TMV_Divide. */
static int lu_solve_col(zview LU, const ptrdiff_t* P, zc* b)
{
    const idx N = LU.m;
    for (idx i = 0; i < N; ++i) {
        const idx p = P[i];
        if (p != i) {
            const zc t = b[i];
            b[i] = b[p];
            b[p] = t;
        }
    }
    for (idx j = 0; j < N - 1; ++j)
        if (b[j] != 0.0)
            for (idx i = j + 1; i < N; ++i) b[i] -= b[j] * ZA(LU, i, j);
    for (idx j = N - 1; j > 0; --j) {
        if (b[j] != 0.0) {
            if (ZA(LU, j, j) == 0.0) return ORACLE_SINGULAR;
            b[j] = b[j] * tmv_inverse_of(ZA(LU, j, j));
            for (idx i = 0; i < j; ++i) b[i] -= b[j] * ZA(LU, i, j);
        }
    }
    if (N > 0 && b[0] != 0.0) {
        if (ZA(LU, 0, 0) == 0.0) return ORACLE_SINGULAR;
        b[0] = b[0] * tmv_inverse_of(ZA(LU, 0, 0));
    }
    return ORACLE_OK;
}

int oracle_lu_ldiveq_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                       ptrdiff_t nrhs, double* B, ptrdiff_t ldb)
{
    zview f = {(zc*)LU, n, n, lda};
    for (idx c = 0; c < nrhs; ++c) {
        const int rc = lu_solve_col(f, P, (zc*)B + c * ldb);
        if (rc) return rc;
    }
    return ORACLE_OK;
}

/* LU_RDivEq (src/TMV_LUDiv.cpp:370-411) for one row x of m: m %= U, m %= L,
 * m.reversePermuteCols(P), where m %= T is T^T.LDivEq(m^T)
 * (include/tmv/TMV_TriMatrix.h:945-946).  U^T and L^T of a column-major LU
 * are row-major, so TMV takes the row-oriented vector solves
 * (src/TMV_TriDiv_V.cpp:59-146, 237-320) after trimming the leading (lower)
 * or trailing (upper) zeros of x (:401-462); a zero U(i,i) met there is
 * singular. */
static int lu_rsolve_row(zview LU, const ptrdiff_t* P, zc* x, idx incx)
{
    const idx N = LU.m;
#define X(i) x[(i) * incx]
    /* x := x U^-1: U^T lower, non-unit */
    idx i1 = 0;
    while (i1 < N && X(i1) == 0.0) ++i1;
    for (idx i = i1; i < N; ++i) {
        for (idx j = i1; j < i; ++j) X(i) -= X(j) * ZA(LU, j, i);
        if (ZA(LU, i, i) == 0.0) return ORACLE_SINGULAR;
        X(i) = X(i) * tmv_inverse_of(ZA(LU, i, i));
    }
    /* x := x L^-1: L^T upper, unit */
    idx i2 = N;
    while (i2 > 0 && X(i2 - 1) == 0.0) --i2;
    for (idx i = i2 - 1; i >= 0; --i)
        for (idx j = i + 1; j < i2; ++j) X(i) -= X(j) * ZA(LU, j, i);
    /* reversePermuteCols(P) */
    for (idx i = N - 1; i >= 0; --i) {
        const idx p = P[i];
        if (p != i) {
            const zc t = X(i);
            X(i) = X(p);
            X(p) = t;
        }
    }
#undef X
    return ORACLE_OK;
}

int oracle_lu_rdiveq_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                       ptrdiff_t nrows, double* B, ptrdiff_t ldb)
{
    /* B: nrows x n, column-major (leading dimension ldb); each row in turn */
    zview f = {(zc*)LU, n, n, lda};
    for (idx r = 0; r < nrows; ++r) {
        const int rc = lu_rsolve_row(f, P, (zc*)B + r, ldb);
        if (rc) return rc;
    }
    return ORACLE_OK;
}

/* LUDiv::det / logDet (src/TMV_LUD.cpp:132-156) with GenDiagMatrix::logDet
 * (src/TMV_DiagMatrix.cpp:59-85): logdet sums log TMV_ABS(U_jj) and the
 * sign multiplies by TMV_SIGN(U_jj, |U_jj|) = U_jj / |U_jj| componentwise
 * (include/tmv/TMV_Base.h:708-716); a zero U_jj gives log(0) = -inf and sign
 * 0; the permutation's determinant multiplies the sign; det = sign
 * exp(logdet), 0 with a zero sign. */
void oracle_lu_det_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                     double* det, double* logdet, double* sign)
{
    zview f = {(zc*)LU, n, n, lda};
    zc s = 1.0;
    double ld = 0.0;
    int pd = 1;
    for (idx j = 0; j < n; ++j) {
        const zc u = ZA(f, j, j);
        if (u == 0.0) {
            ld = log(creal(u));
            s = 0.0;
        } else {
            const double a = tmv_abs(u);
            ld += log(a);
            const zc sg = a > 0 ? CMPLX(creal(u) / a, cimag(u) / a) : CMPLX(1.0, 0.0);
            s *= sg;
        }
        if (P[j] != j) pd = -pd;
    }
    s = (double)pd * s;
    *logdet = ld;
    sign[0] = creal(s);
    sign[1] = cimag(s);
    if (s == 0.0) {
        det[0] = 0.0;
        det[1] = 0.0;
    } else {
        const zc d = s * exp(ld);
        det[0] = creal(d);
        det[1] = cimag(d);
    }
}

/* MultMM<add> for std::complex<double> (src/TMV_MultMM.cpp:405 through the
 * tmv::Matrix expression surface): C = alpha A B, or C += alpha A B with
 * add.  Strided views (element (i, j) of X at X[i*sXi + j*sXj], complex
 * elements).  Each entry is alpha times its k-ordered sum, then stored or
 * added; TMV's blocked complex kernels sum in another order, so values agree
 * to rounding. */
int oracle_multmm_z(int add, const double* alpha, ptrdiff_t m, ptrdiff_t n, ptrdiff_t k,
                    const double* A, ptrdiff_t sAi, ptrdiff_t sAj, const double* B, ptrdiff_t sBi,
                    ptrdiff_t sBj, double* C, ptrdiff_t sCi, ptrdiff_t sCj)
{
    const zc* a = (const zc*)A;
    const zc* b = (const zc*)B;
    zc* c = (zc*)C;
    const zc al = CMPLX(alpha[0], alpha[1]);
    for (idx j = 0; j < n; ++j)
        for (idx i = 0; i < m; ++i) {
            zc s = 0.0;
            for (idx q = 0; q < k; ++q) s += a[i * sAi + q * sAj] * b[q * sBi + j * sBj];
            const zc v = al * s;
            if (add) c[i * sCi + j * sCj] += v;
            else c[i * sCi + j * sCj] = v;
        }
    return ORACLE_OK;
}
