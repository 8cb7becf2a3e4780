/* tmv_oracle_band.c -- CPU restatement of TMV 0.76's band LU (test
 * infrastructure only: the checker of the GPU's batched band LU; the product
 * never loads it).
 *
 * Storage is TMV's column-major band layout: element (i,j) of an n x n band
 * matrix with lo subdiagonals and hu superdiagonals at a[i + j*ldab]
 * (ldab = stepj >= lo + hu), for j - hu <= i <= j + lo.  The factorisation
 * needs hu = min(lo + hi, n - 1) superdiagonals for an input with hi: the
 * interchanges fill them (src/TMV_BandLUDecompose.cpp:93-96).
 *
 * Two algorithms, as TMV picks them by storage:
 *   ORACLE_BAND_GENERAL  NonLapBandLU_Decompose (column-major band,
 *                        src/TMV_BandLUDecompose.cpp:49-143) and the
 *                        column-oriented band upper solve
 *                        (src/TMV_BandTriDiv_V.cpp:148-235);
 *   ORACLE_BAND_TRIDIAG  NonLapTriDiagLU_Decompose (lo = hi = 1, the
 *                        diagonal-major storage BandLUDiv uses for a
 *                        tridiagonal matrix, src/TMV_BandLUD.cpp:61-63,
 *                        src/TMV_BandLUDecompose.cpp:144-200) and the
 *                        row-oriented upper solve (src/TMV_BandTriDiv_V.cpp:
 *                        63-135).
 * The storage here is column-major for both; only the arithmetic differs.
 */
#include <float.h>
#include <math.h>
#include <stddef.h>

#include "tmv_oracle.h"

typedef ptrdiff_t idx;

#define BA(a, ld, i, j) (a)[(i) + (j) * (ld)]

static idx imin(idx x, idx y) { return x < y ? x : y; }
static idx imax(idx x, idx y) { return x > y ? x : y; }

/* v[0..len) *= x as MultXV does it (src/TMV_MultXV.cpp:150-153): nothing
 * for x == 1, zeros for x == 0. */
static void scale(double* v, idx len, double x)
{
    if (len <= 0 || x == 1.0) return;
    for (idx i = 0; i < len; ++i) v[i] = (x == 0.0) ? 0.0 : x * v[i];
}

static void zero_fill(idx n, idx hi, idx hu, double* a, idx ldab)
{
    for (idx j = 0; j < n; ++j)
        for (idx d = hi + 1; d <= hu; ++d)
            if (j - d >= 0) BA(a, ldab, j - d, j) = 0.0;
}

/* NonLapBandLU_Decompose (src/TMV_BandLUDecompose.cpp:49-143): for each
 * column j < n-1 the pivot is the first index of the strict maximum |a| over
 * rows j..endcol-1 (FindMaxAbsElement, src/TMV_Vector.cpp:474-503); a
 * maximum below DBL_MIN (TMV_Underflow, include/tmv/TMV_Base.h:691-696)
 * zeroes the sub-column and takes no interchange; otherwise rows j and ip
 * are swapped over columns j..endrow-1 only (L's earlier columns are not
 * swapped: the solve applies the interchanges as it goes); the sub-column is
 * multiplied by the reciprocal of U(j,j) when that is nonzero (v /= x,
 * include/tmv/TMV_VectorArith.h:104-106, through MultXV); the window
 * (j+1..endcol-1) x (j+1..endrow-1) gets the outer product subtracted
 * column by column, a column whose U(j,c) is zero left alone (ColRank1Update,
 * src/TMV_Rank1_VVM.cpp:54-103).  endcol starts at lo+1, endrow at hu+1,
 * each grows by one per step up to n.  P[n-1] = n-1. */
static void band_general_decompose(idx n, idx lo, idx hu, double* a, idx ldab, idx* P)
{
    idx endcol = imin(lo + 1, n), endrow = imin(hu + 1, n);
    for (idx j = 0; j + 1 < n; ++j) {
        idx ip = 0;
        double piv = fabs(BA(a, ldab, j, j));
        for (idx i = 1; i < endcol - j; ++i) {
            const double v = fabs(BA(a, ldab, j + i, j));
            if (v > piv) {
                piv = v;
                ip = i;
            }
        }
        if (piv < DBL_MIN) {
            ip = 0;
            for (idx i = j; i < endcol; ++i) BA(a, ldab, i, j) = 0.0;
        }
        if (ip != 0) {
            ip += j;
            for (idx c = j; c < endrow; ++c) {
                const double t = BA(a, ldab, ip, c);
                BA(a, ldab, ip, c) = BA(a, ldab, j, c);
                BA(a, ldab, j, c) = t;
            }
            P[j] = ip;
        } else {
            P[j] = j;
        }
        const double ujj = BA(a, ldab, j, j);
        if (ujj != 0.0) scale(&BA(a, ldab, j + 1, j), endcol - j - 1, 1.0 / ujj);
        for (idx c = j + 1; c < endrow; ++c) {
            const double u = BA(a, ldab, j, c);
            if (u == 0.0) continue;
            for (idx i = j + 1; i < endcol; ++i) BA(a, ldab, i, c) -= BA(a, ldab, i, j) * u;
        }
        if (endcol < n) ++endcol;
        if (endrow < n) ++endrow;
    }
    P[n - 1] = n - 1;
}

/* NonLapTriDiagLU_Decompose (src/TMV_BandLUDecompose.cpp:144-200): rows j
 * and j+1 are swapped when |L(j+1,j)| > |U(j,j)| (over U(j,j), U(j,j+1) and,
 * below the last two columns, U(j,j+2)); then L(j+1,j) = L(j+1,j) / U(j,j)
 * (a true division), or both are zeroed when |U(j,j)| < DBL_MIN; then
 * U(j+1,j+1) -= L(j+1,j) U(j,j+1) and, after an interchange,
 * U(j+1,j+2) -= L(j+1,j) U(j,j+2). */
static void band_tridiag_decompose(idx n, double* a, idx ldab, idx* P)
{
    for (idx j = 0; j + 1 < n; ++j) {
        double* ujj = &BA(a, ldab, j, j);
        double* lj = &BA(a, ldab, j + 1, j);
        double* uj1 = &BA(a, ldab, j, j + 1);
        double* dj1 = &BA(a, ldab, j + 1, j + 1);
        const int pivot = fabs(*lj) > fabs(*ujj);
        if (pivot) {
            double t = *lj; *lj = *ujj; *ujj = t;
            t = *dj1; *dj1 = *uj1; *uj1 = t;
            if (j + 2 < n) {
                double* uj2 = &BA(a, ldab, j, j + 2);
                double* ej2 = &BA(a, ldab, j + 1, j + 2);
                t = *ej2; *ej2 = *uj2; *uj2 = t;
            }
            P[j] = j + 1;
        } else {
            P[j] = j;
        }
        if (fabs(*ujj) < DBL_MIN) {
            *ujj = 0.0;
            *lj = 0.0;
        } else {
            *lj = *lj / *ujj;
        }
        *dj1 -= *lj * *uj1;
        if (pivot && j + 2 < n) BA(a, ldab, j + 1, j + 2) -= *lj * BA(a, ldab, j, j + 2);
    }
    P[n - 1] = n - 1;
}

int oracle_band_lu_decompose(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, double* a,
                             ptrdiff_t ldab, ptrdiff_t* P)
{
    if (n < 0 || lo < 0 || hi < 0) return ORACLE_BAD_ARG;
    if (n == 0) return ORACLE_OK;
    if (lo > n - 1 || hi > n - 1) return ORACLE_BAD_ARG;
    if (algo == ORACLE_BAND_TRIDIAG && (lo != 1 || hi != 1)) return ORACLE_BAD_ARG;
    const idx hu = imin(lo + hi, n - 1);
    if (ldab < lo + hu) return ORACLE_BAD_ARG;
    zero_fill(n, hi, hu, a, ldab); /* BandLUDiv's copy: src/TMV_BandLUD.cpp:143-148 */
    if (lo == 0) {
        /* already U: src/TMV_BandLUDecompose.cpp:417-421 */
        for (idx i = 0; i < n; ++i) P[i] = i;
        return ORACLE_OK;
    }
    if (algo == ORACLE_BAND_TRIDIAG) band_tridiag_decompose(n, a, ldab, P);
    else band_general_decompose(n, lo, hu, a, ldab, P);
    return ORACLE_OK;
}

/* LU_PackedPL_LDivEq (src/TMV_BandLUDiv.cpp:79-118) on one column: at step
 * j swap b[j] and b[P[j]], then rows j+1..jn-1 -= L(.,j) b[j] (skipped when
 * b[j] is zero, as ColRank1Update skips a zero y), jn from lo+1 growing to
 * n. */
static void packed_pl(idx n, idx lo, const double* lu, idx ldab, const idx* P, double* b)
{
    if (lo == 0) return;
    idx jn = imin(lo + 1, n);
    for (idx j = 0; j + 1 < n; ++j) {
        if (P[j] != j) {
            const double t = b[j];
            b[j] = b[P[j]];
            b[P[j]] = t;
        }
        const double bj = b[j];
        if (bj != 0.0)
            for (idx i = j + 1; i < jn; ++i) b[i] -= BA(lu, ldab, i, j) * bj;
        if (jn < n) ++jn;
    }
}

/* The band upper solve of one column, as NonBlasTriLDivEq does it
 * (src/TMV_BandTriDiv_V.cpp:445-468): trailing zeros of b are trimmed
 * (i2 = one past the last nonzero; nothing to do when b is zero) and the
 * leading i2 x i2 block is solved with nh = min(hu, i2-1) superdiagonals:
 *   nh == 0: b /= its diagonal (DoDiagLDivEq1, src/TMV_DiagMatrix.cpp:
 *            296-341): every U(i,i), i < i2, must be nonzero, b[i] / U(i,i);
 *   column form (general): from the last row up, a zero b[j] is skipped,
 *            else b[j] / U(j,j) and b[i1..j-1] -= b[j] U(i1..j-1, j);
 *   row form (tridiagonal): from the last row up, b[i] -= U(i,k) b[k] for
 *            k = i+1..i+len (len = min(i2-1-i, nh)), then b[i] / U(i,i),
 *            every U(i,i) checked.
 * ORACLE_SINGULAR for a zero U(i,i) where TMV throws SingularBandLU. */
static int upper_solve(idx n, idx hu, int algo, const double* lu, idx ldab, double* b)
{
    idx i2 = n;
    while (i2 > 0 && b[i2 - 1] == 0.0) --i2;
    if (i2 == 0) return ORACLE_OK;
    const idx nh = imin(hu, i2 - 1);
    if (nh == 0) {
        for (idx i = 0; i < i2; ++i) {
            const double d = BA(lu, ldab, i, i);
            if (d == 0.0) return ORACLE_SINGULAR;
            b[i] = b[i] / d;
        }
        return ORACLE_OK;
    }
    if (algo == ORACLE_BAND_TRIDIAG) {
        for (idx i = i2 - 1; i >= 0; --i) {
            const idx len = imin(i2 - 1 - i, nh);
            for (idx k = i + 1; k <= i + len; ++k) b[i] -= b[k] * BA(lu, ldab, i, k);
            const double d = BA(lu, ldab, i, i);
            if (d == 0.0) return ORACLE_SINGULAR;
            b[i] = b[i] / d;
        }
        return ORACLE_OK;
    }
    for (idx j = i2 - 1; j >= 0; --j) {
        if (b[j] == 0.0) continue;
        const double d = BA(lu, ldab, j, j);
        if (d == 0.0) return ORACLE_SINGULAR;
        b[j] = b[j] / d;
        for (idx i = imax(0, j - nh); i < j; ++i) b[i] -= b[j] * BA(lu, ldab, i, j);
    }
    return ORACLE_OK;
}

/* LU_LDivEq for band factors, NonLapLU_LDivEq (src/TMV_BandLUDiv.cpp:
 * 139-163, 811-831): the packed P L solve, then TriLDivEq with U's hu
 * superdiagonals (src/TMV_BandTriDiv_M.cpp:391-425).  B is n x nrhs
 * column-major with leading dimension ldb, solved column by column; the one
 * exception is a 1 x nrhs B with ldb == 1, which TMV sees as row-major and
 * solves as a whole row (ColUpperTriLDivEq, src/TMV_BandTriDiv_M.cpp:
 * 87-125): U(0,0) must be nonzero and the row is multiplied by its
 * reciprocal. */
int oracle_band_lu_ldiveq(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, const double* lu,
                          ptrdiff_t ldab, const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                          ptrdiff_t ldb)
{
    if (n < 0 || lo < 0 || hi < 0 || nrhs < 0) return ORACLE_BAD_ARG;
    if (n == 0 || nrhs == 0) return ORACLE_OK;
    if (lo > n - 1 || hi > n - 1) return ORACLE_BAD_ARG;
    if (algo == ORACLE_BAND_TRIDIAG && (lo != 1 || hi != 1)) return ORACLE_BAD_ARG;
    const idx hu = imin(lo + hi, n - 1);
    if (n == 1 && nrhs > 1 && ldb == 1) {
        const double d = lu[0];
        if (d == 0.0) return ORACLE_SINGULAR;
        scale(B, nrhs, 1.0 / d);
        return ORACLE_OK;
    }
    for (idx q = 0; q < nrhs; ++q) {
        double* b = B + q * ldb;
        packed_pl(n, lo, lu, ldab, P, b);
        const int rc = upper_solve(n, hu, algo, lu, ldab, b);
        if (rc) return rc;
    }
    return ORACLE_OK;
}

/* LU_RDivEq for band factors, NonLapLU_RDivEq (src/TMV_BandLUDiv.cpp:
 * 244-290, 834-851): x P L U = m for each row of m (nrhs x n, row q at
 * B + q*ldb, unit step), in two passes per row b:
 *
 * 1. y U = b, i.e. TriLDivEq(Transpose(U), b) (src/TMV_BandTriDiv_M.cpp:
 *    391-425 with one column at a time, NonBlasTriLDivEq of
 *    src/TMV_BandTriDiv_V.cpp:445-468).  For hu == 0 the transpose is
 *    diagonal and the solve is upper_solve's diagonal one (trailing zeros
 *    trimmed, every U(i,i) of the leading part checked).  Otherwise leading
 *    zeros are trimmed (i1 = the first nonzero; nothing to do when b is
 *    zero) and the row form runs forward (DoRowLowerTriLDivEq, :240-313):
 *    b[i] -= b[j] U(j,i) for j = max(i1, i-hu) .. i-1 in that order, then
 *    b[i] / U(i,i), every U(i,i) from i1 on checked.
 * 2. z L = y (LU_PackedPL_RDivEq, :190-222): for j = n-2 down to 0,
 *    b[j] -= sum_k b[j+k] L(j+k, j) over k = 1..min(lo, n-1-j), then swap
 *    b[j] and b[P[j]].  The sum is MultMV's (src/TMV_MultMV.cpp:298-380 and
 *    the row form :80-122): a product into a temporary from 0.0, added into
 *    b[j] with alpha = -1.  The column-major factors give it x with unit
 *    step: t = 0.0 + L b ... and b[j] - t; the diagonal-major storage of
 *    the tridiagonal algorithm gives a strided x, which MultMV copies as
 *    alpha x: t' = 0.0 + (-L) b ... and b[j] + t' (the same value but for
 *    the sign of a zero).
 *
 * ORACLE_SINGULAR for a zero U(i,i) where TMV throws SingularBandLU;
 * ORACLE_BAD_ARG for an interchange P[j] outside rows j..min(j+lo, n-1)
 * (factors not made by the band LU), not applied.  The
 * 1 x nrhs special case with ldb == 1 is LDivEq's (the two passes see the
 * same one-entry transpose). */
static int rdiv_row(idx n, idx lo, idx hu, int algo, const double* lu, idx ldab, const idx* P, double* b)
{
    if (hu == 0) {
        const int rc = upper_solve(n, hu, algo, lu, ldab, b);
        if (rc) return rc;
    } else {
        idx i1 = 0;
        while (i1 < n && b[i1] == 0.0) ++i1;
        for (idx i = i1; i < n; ++i) {
            double v = b[i];
            for (idx j = imax(i1, i - hu); j < i; ++j) v -= b[j] * BA(lu, ldab, j, i);
            const double d = BA(lu, ldab, i, i);
            if (d == 0.0) return ORACLE_SINGULAR;
            b[i] = v / d;
        }
    }
    if (lo == 0) return ORACLE_OK;
    for (idx j = n - 2; j >= 0; --j) {
        const idx len = imin(lo, n - 1 - j);
        if (algo == ORACLE_BAND_TRIDIAG) {
            double t = 0.0;
            for (idx k = 1; k <= len; ++k) t += (-BA(lu, ldab, j + k, j)) * b[j + k];
            b[j] = b[j] + t;
        } else {
            double t = 0.0;
            for (idx k = 1; k <= len; ++k) t += BA(lu, ldab, j + k, j) * b[j + k];
            b[j] = b[j] - t;
        }
        const idx pj = P[j];
        if (pj < j || pj > j + lo || pj >= n) return ORACLE_BAD_ARG;
        if (pj != j) {
            const double t = b[j];
            b[j] = b[pj];
            b[pj] = t;
        }
    }
    return ORACLE_OK;
}

int oracle_band_lu_rdiveq(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, const double* lu,
                          ptrdiff_t ldab, const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                          ptrdiff_t ldb)
{
    if (n < 0 || lo < 0 || hi < 0 || nrhs < 0) return ORACLE_BAD_ARG;
    if (n == 0 || nrhs == 0) return ORACLE_OK;
    if (lo > n - 1 || hi > n - 1) return ORACLE_BAD_ARG;
    if (algo == ORACLE_BAND_TRIDIAG && (lo != 1 || hi != 1)) return ORACLE_BAD_ARG;
    const idx hu = imin(lo + hi, n - 1);
    if (n == 1 && nrhs > 1 && ldb == 1) {
        const double d = lu[0];
        if (d == 0.0) return ORACLE_SINGULAR;
        scale(B, nrhs, 1.0 / d);
        return ORACLE_OK;
    }
    for (idx q = 0; q < nrhs; ++q) {
        const int rc = rdiv_row(n, lo, hu, algo, lu, ldab, P, B + q * ldb);
        if (rc) return rc;
    }
    return ORACLE_OK;
}

/* The batched band workload on the host cores: for each system s (OpenMP
 * over systems) LU_Decompose and LU_LDivEq in place, system s's band at
 * ab + s*sab, interchanges at P + s*sp, right-hand sides at B + s*sb;
 * status[s] as oracle_band_lu_ldiveq returns it. */
int oracle_band_batched_solve(ptrdiff_t count, ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo,
                              double* ab, ptrdiff_t ldab, ptrdiff_t sab, ptrdiff_t* P, ptrdiff_t sp,
                              ptrdiff_t nrhs, double* B, ptrdiff_t ldb, ptrdiff_t sb, int* status)
{
#pragma omp parallel for schedule(static)
    for (idx s = 0; s < count; ++s) {
        int rc = oracle_band_lu_decompose(n, lo, hi, algo, ab + s * sab, ldab, P + s * sp);
        if (rc == ORACLE_OK)
            rc = oracle_band_lu_ldiveq(n, lo, hi, algo, ab + s * sab, ldab, P + s * sp, nrhs, B + s * sb,
                                       ldb);
        status[s] = rc;
    }
    return ORACLE_OK;
}
