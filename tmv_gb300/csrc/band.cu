// band.cu -- batched band LU: TMV's LU_Decompose(BandMatrixView<double>)
// (src/TMV_BandLUDecompose.cpp:383-425), LU_LDivEq and LU_RDivEq on band
// factors (src/TMV_BandLUDiv.cpp:811-851) for many systems of one shape, one
// thread per system.
//
// A band LU is a chain of n dependent steps, each touching a window of at
// most (lo+1) x (hu+1) entries, so one system offers no parallelism worth a
// CTA.  The GPU form is a batch: thousands of same-shaped band systems (line
// solves of a PDE grid, spline and filter systems), each run by one thread
// that keeps its window in registers.  The work is FP64 arithmetic (one IEEE
// division and about 2 lo hu products and differences per step), so the FP64
// pipe bounds it.
//
// Storage is TMV's column-major band layout per system: element (i,j) at
// ab[s*sab + i + j*ldab] for j-hu <= i <= j+lo, hu = min(lo+hi, n-1), with
// ldab >= lo + hu.  The fill diagonals hi+1..hu are outputs (the kernel writes
// every band slot once, as it leaves the window) and are never read.
//
// Results are TMV's bit for bit: the same pivot rule, the same operations in
// the same order, products and differences rounded separately (__dmul_rn,
// __dsub_rn: no contraction into FMA), true IEEE divisions.  Two algorithms,
// as TMV picks them by storage:
//   TMVG_BAND_GENERAL  NonLapBandLU_Decompose (:49-143) and the
//                      column-oriented upper solve (src/TMV_BandTriDiv_V.cpp:
//                      148-235);
//   TMVG_BAND_TRIDIAG  NonLapTriDiagLU_Decompose (:144-200), which BandLUDiv
//                      uses for a tridiagonal matrix (src/TMV_BandLUD.cpp:
//                      61-63), and the row-oriented upper solve
//                      (src/TMV_BandTriDiv_V.cpp:63-135).
#include <float.h>

#include <algorithm>

#include "common.cuh"

namespace tmvg {

namespace {

constexpr int kBandThreads = 128;

struct BandArgs {
    double* ab;
    int64_t sab, ldab;
    int64_t* P;
    int64_t sp;
    double* B;
    int64_t ldb, sb;
    int32_t* status;
    int64_t count;
    int64_t n;
    int lo, hi, hu, nrhs;
    int factor, solve;
    int trans;  // the solve is LU_RDivEq: each right-hand side is a row x of x P L U = m
};

__host__ __device__ __forceinline__ int64_t lmin(int64_t x, int64_t y) { return x < y ? x : y; }
__host__ __device__ __forceinline__ int64_t lmax(int64_t x, int64_t y) { return x > y ? x : y; }

// a - b*c with the product rounded first, as TMV's C++ evaluates it.
__device__ __forceinline__ double msub(double a, double b, double c)
{
    return __dsub_rn(a, __dmul_rn(b, c));
}

// Comparisons on the integer pipe: on GB300 a double comparison occupies the
// FP64 pipe (2 operations per SM per clock), the pipe this kernel is bound by.
// Non-negative doubles order like their bit patterns; |x| > |y| (false when
// either is NaN) is absbits(x) > absbits(y) with absbits(x) <= inf.
constexpr long long kAbs = 0x7fffffffffffffffLL;
constexpr long long kInfBits = 0x7ff0000000000000LL;
constexpr long long kDblMinBits = 0x0010000000000000LL;  // DBL_MIN
constexpr long long kOneBits = 0x3ff0000000000000LL;     // 1.0
__device__ __forceinline__ long long absbits(double x) { return __double_as_longlong(x) & kAbs; }
__device__ __forceinline__ bool nonzero(double x) { return absbits(x) != 0; }
__device__ __forceinline__ bool abs_greater(double x, double y)
{
    const long long bx = absbits(x);
    return bx > absbits(y) && bx <= kInfBits;
}
__device__ __forceinline__ bool underflows(double x) { return absbits(x) < kDblMinBits; }

// v *= x as MultXV does it (src/TMV_MultXV.cpp:150-153): unchanged for
// x == 1, zero for x == 0.
__device__ __forceinline__ double scale_by(double v, double x)
{
    const long long b = __double_as_longlong(x);
    return b == kOneBits ? v : ((b & kAbs) == 0 ? 0.0 : __dmul_rn(x, v));
}

// Steps whose loads are issued ahead (the loop is unrolled by this many so
// that each prefetch has a register slot of its own).  One: the next step's
// loads are issued as a step ends.  Deeper prefetching (2 and 4 steps) was
// measured on the 65536-system benchmark batch and gained nothing for the
// tridiagonal kernel (6.1 ms) and cost the (2,4) one occupancy (152
// registers: 8.7 -> 12.8 ms); the kernel is bound by the FP64 issue of its
// two IEEE divisions and few products per step, not by load latency.
template <int LOC, int HUC>
__host__ __device__ constexpr int band_prefetch() { return 1; }

// Row j+1+lo of the band, columns j+1..j+1+hu: the row that enters the window
// at the end of step j (zero outside the matrix).
template <int HUC>
__device__ __forceinline__ void band_load_row(const double* __restrict__ a, int64_t ldab, int64_t n, int lo,
                                              int hu, int64_t j, double (&dst)[HUC + 1])
{
    const int64_t nr = j + 1 + lo;
#pragma unroll
    for (int c = 0; c <= HUC; ++c)
        dst[c] = (c <= hu && nr < n && j + 1 + c < n) ? a[nr + (j + 1 + c) * ldab] : 0.0;
}

// ---------------------------------------------------------------------------
// Factorisation with the window W[r][c] = A(j+r, j+c), r <= lo, c <= hu, in
// registers.  LOC >= lo and HUC >= hu are the compile-time capacities;
// entries outside the runtime window stay zero.  At step j the column j
// (rows j..j+lo) and the row j (columns j+1..j+hu) are final and stored; the
// window then moves one step down the diagonal and takes in row j+1+lo,
// which no earlier step touched (its loads were issued PD steps earlier).
// Its new column j+1+hu holds fill above row j+1+lo (zero).
// ---------------------------------------------------------------------------
//
// With FUSE, the packed P L solve of one right-hand side b (the forward part
// of band_solve_one, LU_PackedPL_LDivEq) runs inside the same loop: step j's
// interchange and L column are final when the step ends (TMV's band LU never
// swaps L's earlier columns), so b's window y[r] = b[j+r] takes the same
// operations in the same order as in a separate pass, without reloading L,
// P and b.  *last_nz receives the last nonzero row of the result (-1: none).
// Needs lo >= 1.
template <int LOC, int HUC, bool TRID, bool FUSE = false>
__device__ void band_factor(double* __restrict__ a, int64_t ldab, int64_t* __restrict__ P, int64_t n,
                            int lo, int hi, int hu, double* __restrict__ b = nullptr,
                            int64_t* last_nz = nullptr)
{
    if (lo == 0) {  // already U (src/TMV_BandLUDecompose.cpp:417-421); no fill
        for (int64_t i = 0; i < n; ++i) P[i] = i;
        return;
    }
    constexpr int PD = band_prefetch<LOC, HUC>();
    double y[LOC + 1];
    double ypre[PD];
    int64_t lnz = -1;
    if (FUSE) {
#pragma unroll
        for (int r = 0; r <= LOC; ++r) y[r] = (r <= lo && r < n) ? b[r] : 0.0;
#pragma unroll
        for (int u = 0; u < PD; ++u) ypre[u] = (u + 1 + lo < n) ? b[u + 1 + lo] : 0.0;
    }
    double W[LOC + 1][HUC + 1];
#pragma unroll
    for (int r = 0; r <= LOC; ++r)
#pragma unroll
        for (int c = 0; c <= HUC; ++c) {
            const bool in = r <= lo && c <= hu && r < n && c < n && c - r <= hi;
            W[r][c] = in ? a[r + c * ldab] : 0.0;
        }
    double pre[PD][HUC + 1];
#pragma unroll
    for (int u = 0; u < PD; ++u) band_load_row<HUC>(a, ldab, n, lo, hu, u, pre[u]);
    for (int64_t j0 = 0; j0 < n; j0 += PD) {
#pragma unroll
        for (int u = 0; u < PD; ++u) {
            const int64_t j = j0 + u;
            if (j >= n) break;
            const int rlim = (int)lmin(lo + 1, n - j);  // rows j..j+rlim-1
            const int clim = (int)lmin(hu + 1, n - j);  // columns j..j+clim-1
            if (j + 1 < n) {
                if (TRID) {
                    const bool pivot = abs_greater(W[1][0], W[0][0]);
                    if (pivot) {
#pragma unroll
                        for (int c = 0; c <= 2; ++c) {
                            const double t = W[0][c];
                            W[0][c] = W[1][c];
                            W[1][c] = t;
                        }
                    }
                    P[j] = j + (pivot ? 1 : 0);
                    if (underflows(W[0][0])) {
                        W[0][0] = 0.0;
                        W[1][0] = 0.0;
                    } else {
                        W[1][0] = W[1][0] / W[0][0];
                    }
                    W[1][1] = msub(W[1][1], W[1][0], W[0][1]);
                    if (pivot && j + 2 < n) W[1][2] = msub(W[1][2], W[1][0], W[0][2]);
                    if (FUSE) {
                        if (pivot) {
                            const double t = y[0];
                            y[0] = y[1];
                            y[1] = t;
                        }
                        if (nonzero(y[0])) y[1] = msub(y[1], W[1][0], y[0]);
                    }
                } else {
                    // first strict maximum of |A(j..j+rlim-1, j)|
                    double piv = W[0][0];
                    int ip = 0;
#pragma unroll
                    for (int r = 1; r <= LOC; ++r)
                        if (r < rlim && abs_greater(W[r][0], piv)) {
                            piv = W[r][0];
                            ip = r;
                        }
                    if (underflows(piv)) {  // TMV_Underflow: zero the column, no interchange
                        ip = 0;
#pragma unroll
                        for (int r = 0; r <= LOC; ++r)
                            if (r < rlim) W[r][0] = 0.0;
                    }
#pragma unroll
                    for (int r = 1; r <= LOC; ++r)
                        if (r == ip)
#pragma unroll
                            for (int c = 0; c <= HUC; ++c) {
                                const double t = W[0][c];
                                W[0][c] = W[r][c];
                                W[r][c] = t;
                            }
                    P[j] = j + ip;
                    const double ujj = W[0][0];
                    if (nonzero(ujj)) {
                        const double inv = 1.0 / ujj;
#pragma unroll
                        for (int r = 1; r <= LOC; ++r)
                            if (r < rlim) W[r][0] = scale_by(W[r][0], inv);
                    }
                    // outer-product update, a column with a zero U(j,c) left alone
#pragma unroll
                    for (int c = 1; c <= HUC; ++c) {
                        const double uc = W[0][c];
                        if (c < clim && nonzero(uc))
#pragma unroll
                            for (int r = 1; r <= LOC; ++r)
                                if (r < rlim) W[r][c] = msub(W[r][c], W[r][0], uc);
                    }
                    if (FUSE) {
#pragma unroll
                        for (int r = 1; r <= LOC; ++r)
                            if (r == ip) {
                                const double t = y[0];
                                y[0] = y[r];
                                y[r] = t;
                            }
                        const double bj = y[0];
                        if (nonzero(bj))
#pragma unroll
                            for (int r = 1; r <= LOC; ++r)
                                if (r < rlim) y[r] = msub(y[r], W[r][0], bj);
                    }
                }
            } else {
                P[j] = j;
            }
            // column j (L and U(j,j)) and row j of U leave the window
#pragma unroll
            for (int r = 0; r <= LOC; ++r)
                if (r < rlim) a[(j + r) + j * ldab] = W[r][0];
#pragma unroll
            for (int c = 1; c <= HUC; ++c)
                if (c < clim) a[j + (j + c) * ldab] = W[0][c];
            if (FUSE) {
                b[j] = y[0];
                if (nonzero(y[0])) lnz = j;
            }
            if (j + 1 == n) break;
            if (FUSE) {
                // b[j+1+lo] enters (untouched so far: the window reached row j+lo)
#pragma unroll
                for (int r = 0; r < LOC; ++r) y[r] = y[r + 1];
                y[LOC] = 0.0;
#pragma unroll
                for (int r = 0; r <= LOC; ++r)
                    if (r == lo) y[r] = ypre[u];
                ypre[u] = (j + 1 + lo + PD < n) ? b[j + 1 + lo + PD] : 0.0;
            }
#pragma unroll
            for (int r = 0; r <= LOC; ++r)
#pragma unroll
                for (int c = 0; c <= HUC; ++c) W[r][c] = (r < LOC && c < HUC) ? W[r + 1][c + 1] : 0.0;
#pragma unroll
            for (int r = 0; r <= LOC; ++r)
                if (r == lo)
#pragma unroll
                    for (int c = 0; c <= HUC; ++c)
                        if (c <= hu) W[r][c] = pre[u][c];
            band_load_row<HUC>(a, ldab, n, lo, hu, j + PD, pre[u]);
        }
    }
    if (FUSE) *last_nz = lnz;
}

// ---------------------------------------------------------------------------
// One right-hand side: the packed P L solve (LU_PackedPL_LDivEq,
// src/TMV_BandLUDiv.cpp:79-118) with the window y[r] = b[j+r] in registers,
// then the upper solve on the leading i2 rows, i2 = one past the last nonzero
// (NonBlasTriLDivEq trims trailing zeros, src/TMV_BandTriDiv_V.cpp:455-466):
// a diagonal U (hu == 0) divides every row < i2 after checking its U(i,i)
// (DoDiagLDivEq1, src/TMV_DiagMatrix.cpp:296-341); otherwise the column form
// (zero entries skipped) or, for the tridiagonal algorithm, the row form,
// each with its window x[k] = b[j-k] (column) or b[i+k] (row) in registers.
// The loads of each step (interchange, L or U column, entering b) are issued
// PD steps ahead.  Returns 0, 1 for a zero U(j,j) where TMV throws
// SingularBandLU, or 2 for an interchange P[j] outside rows
// j..min(j+lo, n-1) (factors not made by the band LU), which is not applied.
// ---------------------------------------------------------------------------
template <int LOC>
struct FwdLoads {
    int64_t p;
    double l[LOC + 1];  // L(j+r, j), r = 1..lo
    double bn;          // b[j+1+lo]
};

template <int LOC>
__device__ __forceinline__ void band_fwd_load(const double* __restrict__ a, int64_t ldab,
                                              const int64_t* __restrict__ P, const double* __restrict__ b,
                                              int64_t n, int lo, int64_t j, FwdLoads<LOC>& f)
{
    f.p = j + 1 < n ? P[j] : j;
#pragma unroll
    for (int r = 1; r <= LOC; ++r) f.l[r] = (r <= lo && j + r < n) ? a[(j + r) + j * ldab] : 0.0;
    const int64_t nr = j + 1 + lo;
    f.bn = nr < n ? b[nr] : 0.0;
}

template <int HUC>
struct BwdLoads {
    double u[HUC + 1];  // U(j-k, j), k = 0..hu (u[0] = U(j,j))
    double bn;          // b[j-1-hu]
};

template <int HUC>
__device__ __forceinline__ void band_bwd_load(const double* __restrict__ a, int64_t ldab,
                                              const double* __restrict__ b, int hu, int64_t j, BwdLoads<HUC>& f)
{
#pragma unroll
    for (int k = 0; k <= HUC; ++k) f.u[k] = (k <= hu && j - k >= 0 && j >= 0) ? a[(j - k) + j * ldab] : 0.0;
    const int64_t nr = j - 1 - hu;
    f.bn = (nr >= 0 && j >= 0) ? b[nr] : 0.0;
}

// The upper solve of band_solve_one on rows below i2 (one past the last
// nonzero after the P L solve).
template <int HUC, bool TRID>
__device__ int band_upper_solve(const double* __restrict__ a, int64_t ldab, int64_t n, int hu,
                                double* __restrict__ b, int64_t i2)
{
    constexpr int PD = band_prefetch<1, HUC>();
    if (i2 == 0) return 0;
    if (hu == 0) {
        for (int64_t i = 0; i < i2; ++i) {
            const double d = a[i + i * ldab];
            if (!nonzero(d)) return 1;
            b[i] = b[i] / d;
        }
        return 0;
    }
    if (TRID) {
        const int64_t nh = lmin(hu, i2 - 1);
        double x1 = 0.0, x2 = 0.0;  // b[i+1], b[i+2], solved
        for (int64_t i = i2 - 1; i >= 0; --i) {
            const int64_t len = lmin(i2 - 1 - i, nh);
            double v = b[i];
            if (len >= 1) v = msub(v, x1, a[i + (i + 1) * ldab]);
            if (len >= 2) v = msub(v, x2, a[i + (i + 2) * ldab]);
            const double d = a[i + i * ldab];
            if (!nonzero(d)) return 1;
            v = v / d;
            b[i] = v;
            x2 = x1;
            x1 = v;
        }
        return 0;
    }
    double x[HUC + 1];
    {
        const int64_t j = i2 - 1;
#pragma unroll
        for (int k = 0; k <= HUC; ++k) x[k] = (k <= hu && j - k >= 0) ? b[j - k] : 0.0;
    }
    BwdLoads<HUC> f[PD];
#pragma unroll
    for (int u = 0; u < PD; ++u) band_bwd_load<HUC>(a, ldab, b, hu, i2 - 1 - u, f[u]);
    for (int64_t j0 = i2 - 1; j0 >= 0; j0 -= PD) {
#pragma unroll
        for (int u = 0; u < PD; ++u) {
            const int64_t j = j0 - u;
            if (j < 0) break;
            const double bj0 = x[0];
            if (nonzero(bj0)) {
                const double d = f[u].u[0];
                if (!nonzero(d)) return 1;
                const double bj = bj0 / d;
                x[0] = bj;
#pragma unroll
                for (int k = 1; k <= HUC; ++k)
                    if (k <= hu && j - k >= 0) x[k] = msub(x[k], bj, f[u].u[k]);
            }
            b[j] = x[0];
            const double bn = f[u].bn;
#pragma unroll
            for (int k = 0; k < HUC; ++k) x[k] = x[k + 1];
            x[HUC] = 0.0;
#pragma unroll
            for (int k = 0; k <= HUC; ++k)
                if (k == hu) x[k] = bn;
            // b[j-1-hu-PD] is below the window: not yet touched by this pass
            band_bwd_load<HUC>(a, ldab, b, hu, j - PD, f[u]);
        }
    }
    return 0;
}

template <int LOC, int HUC, bool TRID>
__device__ int band_solve_one(const double* __restrict__ a, int64_t ldab, const int64_t* __restrict__ P,
                              int64_t n, int lo, int hu, double* __restrict__ b)
{
    constexpr int PD = band_prefetch<LOC, HUC>();
    int64_t last_nz = -1;
    if (lo == 0) {
        for (int64_t j = n - 1; j >= 0; --j)
            if (nonzero(b[j])) {
                last_nz = j;
                break;
            }
    } else {
        double y[LOC + 1];
#pragma unroll
        for (int r = 0; r <= LOC; ++r) y[r] = (r <= lo && r < n) ? b[r] : 0.0;
        FwdLoads<LOC> f[PD];
#pragma unroll
        for (int u = 0; u < PD; ++u) band_fwd_load<LOC>(a, ldab, P, b, n, lo, u, f[u]);
        for (int64_t j0 = 0; j0 < n; j0 += PD) {
#pragma unroll
            for (int u = 0; u < PD; ++u) {
                const int64_t j = j0 + u;
                if (j >= n) break;
                if (j + 1 < n) {
                    const int64_t pj = f[u].p;
                    if (pj < j || pj > j + lo || pj >= n) return 2;
                    const int d = (int)(pj - j);
#pragma unroll
                    for (int r = 1; r <= LOC; ++r)
                        if (r == d) {
                            const double t = y[0];
                            y[0] = y[r];
                            y[r] = t;
                        }
                    const double bj = y[0];
                    if (nonzero(bj))
#pragma unroll
                        for (int r = 1; r <= LOC; ++r)
                            if (r <= lo && j + r < n) y[r] = msub(y[r], f[u].l[r], bj);
                }
                b[j] = y[0];
                if (nonzero(y[0])) last_nz = j;
                const double bn = f[u].bn;
#pragma unroll
                for (int r = 0; r < LOC; ++r) y[r] = y[r + 1];
                y[LOC] = 0.0;
#pragma unroll
                for (int r = 0; r <= LOC; ++r)
                    if (r == lo) y[r] = bn;
                // b[j+1+lo+PD] is not yet touched: the window covers rows up to j+1+lo
                band_fwd_load<LOC>(a, ldab, P, b, n, lo, j + PD, f[u]);
            }
        }
    }
    return band_upper_solve<HUC, TRID>(a, ldab, n, hu, b, last_nz + 1);
}

// ---------------------------------------------------------------------------
// One row of LU_RDivEq (NonLapLU_RDivEq, src/TMV_BandLUDiv.cpp:244-290):
// x P L U = m, b a row of m with unit step.
//  1. y U = b, TriLDivEq(Transpose(U), b) (NonBlasTriLDivEq,
//     src/TMV_BandTriDiv_V.cpp:445-468): for hu == 0 the diagonal solve of the
//     leading part up to the last nonzero (every U(i,i) there checked);
//     otherwise, from the first nonzero i1 on, the forward row form
//     (DoRowLowerTriLDivEq, :240-313): b[i] -= b[j] U(j,i) for j =
//     max(i1, i-hu) .. i-1 in that order, then b[i] / U(i,i), every U(i,i)
//     checked.  Window x[k] = solved b[i-1-k] in registers; the loads of
//     step i (U's column i, b[i]) are issued PD steps ahead.
//  2. z L = y (LU_PackedPL_RDivEq, :190-222): for j = n-2 down to 0,
//     b[j] -= sum_k L(j+k, j) b[j+k], k = 1..min(lo, n-1-j), the sum formed
//     from 0.0 as MultMV forms it (src/TMV_MultMV.cpp:298-380, row form
//     :80-122); the diagonal-major factors of the tridiagonal algorithm give
//     MultMV a strided x, which it copies scaled by -1, so there the sum is of
//     (-L) b and is added.  Then b[j] and b[P[j]] are swapped.  Window
//     y[r] = b[j+r] in registers; b[j+lo] is final once step j is done.
// Returns 0, 1 for a zero U(i,i) where TMV throws SingularBandLU, or 2 for
// an interchange outside rows j..min(j+lo, n-1), which is not applied.
// ---------------------------------------------------------------------------
template <int HUC>
struct RFwdLoads {
    double u[HUC + 1];  // U(i-k, i), k = 0..hu (u[0] = U(i,i))
    double bn;          // b[i]
};

template <int HUC>
__device__ __forceinline__ void band_rfwd_load(const double* __restrict__ a, int64_t ldab,
                                               const double* __restrict__ b, int64_t n, int hu, int64_t i,
                                               RFwdLoads<HUC>& f)
{
#pragma unroll
    for (int k = 0; k <= HUC; ++k) f.u[k] = (k <= hu && i - k >= 0 && i < n) ? a[(i - k) + i * ldab] : 0.0;
    f.bn = i < n ? b[i] : 0.0;
}

template <int LOC>
struct RBwdLoads {
    int64_t p;
    double l[LOC + 1];  // L(j+r, j), r = 1..lo
    double bn;          // b[j]
};

template <int LOC>
__device__ __forceinline__ void band_rbwd_load(const double* __restrict__ a, int64_t ldab,
                                               const int64_t* __restrict__ P, const double* __restrict__ b,
                                               int64_t n, int lo, int64_t j, RBwdLoads<LOC>& f)
{
    f.p = j >= 0 ? P[j] : 0;
#pragma unroll
    for (int r = 1; r <= LOC; ++r) f.l[r] = (r <= lo && j >= 0 && j + r < n) ? a[(j + r) + j * ldab] : 0.0;
    f.bn = j >= 0 ? b[j] : 0.0;
}

// b[i] / U(i,i) for i below one past the last nonzero, every U(i,i) there
// checked (the diagonal solve of both directions, DoDiagLDivEq1,
// src/TMV_DiagMatrix.cpp:296-341).
__device__ __forceinline__ int band_diag_solve(const double* __restrict__ a, int64_t ldab, int64_t n,
                                               double* __restrict__ b)
{
    int64_t i2 = n;
    while (i2 > 0 && !nonzero(b[i2 - 1])) --i2;
    for (int64_t i = 0; i < i2; ++i) {
        const double d = a[i + i * ldab];
        if (!nonzero(d)) return 1;
        b[i] = b[i] / d;
    }
    return 0;
}

template <int LOC, int HUC, bool TRID>
__device__ int band_rsolve_one(const double* __restrict__ a, int64_t ldab, const int64_t* __restrict__ P,
                               int64_t n, int lo, int hu, double* __restrict__ b)
{
    constexpr int PD = band_prefetch<LOC, HUC>();
    if (hu == 0) {
        const int st = band_diag_solve(a, ldab, n, b);
        if (st) return st;
    } else {
        int64_t i1 = 0;
        while (i1 < n && !nonzero(b[i1])) ++i1;
        double x[HUC];
#pragma unroll
        for (int k = 0; k < HUC; ++k) x[k] = 0.0;
        RFwdLoads<HUC> f[PD];
#pragma unroll
        for (int u = 0; u < PD; ++u) band_rfwd_load<HUC>(a, ldab, b, n, hu, i1 + u, f[u]);
        for (int64_t i0 = i1; i0 < n; i0 += PD) {
#pragma unroll
            for (int u = 0; u < PD; ++u) {
                const int64_t i = i0 + u;
                if (i >= n) break;
                double v = f[u].bn;
#pragma unroll
                for (int k = HUC - 1; k >= 0; --k)
                    if (k < hu && i - 1 - k >= i1) v = msub(v, x[k], f[u].u[k + 1]);
                const double d = f[u].u[0];
                if (!nonzero(d)) return 1;
                v = v / d;
                b[i] = v;
#pragma unroll
                for (int k = HUC - 1; k > 0; --k) x[k] = x[k - 1];
                x[0] = v;
                // b[i+PD] is not yet written: this pass writes b[i] in order
                band_rfwd_load<HUC>(a, ldab, b, n, hu, i + PD, f[u]);
            }
        }
    }
    if (lo == 0) return 0;
    double y[LOC + 1];
    y[0] = 0.0;
#pragma unroll
    for (int r = 1; r <= LOC; ++r) y[r] = (r <= lo && n - 2 + r < n) ? b[n - 2 + r] : 0.0;
    RBwdLoads<LOC> g[PD];
#pragma unroll
    for (int u = 0; u < PD; ++u) band_rbwd_load<LOC>(a, ldab, P, b, n, lo, n - 2 - u, g[u]);
    for (int64_t j0 = n - 2; j0 >= 0; j0 -= PD) {
#pragma unroll
        for (int u = 0; u < PD; ++u) {
            const int64_t j = j0 - u;
            if (j < 0) break;
            y[0] = g[u].bn;
            double t = 0.0;
            if (TRID) {
#pragma unroll
                for (int r = 1; r <= LOC; ++r)
                    if (r <= lo && j + r < n) t = __dadd_rn(t, __dmul_rn(-g[u].l[r], y[r]));
                y[0] = __dadd_rn(y[0], t);
            } else {
#pragma unroll
                for (int r = 1; r <= LOC; ++r)
                    if (r <= lo && j + r < n) t = __dadd_rn(t, __dmul_rn(g[u].l[r], y[r]));
                y[0] = __dsub_rn(y[0], t);
            }
            const int64_t pj = g[u].p;
            if (pj < j || pj > j + lo || pj >= n) return 2;
            const int dd = (int)(pj - j);
#pragma unroll
            for (int r = 1; r <= LOC; ++r)
                if (r == dd) {
                    const double w = y[0];
                    y[0] = y[r];
                    y[r] = w;
                }
            // b[j+lo] is final: later steps reach rows below j+lo only
#pragma unroll
            for (int r = 1; r <= LOC; ++r)
                if (r == lo && j + r < n) b[j + r] = y[r];
#pragma unroll
            for (int r = LOC; r > 0; --r) y[r] = y[r - 1];
            // b[j-PD] is below every row this pass has written
            band_rbwd_load<LOC>(a, ldab, P, b, n, lo, j - PD, g[u]);
        }
    }
    // rows 0..lo-1, still in the window (y[r] = b[r-1])
#pragma unroll
    for (int r = 1; r <= LOC; ++r)
        if (r <= lo) b[r - 1] = y[r];
    return 0;
}

template <int LOC, int HUC, bool TRID, bool TRANS>
__global__ void __launch_bounds__(kBandThreads) band_lu_kernel(const BandArgs g)
{
    const int64_t s = (int64_t)blockIdx.x * kBandThreads + threadIdx.x;
    if (s >= g.count) return;
    double* a = g.ab + s * g.sab;
    int64_t* P = g.P + s * g.sp;
    if (!TRANS && LOC <= 2 && g.factor && g.solve && g.nrhs == 1 && g.lo > 0) {
        // factor and solve of one right-hand side: the P L solve inside the
        // factorisation's loop, then the upper solve (not for the widest
        // register class, whose window already takes most registers)
        double* B = g.B + s * g.sb;
        int64_t lnz = -1;
        band_factor<LOC, HUC, TRID, true>(a, g.ldab, P, g.n, g.lo, g.hi, g.hu, B, &lnz);
        g.status[s] = band_upper_solve<HUC, TRID>(a, g.ldab, g.n, g.hu, B, lnz + 1);
        return;
    }
    if (g.factor) band_factor<LOC, HUC, TRID>(a, g.ldab, P, g.n, g.lo, g.hi, g.hu);
    if (!g.solve) return;
    int st = 0;
    if (g.nrhs > 0) {
        double* B = g.B + s * g.sb;
        if (g.n == 1 && g.nrhs > 1 && g.ldb == 1) {
            // a 1 x nrhs B with ldb == 1 is row-major to TMV: ColUpperTriLDivEq
            // (src/TMV_BandTriDiv_M.cpp:87-125) checks U(0,0) and scales the
            // row by its reciprocal
            const double d = a[0];
            if (d == 0.0) {
                st = 1;
            } else {
                const double inv = 1.0 / d;
                for (int q = 0; q < g.nrhs; ++q) B[q] = scale_by(B[q], inv);
            }
        } else if (TRANS) {
            for (int q = 0; q < g.nrhs && st == 0; ++q)
                st = band_rsolve_one<LOC, HUC, TRID>(a, g.ldab, P, g.n, g.lo, g.hu, B + q * g.ldb);
        } else {
            for (int q = 0; q < g.nrhs && st == 0; ++q)
                st = band_solve_one<LOC, HUC, TRID>(a, g.ldab, P, g.n, g.lo, g.hu, B + q * g.ldb);
        }
    }
    g.status[s] = st;
}

// The same algorithm for bands wider than the register kernels hold: the
// window stays in the band storage itself (the thread's own slots, cached in
// L1/L2), each step a direct transcription of the loops of
// NonLapBandLU_Decompose and of the solves above (the general algorithm
// only: the tridiagonal one always fits the register kernel).
__global__ void __launch_bounds__(kBandThreads) band_lu_wide_kernel(const BandArgs g)
{
    const int64_t s = (int64_t)blockIdx.x * kBandThreads + threadIdx.x;
    if (s >= g.count) return;
    double* a = g.ab + s * g.sab;
    int64_t* P = g.P + s * g.sp;
    const int64_t n = g.n, ld = g.ldab;
    const int lo = g.lo, hi = g.hi, hu = g.hu;
    if (g.factor) {
        for (int64_t j = 0; j < n; ++j)
            for (int d = hi + 1; d <= hu; ++d)
                if (j - d >= 0) a[(j - d) + j * ld] = 0.0;
        if (lo == 0) {
            for (int64_t i = 0; i < n; ++i) P[i] = i;
        } else {
            int64_t endcol = lmin(lo + 1, n), endrow = lmin(hu + 1, n);
            for (int64_t j = 0; j + 1 < n; ++j) {
                int64_t ip = 0;
                double piv = fabs(a[j + j * ld]);
                for (int64_t i = 1; i < endcol - j; ++i) {
                    const double v = fabs(a[(j + i) + j * ld]);
                    if (v > piv) {
                        piv = v;
                        ip = i;
                    }
                }
                if (piv < DBL_MIN) {
                    ip = 0;
                    for (int64_t i = j; i < endcol; ++i) a[i + j * ld] = 0.0;
                }
                if (ip != 0) {
                    ip += j;
                    for (int64_t c = j; c < endrow; ++c) {
                        const double t = a[ip + c * ld];
                        a[ip + c * ld] = a[j + c * ld];
                        a[j + c * ld] = t;
                    }
                }
                P[j] = ip != 0 ? ip : j;
                const double ujj = a[j + j * ld];
                if (ujj != 0.0) {
                    const double inv = 1.0 / ujj;
                    for (int64_t i = j + 1; i < endcol; ++i) a[i + j * ld] = scale_by(a[i + j * ld], inv);
                }
                for (int64_t c = j + 1; c < endrow; ++c) {
                    const double u = a[j + c * ld];
                    if (u == 0.0) continue;
                    for (int64_t i = j + 1; i < endcol; ++i)
                        a[i + c * ld] = msub(a[i + c * ld], a[i + j * ld], u);
                }
                if (endcol < n) ++endcol;
                if (endrow < n) ++endrow;
            }
            P[n - 1] = n - 1;
        }
    }
    if (!g.solve) return;
    int st = 0;
    const bool row_b = n == 1 && g.nrhs > 1 && g.ldb == 1;
    double* B = g.nrhs > 0 ? g.B + s * g.sb : nullptr;
    if (row_b) {
        const double d = a[0];
        if (d == 0.0) {
            st = 1;
        } else {
            const double inv = 1.0 / d;
            for (int q = 0; q < g.nrhs; ++q) B[q] = scale_by(B[q], inv);
        }
    }
    for (int q = 0; q < g.nrhs && st == 0 && !row_b && g.trans; ++q) {
        double* b = B + q * g.ldb;
        if (hu == 0) {
            st = band_diag_solve(a, ld, n, b);
        } else {
            int64_t i1 = 0;
            while (i1 < n && b[i1] == 0.0) ++i1;
            for (int64_t i = i1; i < n; ++i) {
                double v = b[i];
                for (int64_t j = lmax(i1, i - hu); j < i; ++j) v = msub(v, b[j], a[j + i * ld]);
                const double d = a[i + i * ld];
                if (d == 0.0) {
                    st = 1;
                    break;
                }
                b[i] = v / d;
            }
        }
        if (st || lo == 0) continue;
        for (int64_t j = n - 2; j >= 0; --j) {
            const int64_t len = lmin(lo, n - 1 - j);
            double t = 0.0;
            for (int64_t k = 1; k <= len; ++k) t = __dadd_rn(t, __dmul_rn(a[(j + k) + j * ld], b[j + k]));
            b[j] = __dsub_rn(b[j], t);
            const int64_t pj = P[j];
            if (pj < j || pj > j + lo || pj >= n) {
                st = 2;
                break;
            }
            if (pj != j) {
                const double w = b[j];
                b[j] = b[pj];
                b[pj] = w;
            }
        }
    }
    for (int q = 0; q < g.nrhs && st == 0 && !row_b && !g.trans; ++q) {
        double* b = B + q * g.ldb;
        if (lo > 0) {
            int64_t jn = lmin(lo + 1, n);
            for (int64_t j = 0; j + 1 < n && st == 0; ++j) {
                const int64_t pj = P[j];
                if (pj < j || pj > j + lo || pj >= n) {
                    st = 2;
                    break;
                }
                if (pj != j) {
                    const double t = b[j];
                    b[j] = b[pj];
                    b[pj] = t;
                }
                const double bj = b[j];
                if (bj != 0.0)
                    for (int64_t i = j + 1; i < jn; ++i) b[i] = msub(b[i], a[i + j * ld], bj);
                if (jn < n) ++jn;
            }
        }
        if (st) break;
        int64_t i2 = n;
        while (i2 > 0 && b[i2 - 1] == 0.0) --i2;
        if (i2 == 0) continue;
        if (hu == 0) {
            for (int64_t i = 0; i < i2 && st == 0; ++i) {
                const double d = a[i + i * ld];
                if (d == 0.0) st = 1;
                else b[i] = b[i] / d;
            }
            continue;
        }
        for (int64_t j = i2 - 1; j >= 0; --j) {
            if (b[j] == 0.0) continue;
            const double d = a[j + j * ld];
            if (d == 0.0) {
                st = 1;
                break;
            }
            const double bj = b[j] / d;
            b[j] = bj;
            for (int64_t i = lmax(0, j - hu); i < j; ++i) b[i] = msub(b[i], bj, a[i + j * ld]);
        }
    }
    g.status[s] = st;
}

// BandLUDiv's copy of A into its factor storage (src/TMV_BandLUD.cpp:60-93,
// 133-137): lo' = min(lo, hi) subdiagonals, hu = min(lo+hi, n-1)
// superdiagonals, A itself or, when hi < lo, its transpose; the slots outside
// A's band are zero.  One thread per column of one system.
__global__ void __launch_bounds__(kBandThreads)
band_copy_kernel(int64_t count, int64_t n, int lo, int hi, int lo2, int hu, bool trans,
                 const double* __restrict__ ab, int64_t ldab, int64_t sab, double* __restrict__ lu,
                 int64_t ldlu, int64_t slu)
{
    const int64_t t = (int64_t)blockIdx.x * kBandThreads + threadIdx.x;
    if (t >= count * n) return;
    const int64_t s = t / n, j = t % n;
    const double* a = ab + s * sab;
    double* o = lu + s * slu;
    for (int64_t i = lmax(0, j - hu); i <= lmin(n - 1, j + lo2); ++i) {
        const int64_t r = trans ? j : i, c = trans ? i : j;  // the entry of A
        o[i + j * ldlu] = (r >= c - hi && r <= c + lo) ? a[r + c * ldab] : 0.0;
    }
}

// The register kernel's window capacity for (lo, hu), or -1 for the wide kernel.
int band_class(int lo, int hu, int algo)
{
    if (algo == TMVG_BAND_TRIDIAG) return 0;
    if (lo <= 1 && hu <= 2) return 1;
    if (lo <= 2 && hu <= 4) return 2;
    if (lo <= 4 && hu <= 8) return 3;
    return -1;
}

tmvg_status band_run(Context* c, int64_t count, int64_t n, int64_t lo, int64_t hi, int algo, double* AB,
                     int64_t ldab, int64_t sab, int64_t* P, int64_t sp, int64_t nrhs, double* B, int64_t ldb,
                     int64_t sb, int32_t* status, bool factor, bool solve, const char* what,
                     bool trans = false)
{
    std::string w(what);
    if (count < 0 || n < 0 || lo < 0 || hi < 0 || nrhs < 0) return set_error(c, TMVG_BAD_ARG, w + ": negative size");
    if (algo != TMVG_BAND_GENERAL && algo != TMVG_BAND_TRIDIAG)
        return set_error(c, TMVG_BAD_ARG, w + ": unknown algorithm");
    if (count == 0 || n == 0) return TMVG_OK;
    if (lo > n - 1 || hi > n - 1) return set_error(c, TMVG_BAD_ARG, w + ": lo and hi must be < n");
    if (algo == TMVG_BAND_TRIDIAG && (lo != 1 || hi != 1))
        return set_error(c, TMVG_BAD_ARG, w + ": the tridiagonal algorithm needs lo == hi == 1");
    if (lo > 1 << 20 || hi > 1 << 20) return set_error(c, TMVG_BAD_ARG, w + ": band too wide");
    const int64_t hu = std::min(lo + hi, n - 1);
    if (ldab < lo + hu || ldab < 1) return set_error(c, TMVG_BAD_ARG, w + ": ldab < lo + min(lo+hi, n-1)");
    const int64_t len = (n - 1) * (ldab + 1) + 1;
    if (count > 1 && sab < len) return set_error(c, TMVG_BAD_ARG, w + ": band systems overlap (stride_ab)");
    if (count > 1 && sp < n) return set_error(c, TMVG_BAD_ARG, w + ": stride_p < n");
    if (!AB || !P) return set_error(c, TMVG_BAD_ARG, w + ": null band or pivot pointer");
    if (solve) {
        if (nrhs > (1 << 30)) return set_error(c, TMVG_BAD_ARG, w + ": too many right-hand sides");
        if (!status) return set_error(c, TMVG_BAD_ARG, w + ": null status pointer");
        if (nrhs > 0) {
            if (!B) return set_error(c, TMVG_BAD_ARG, w + ": null right-hand side pointer");
            if (ldb < n) return set_error(c, TMVG_BAD_ARG, w + ": ldb < n");
            if (count > 1 && sb < ldb * (nrhs - 1) + n)
                return set_error(c, TMVG_BAD_ARG, w + ": right-hand sides overlap (stride_b)");
        }
    }
    BandArgs g;
    g.ab = AB;
    g.sab = sab;
    g.ldab = ldab;
    g.P = P;
    g.sp = sp;
    g.B = B;
    g.ldb = ldb;
    g.sb = sb;
    g.status = status;
    g.count = count;
    g.n = n;
    g.lo = (int)lo;
    g.hi = (int)hi;
    g.hu = (int)hu;
    g.nrhs = solve ? (int)nrhs : 0;
    g.factor = factor;
    g.solve = solve;
    g.trans = trans;
    const int64_t blocks = (count + kBandThreads - 1) / kBandThreads;
    if (blocks > INT32_MAX) return set_error(c, TMVG_BAD_ARG, w + ": too many systems");
    const dim3 grid((unsigned)blocks);
    // the row solve (LU_RDivEq) has kernels of its own, so that the factor
    // and column-solve kernels keep their register budget
    const int cls = band_class((int)lo, (int)hu, algo);
    switch (cls < 0 ? -1 : cls + (trans ? 4 : 0)) {
        case 0: band_lu_kernel<1, 2, true, false><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 1: band_lu_kernel<1, 2, false, false><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 2: band_lu_kernel<2, 4, false, false><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 3: band_lu_kernel<4, 8, false, false><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 4: band_lu_kernel<1, 2, true, true><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 5: band_lu_kernel<1, 2, false, true><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 6: band_lu_kernel<2, 4, false, true><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        case 7: band_lu_kernel<4, 8, false, true><<<grid, kBandThreads, 0, c->stream>>>(g); break;
        default: band_lu_wide_kernel<<<grid, kBandThreads, 0, c->stream>>>(g); break;
    }
    c->launches += 1;
    return check_cuda(c, cudaGetLastError(), what);
}

}  // namespace

}  // namespace tmvg

using namespace tmvg;

extern "C" {

tmvg_status tmvg_band_lu_decompose_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo,
                                               int64_t hi, int algo, double* AB, int64_t ldab,
                                               int64_t stride_ab, int64_t* P, int64_t stride_p)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_BAD_ARG;
    c->last_error.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, TMVG_CUDA_ERROR, "cudaSetDevice failed");
    return band_run(c, count, n, lo, hi, algo, AB, ldab, stride_ab, P, stride_p, 0, nullptr, 1, 0, nullptr, true,
                    false, "band_lu_decompose");
}

tmvg_status tmvg_band_lu_ldiveq_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo, int64_t hi,
                                            int algo, const double* AB, int64_t ldab, int64_t stride_ab,
                                            const int64_t* P, int64_t stride_p, int64_t nrhs, double* B,
                                            int64_t ldb, int64_t stride_b, int32_t* status)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_BAD_ARG;
    c->last_error.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, TMVG_CUDA_ERROR, "cudaSetDevice failed");
    return band_run(c, count, n, lo, hi, algo, const_cast<double*>(AB), ldab, stride_ab, const_cast<int64_t*>(P),
                    stride_p, nrhs, B, ldb, stride_b, status, false, true, "band_lu_ldiveq");
}

tmvg_status tmvg_band_lu_rdiveq_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo, int64_t hi,
                                            int algo, const double* AB, int64_t ldab, int64_t stride_ab,
                                            const int64_t* P, int64_t stride_p, int64_t nrhs, double* B,
                                            int64_t ldb, int64_t stride_b, int32_t* status)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_BAD_ARG;
    c->last_error.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, TMVG_CUDA_ERROR, "cudaSetDevice failed");
    return band_run(c, count, n, lo, hi, algo, const_cast<double*>(AB), ldab, stride_ab, const_cast<int64_t*>(P),
                    stride_p, nrhs, B, ldb, stride_b, status, false, true, "band_lu_rdiveq", true);
}

tmvg_status tmvg_band_divide_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo, int64_t hi,
                                         const double* AB, int64_t ldab, int64_t stride_ab, double* LU,
                                         int64_t ldlu, int64_t stride_lu, int64_t* P, int64_t stride_p,
                                         int64_t nrhs, double* B, int64_t ldb, int64_t stride_b,
                                         int32_t* status)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_BAD_ARG;
    c->last_error.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, TMVG_CUDA_ERROR, "cudaSetDevice failed");
    if (count < 0 || n < 0 || lo < 0 || hi < 0 || nrhs < 0)
        return set_error(c, TMVG_BAD_ARG, "band_divide: negative size");
    if (count == 0 || n == 0) return TMVG_OK;
    if (lo > n - 1 || hi > n - 1) return set_error(c, TMVG_BAD_ARG, "band_divide: lo and hi must be < n");
    if (!AB || !LU) return set_error(c, TMVG_BAD_ARG, "band_divide: null band pointer");
    if (ldab < std::max<int64_t>(lo + hi, 1)) return set_error(c, TMVG_BAD_ARG, "band_divide: ldab < lo + hi");
    if (count > 1 && stride_ab < (n - 1) * (ldab + 1) + 1)
        return set_error(c, TMVG_BAD_ARG, "band_divide: band systems overlap (stride_ab)");
    // BandLUDiv: the tridiagonal algorithm for lo == hi == 1; the transpose
    // factored when hi < lo (src/TMV_BandLUD.cpp:60-93)
    const bool trans = hi < lo;
    const int algo = (lo == 1 && hi == 1) ? TMVG_BAND_TRIDIAG : TMVG_BAND_GENERAL;
    const int64_t lo2 = trans ? hi : lo, hi2 = trans ? lo : hi;
    const int64_t hu = std::min(lo + hi, n - 1);
    if (ldlu < std::max<int64_t>(lo2 + hu, 1)) return set_error(c, TMVG_BAD_ARG, "band_divide: ldlu < min(lo,hi) + hu");
    if (count > 1 && stride_lu < (n - 1) * (ldlu + 1) + 1)
        return set_error(c, TMVG_BAD_ARG, "band_divide: factor systems overlap (stride_lu)");
    const int64_t threads = count * n;
    const int64_t blocks = (threads + kBandThreads - 1) / kBandThreads;
    if (blocks > INT32_MAX) return set_error(c, TMVG_BAD_ARG, "band_divide: too many systems");
    band_copy_kernel<<<(unsigned)blocks, kBandThreads, 0, c->stream>>>(count, n, (int)lo, (int)hi, (int)lo2,
                                                                     (int)hu, trans, AB, ldab, stride_ab, LU,
                                                                     ldlu, stride_lu);
    c->launches += 1;
    tmvg_status st = check_cuda(c, cudaGetLastError(), "band_divide: copy");
    if (st) return st;
    return band_run(c, count, n, lo2, hi2, algo, LU, ldlu, stride_lu, P, stride_p, nrhs, B, ldb, stride_b, status,
                    true, true, "band_divide", trans);
}

tmvg_status tmvg_band_lu_solve_batched_f64(tmvg_handle h, int64_t count, int64_t n, int64_t lo, int64_t hi,
                                           int algo, double* AB, int64_t ldab, int64_t stride_ab, int64_t* P,
                                           int64_t stride_p, int64_t nrhs, double* B, int64_t ldb,
                                           int64_t stride_b, int32_t* status)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_BAD_ARG;
    c->last_error.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, TMVG_CUDA_ERROR, "cudaSetDevice failed");
    return band_run(c, count, n, lo, hi, algo, AB, ldab, stride_ab, P, stride_p, nrhs, B, ldb, stride_b, status,
                    true, true, "band_lu_solve");
}

}  // extern "C"
