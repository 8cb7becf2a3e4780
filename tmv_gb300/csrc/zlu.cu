// zlu.cu -- LU_Decompose and LU_LDivEq for std::complex<double> on sm_103a.
//
// TMV's complex instantiations (src/TMV_LUDecompose.cpp:514, src/TMV_LUDiv.cpp:186
// with T = std::complex<double>) with TMV's complex arithmetic:
//   - pivot: the first index of the strict maximum of TMV_ABS, TMV's
//     overflow-guarded modulus (include/tmv/TMV_Base.h:312-325; the scan of
//     src/TMV_Vector.cpp:474-503: a NaN modulus is chosen only as the first
//     entry); a maximum below DBL_MIN zeroes the column with P[j] = j;
//   - a column is scaled by TMV_InverseOf of the pivot, TMV's guarded
//     reciprocal (include/tmv/TMV_Base.h:722-742);
//   - the solves divide by U(j,j) as TMV_Divide = b * TMV_InverseOf(d) and
//     skip zero entries, as TMV's column-oriented vector solves do
//     (src/TMV_TriDiv_V.cpp:148-236, 322-398), one right-hand side at a time.
// The scaling and the solves' complex products are (ac - bd, ad + bc) with
// separately rounded products (no fused multiply-add), as the host computes
// them; the blocked trailing products and solves' off-diagonal products use
// fused multiply-adds (values to rounding).
//
// Small matrices (n < 128) factor one column per step (pivot search in one
// CTA, row interchange, scaling, rank-1 update over the grid) and solve one
// CTA per right-hand side; larger ones factor by panels with look-ahead
// (zlu_factor_blocked) and solve by 64-row blocks (zlu_ldiveq_blocked).  The
// right solve (LU_RDivEq) runs one row per CTA substituted in TMV's order.
// Values agree with TMV's recursive factorisation to rounding; pivots are
// TMV's wherever rounding does not decide a tie.
#include "zlu.cuh"
#include "trsv.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <climits>

namespace tmvg {

constexpr int kZPivThreads = 1024;
constexpr int kZThreads = 256;
constexpr int kZTile = 16;  // rank-1 update: 16 x 16 threads per CTA

__device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

__device__ __forceinline__ double2 zsub(double2 a, double2 b)
{
    return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}

__device__ __forceinline__ bool znonzero(double2 a) { return a.x != 0.0 || a.y != 0.0; }

// TMV_ABS(std::complex<T>)
__device__ __forceinline__ double tmv_abs(double2 x)
{
    double xr = x.x, xi = x.y;
    const double ar = fabs(xr), ai = fabs(xi);
    const double s = ar < ai ? ai : ar;
    if (s == 0.0) return s;
    xr = __ddiv_rn(xr, s);
    xi = __ddiv_rn(xi, s);
    return __dmul_rn(s, __dsqrt_rn(__dadd_rn(__dmul_rn(xr, xr), __dmul_rn(xi, xi))));
}

// TMV_InverseOf(std::complex<T>)
__device__ __forceinline__ double2 tmv_inverse_of(double2 x)
{
    double xr = x.x, xi = x.y;
    if (fabs(xr) > fabs(xi)) {
        xi = __ddiv_rn(xi, xr);
        const double denom = __dmul_rn(xr, __dadd_rn(1.0, __dmul_rn(xi, xi)));
        return make_double2(__ddiv_rn(1.0, denom), __ddiv_rn(-xi, denom));
    } else if (fabs(xi) > 0.0) {
        xr = __ddiv_rn(xr, xi);
        const double denom = __dmul_rn(xi, __dadd_rn(1.0, __dmul_rn(xr, xr)));
        return make_double2(__ddiv_rn(xr, denom), __ddiv_rn(-1.0, denom));
    }
    return make_double2(__ddiv_rn(1.0, xi), 0.0);
}

// Pivot of column k over rows [k, n): keys order as TMV's scan does (a NaN
// modulus counts as +inf in row k and loses elsewhere; ties keep the lowest
// row).  Writes P[k] and flag[0] = 1 when the column underflows (zeroed).
__global__ void __launch_bounds__(kZPivThreads)
zlu_pivot_kernel(int64_t n, double2* A, int64_t lda, int64_t k, int64_t* P, int* flag)
{
    __shared__ double s_key[kZPivThreads / 32];
    __shared__ int64_t s_idx[kZPivThreads / 32];
    __shared__ double s_piv;
    __shared__ int64_t s_row;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double bk = -1.0;
    int64_t bi = INT64_MAX;
    for (int64_t i = k + tid; i < n; i += kZPivThreads) {
        double a = tmv_abs(A[i + k * lda]);
        if (a != a) a = i == k ? INFINITY : -1.0;
        if (a > bk) { bk = a; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ok = __shfl_xor_sync(0xffffffffu, bk, o);
        const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ok > bk || (ok == bk && oi < bi)) { bk = ok; bi = oi; }
    }
    if (lane == 0) { s_key[warp] = bk; s_idx[warp] = bi; }
    __syncthreads();
    if (warp == 0) {
        bk = lane < kZPivThreads / 32 ? s_key[lane] : -1.0;
        bi = lane < kZPivThreads / 32 ? s_idx[lane] : INT64_MAX;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ok = __shfl_xor_sync(0xffffffffu, bk, o);
            const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ok > bk || (ok == bk && oi < bi)) { bk = ok; bi = oi; }
        }
        if (lane == 0) {
            // the pivot's own modulus (a NaN in row k stays NaN: no underflow)
            const double piv = bi == k ? tmv_abs(A[k + k * lda]) : bk;
            s_piv = piv;
            s_row = bi;
        }
    }
    __syncthreads();
    const bool under = fabs(s_piv) < DBL_MIN;
    if (under) {
        for (int64_t i = k + tid; i < n; i += kZPivThreads) A[i + k * lda] = make_double2(0.0, 0.0);
    }
    if (tid == 0) {
        P[k] = under ? k : s_row;
        flag[0] = under ? 1 : 0;
    }
}

// Rows k and P[k] interchanged over all columns.
__global__ void zlu_swap_kernel(int64_t n, double2* A, int64_t lda, int64_t k, const int64_t* P)
{
    const int64_t p = P[k];
    if (p == k) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double2 t = A[k + j * lda];
        A[k + j * lda] = A[p + j * lda];
        A[p + j * lda] = t;
    }
}

// L(k+1:n, k) *= TMV_InverseOf(A(k, k)) unless the column underflowed.
__global__ void zlu_scale_kernel(int64_t n, double2* A, int64_t lda, int64_t k, const int* flag)
{
    if (flag[0]) return;
    const double2 inv = tmv_inverse_of(A[k + k * lda]);
    for (int64_t i = k + 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        A[i + k * lda] = zmul(A[i + k * lda], inv);
}

// A(i, j) -= L(i, k) U(k, j) for i, j > k.
__global__ void __launch_bounds__(kZTile * kZTile)
zlu_update_kernel(int64_t n, double2* A, int64_t lda, int64_t k)
{
    const int64_t i = k + 1 + blockIdx.x * (int64_t)kZTile + threadIdx.x;
    const int64_t j = k + 1 + blockIdx.y * (int64_t)kZTile + threadIdx.y;
    if (i >= n || j >= n) return;
    A[i + j * lda] = zsub(A[i + j * lda], zmul(A[i + k * lda], A[k + j * lda]));
}

// ---------------------------------------------------------------------------
// Blocked factorisation (n >= kZBlockedMin): right-looking over panels of KB
// columns (32, or 16 where a 32-wide panel's rows exceed shared memory).
// Each panel is factored by one 16-CTA cluster with the rows dealt
// cyclically to the CTAs and held in their shared memory; the column steps
// are the column path's (pivot, interchange within the panel, scaling by
// TMV_InverseOf, rank-1 update of the panel's later columns).  The panel's
// interchanges are then applied to the other columns, U12 = L11^-1 A12 is
// solved, and A22 -= L21 U12 runs as a register-tiled complex DFMA product.
// Column values differ from the unblocked updates only by rounding, so the
// pivots are the column path's (TMV's) wherever rounding does not decide a
// tie.
//
// Pivot search in two stages, so that TMV_ABS (two divisions and a square
// root) is evaluated only where it can decide: a proxy key per row, the bits
// of |z|^2 computed after scaling z by a power of two (two FP64 operations,
// relative error below 2^-51), selects the rows within 256 ulps of |z|^2 of
// the CTA's largest key; those get TMV_ABS and the largest TMV_ABS (lowest
// row on ties) is the CTA's candidate.  TMV_ABS differs from |z| by at most a few
// ulps, so no row outside the margin can hold the maximum.  Infinite and NaN
// entries follow TMV_ABS (NaN): chosen only as the column's first entry.
// ---------------------------------------------------------------------------
constexpr int kZPanelCtas = 16;
constexpr int kZPanelThreads = 512;
constexpr int64_t kZBlockedMin = 128;
constexpr size_t kZPanelSmemMax = 200 * 1024;
constexpr long long kZKeyNaNFirst = 0x7fffffffffffffffLL;  // NaN/inf as row j
constexpr long long kZKeyNaN = -0x7fffffffffffffffLL;      // NaN/inf elsewhere
constexpr long long kZKeyZero = -(1LL << 62);
constexpr long long kZAbsBits = 0x7fffffffffffffffLL;
constexpr long long kZInfBits = 0x7ff0000000000000LL;

// Proxy key of z: increasing in |z| up to its rounding.  Comparisons and
// scaling run on the integer pipe (a double comparison occupies the FP64
// pipe, which GB300 issues at 2 per SM per clock); |z|^2 itself takes one
// DMUL and one DFMA.
__device__ __forceinline__ long long zproxy_key(double2 z, bool first)
{
    const long long ur = __double_as_longlong(z.x) & kZAbsBits;
    const long long ui = __double_as_longlong(z.y) & kZAbsBits;
    const long long us = ur > ui ? ur : ui;
    if (us >= kZInfBits) return first ? kZKeyNaNFirst : kZKeyNaN;  // inf or NaN
    if (us == 0) return kZKeyZero;
    const int eb = (int)(us >> 52);  // biased exponent of the larger part
    double r, t;
    int e2;  // |z|^2 = K 4^e2
    if (eb == 0) {  // subnormal: scale by 2^600 first (exact)
        const double ar = fabs(z.x) * 0x1p600, ai = fabs(z.y) * 0x1p600;
        const long long vs = __double_as_longlong(fmax(ar, ai));
        const int e = (int)(vs >> 52) - 1023;
        const double sc = __longlong_as_double((long long)(1023 - e) << 52);
        r = ar * sc;
        t = ai * sc;
        e2 = e - 600;
    } else {
        // both parts scaled by 2^-(eb-1023) through their exponent fields; a
        // smaller part pushed below the normal range counts as zero (its
        // square is below 2^-1000 of K's); a subnormal smaller part is scaled
        // by a multiplication (exact)
        const long long shift = (long long)(eb - 1023) << 52;
        const long long ul = ur > ui ? ui : ur;
        const double big = __longlong_as_double(us - shift);
        const int lb = (int)(ul >> 52);
        double small;
        if (lb == 0)
            small = ul == 0 ? 0.0 : __longlong_as_double(ul) * __longlong_as_double((long long)(2046 - eb) << 52);
        else
            small = lb - (eb - 1023) >= 1 ? __longlong_as_double(ul - shift) : 0.0;
        r = big;
        t = small;
        e2 = eb - 1023;
    }
    const double K = fma(r, r, t * t);  // in [1, 8)
    // exponent 2 e2 in [-2148, 2046] above K's bits less 1.0's (K's binade
    // offset 0..2 and mantissa), the mantissa's last two bits dropped so that
    // the sum fits 64 bits; one key unit is 4 ulps of K
    const long long kb = (__double_as_longlong(K) - __double_as_longlong(1.0)) >> 2;
    return ((long long)(2 * e2) << 50) + kb;
}

// TMV_ABS as an ordered integer key: its bits (non-negative), a NaN as the
// column's first entry above everything, elsewhere below everything.
__device__ __forceinline__ long long zabs_key(double raw, bool first)
{
    const long long b = __double_as_longlong(raw);
    if ((b & kZAbsBits) > kZInfBits) return first ? kZKeyNaNFirst : -1;
    return b;
}

template <int KB>
struct ZPanelShared {
    long long cand_key[2];     // this CTA's candidate: zabs_key (-2: none)
    double cand_abs[2];        // its TMV_ABS (NaN kept)
    long long cand_row[2];     // its global row (LLONG_MAX: none)
    double2 cand_inv[2];       // TMV_InverseOf of its entry
    double2 cand_rowv[2][KB];  // its row's panel entries
    double2 diag_rowv[2][KB];  // row j's panel entries (the CTA owning row j)
    double2 prow[KB];          // the pivot row after the interchange: U's row j
    double2 inv;
    int under;
    long long wkey[kZPanelThreads / 32];
    int wrow[kZPanelThreads / 32];
};

template <int KB>
__global__ void __launch_bounds__(kZPanelThreads)
zlu_panel_smem_kernel(int64_t n, double2* __restrict__ A, int64_t lda, int64_t k, int kb, int64_t* __restrict__ P,
                      int rpc)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ double2 s_rows[];  // rpc rows, stride KB + 1
    __shared__ ZPanelShared<KB> sh;
    constexpr int RS = KB + 1;
    const int cta = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // local row r is global row k + cta + 16 r
    for (int t = tid; t < rpc * kb; t += kZPanelThreads) {
        const int r = t % rpc, c = t / rpc;
        const int64_t i = k + cta + (int64_t)kZPanelCtas * r;
        s_rows[r * RS + c] = i < n ? A[i + (k + c) * lda] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int jj = 0; jj < kb; ++jj) {
        const int par = jj & 1;
        const int64_t j = k + jj;
        // rows of this CTA at or below j: r >= r0
        const int64_t d0 = j - k - cta;
        const int r0 = d0 <= 0 ? 0 : (int)((d0 + kZPanelCtas - 1) / kZPanelCtas);
        const int lj = (d0 >= 0 && d0 % kZPanelCtas == 0) ? (int)(d0 / kZPanelCtas) : -1;
        // stage 1: largest proxy key (the first row's key kept for stage 2)
        long long bk = LLONG_MIN, key0 = LLONG_MIN;
        for (int r = r0 + tid; r < rpc; r += kZPanelThreads) {
            const int64_t i = k + cta + (int64_t)kZPanelCtas * r;
            if (i >= n) break;
            const long long key = zproxy_key(s_rows[r * RS + jj], i == j);
            if (r == r0 + tid) key0 = key;
            bk = key > bk ? key : bk;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
            bk = ok > bk ? ok : bk;
        }
        if (lane == 0) sh.wkey[warp] = bk;
        __syncthreads();
        long long mk = sh.wkey[0];
#pragma unroll
        for (int w = 1; w < kZPanelThreads / 32; ++w) mk = sh.wkey[w] > mk ? sh.wkey[w] : mk;
        // stage 2: TMV_ABS (and TMV_InverseOf) of the rows within 64 key units
        // (256 ulps of |z|^2) of the largest
        const long long thr = mk <= LLONG_MIN + 64 ? LLONG_MIN + 1 : mk - 64;
        long long ba = -2;
        int br = INT_MAX;
        double braw = 0.0;
        double2 binv = make_double2(0.0, 0.0);
        for (int r = r0 + tid; r < rpc && mk != LLONG_MIN; r += kZPanelThreads) {
            const int64_t i = k + cta + (int64_t)kZPanelCtas * r;
            if (i >= n) break;
            const double2 z = s_rows[r * RS + jj];
            const long long key = r == r0 + tid ? key0 : zproxy_key(z, i == j);
            if (key < thr) continue;
            const double raw = tmv_abs(z);
            const long long a = zabs_key(raw, i == j);
            if (a > ba || (a == ba && r < br)) {
                ba = a;
                br = r;
                braw = raw;
                binv = tmv_inverse_of(z);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long oa = __shfl_xor_sync(0xffffffffu, ba, o);
            const int orow = __shfl_xor_sync(0xffffffffu, br, o);
            if (oa > ba || (oa == ba && orow < br)) { ba = oa; br = orow; }
        }
        if (lane == 0) { sh.wkey[warp] = ba; sh.wrow[warp] = br; }
        __syncthreads();
        ba = sh.wkey[0];
        br = sh.wrow[0];
#pragma unroll
        for (int w = 1; w < kZPanelThreads / 32; ++w)
            if (sh.wkey[w] > ba || (sh.wkey[w] == ba && sh.wrow[w] < br)) { ba = sh.wkey[w]; br = sh.wrow[w]; }
        // stage the candidate (its owner thread writes its TMV_ABS and
        // inverse) and, where owned, row j
        if (tid < kb) {
            if (br != INT_MAX) sh.cand_rowv[par][tid] = s_rows[br * RS + tid];
            if (lj >= 0) sh.diag_rowv[par][tid] = s_rows[lj * RS + tid];
        }
        if (br != INT_MAX && (br - r0) % kZPanelThreads == tid && br >= r0) {
            sh.cand_abs[par] = braw;
            sh.cand_inv[par] = binv;
        }
        if (tid == 0) {
            sh.cand_key[par] = ba;
            sh.cand_row[par] = br == INT_MAX ? LLONG_MAX : k + cta + (long long)kZPanelCtas * br;
        }
        cluster.sync();
        // the winner over the cluster: lanes 0..15 of every warp read one CTA each
        long long wa = -3, wr = LLONG_MAX;
        int wc = 0;
        if (lane < kZPanelCtas) {
            ZPanelShared<KB>* o = cluster.map_shared_rank(&sh, lane);
            wa = o->cand_key[par];
            wr = o->cand_row[par];
            wc = lane;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long oa = __shfl_xor_sync(0xffffffffu, wa, o);
            const long long orow = __shfl_xor_sync(0xffffffffu, wr, o);
            const int oc = __shfl_xor_sync(0xffffffffu, wc, o);
            if (oa > wa || (oa == wa && orow < wr)) { wa = oa; wr = orow; wc = oc; }
        }
        const int owner_j = (int)((j - k) % kZPanelCtas);
        // U's row j: the pivot row (or row j with its column zeroed)
        if (tid < kb) {
            ZPanelShared<KB>* w = cluster.map_shared_rank(&sh, wc);
            // the pivot's own modulus (a NaN stays NaN: no underflow)
            const long long rb = __double_as_longlong(w->cand_abs[par]) & kZAbsBits;
            const bool under = rb < __double_as_longlong(DBL_MIN);
            const int64_t p = under ? j : (int64_t)wr;
            double2 v;
            if (under) {
                v = cluster.map_shared_rank(&sh.diag_rowv[par][0], owner_j)[tid];
                if (tid == jj) v = make_double2(0.0, 0.0);
            } else {
                v = w->cand_rowv[par][tid];
            }
            sh.prow[tid] = v;
            if (lj >= 0) s_rows[lj * RS + tid] = v;
            if (p != j && (int)((p - k) % kZPanelCtas) == cta)
                s_rows[(int)((p - k) / kZPanelCtas) * RS + tid] =
                    cluster.map_shared_rank(&sh.diag_rowv[par][0], owner_j)[tid];
            if (tid == 0) {
                sh.under = under ? 1 : 0;
                sh.inv = under ? make_double2(0.0, 0.0) : w->cand_inv[par];
                if (cta == 0) P[j] = p;
            }
        }
        __syncthreads();
        // scale and update this CTA's rows below j
        const double2 inv = sh.inv;
        const bool und = sh.under != 0;
        for (int r = r0 + tid; r < rpc; r += kZPanelThreads) {
            const int64_t i = k + cta + (int64_t)kZPanelCtas * r;
            if (i >= n) break;
            if (i == j) continue;
            double2* row = &s_rows[r * RS];
            const double2 l = und ? make_double2(0.0, 0.0) : zmul(row[jj], inv);
            row[jj] = l;
            for (int c = jj + 1; c < kb; ++c) {
                const double2 u = sh.prow[c];
                double2 a = row[c];
                a.x = fma(-l.x, u.x, a.x);
                a.x = fma(l.y, u.y, a.x);
                a.y = fma(-l.x, u.y, a.y);
                a.y = fma(-l.y, u.x, a.y);
                row[c] = a;
            }
        }
        // (the next column reads only this thread's rows until its first
        // __syncthreads; sh.prow is rewritten only after the next cluster.sync)
    }
    __syncthreads();
    for (int t = tid; t < rpc * kb; t += kZPanelThreads) {
        const int r = t % rpc, c = t / rpc;
        const int64_t i = k + cta + (int64_t)kZPanelCtas * r;
        if (i < n) A[i + (k + c) * lda] = s_rows[r * RS + c];
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// The panel's interchanges P[k..k+kb) applied in order to the columns
// [c0, c1), one column per thread.
__global__ void zlu_swap_rest_kernel(int64_t c0, int64_t c1, double2* A, int64_t lda, int64_t k, int kb,
                                     const int64_t* __restrict__ P)
{
    const int64_t col = c0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (col >= c1) return;
    double2* a = A + col * lda;
    for (int jj = 0; jj < kb; ++jj) {
        const int64_t j = k + jj, p = P[j];
        if (p != j) {
            const double2 x = a[j];
            a[j] = a[p];
            a[p] = x;
        }
    }
}

// U12 = L11^-1 A12 (L11 unit lower, KB x KB) for the columns [c0, c1): a
// warp per column, lane r holding row r; at step q lane q's entry is final and
// is broadcast by shuffle, and the lanes below subtract L(r, q) x_q.  (One
// column per thread kept the 32-step chain of four dependent DFMA per step in
// one lane: about 60 us for a 32-column narrow update on the look-ahead
// chain; a warp per column takes a few.)
constexpr int kZTrsmWarps = 4;
template <int KB>
__global__ void __launch_bounds__(32 * kZTrsmWarps)
zlu_trsm_kernel(int64_t c1, double2* A, int64_t lda, int64_t k, int64_t c0)
{
    static_assert(KB <= 32, "a lane per row");
    __shared__ double2 s_l[KB][KB + 1];
    for (int t = threadIdx.x; t < KB * KB; t += blockDim.x) {
        const int r = t % KB, q = t / KB;
        s_l[r][q] = A[(k + r) + (k + q) * lda];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t col = c0 + (int64_t)blockIdx.x * kZTrsmWarps + warp;
    if (col >= c1) return;
    double2* a = A + k + col * lda;
    double2 x = lane < KB ? a[lane] : make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < KB; ++q) {
        const double xr = __shfl_sync(0xffffffffu, x.x, q), xi = __shfl_sync(0xffffffffu, x.y, q);
        if (lane > q && lane < KB) {
            const double2 l = s_l[lane][q];
            x.x = fma(-l.x, xr, x.x);
            x.x = fma(l.y, xi, x.x);
            x.y = fma(-l.x, xi, x.y);
            x.y = fma(-l.y, xr, x.y);
        }
    }
    if (lane < KB) a[lane] = x;
}

// A22 -= L21 U12 (K = KB): 64 x 64 complex tiles, each of the 256 threads a
// 4 x 4 block, complex products on the DFMA pipe.
constexpr int kZgBM = 64, kZgBN = 64, kZgBK = 8;
template <int KB>
__global__ void __launch_bounds__(256)
zlu_gemm_kernel(int64_t n, double2* A, int64_t lda, int64_t k, int64_t cbeg, int64_t cend)
{
    __shared__ double2 s_a[kZgBK][kZgBM];
    __shared__ double2 s_b[kZgBK][kZgBN + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t r0 = k + KB + (int64_t)blockIdx.x * kZgBM;  // rows of A22
    const int64_t c0 = cbeg + (int64_t)blockIdx.y * kZgBN;    // columns [cbeg, cend) of A22
    double2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);
    for (int kk = 0; kk < KB; kk += kZgBK) {
        for (int t = tid; t < kZgBK * kZgBM; t += 256) {
            const int r = t % kZgBM, q = t / kZgBM;
            const int64_t gi = r0 + r;
            s_a[q][r] = gi < n ? A[gi + (k + kk + q) * lda] : make_double2(0.0, 0.0);
        }
        for (int t = tid; t < kZgBK * kZgBN; t += 256) {
            const int q = t % kZgBK, cc = t / kZgBK;
            const int64_t gj = c0 + cc;
            s_b[q][cc] = gj < cend ? A[(k + kk + q) + gj * lda] : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kZgBK; ++q) {
            double2 av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = s_a[q][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = s_b[q][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    acc[a][b].x = fma(av[a].x, bv[b].x, acc[a][b].x);
                    acc[a][b].x = fma(-av[a].y, bv[b].y, acc[a][b].x);
                    acc[a][b].y = fma(av[a].x, bv[b].y, acc[a][b].y);
                    acc[a][b].y = fma(av[a].y, bv[b].x, acc[a][b].y);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int64_t gj = c0 + ty + 16 * b;
        if (gj >= cend) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int64_t gi = r0 + tx + 16 * a;
            if (gi < n) {
                double2* p = &A[gi + gj * lda];
                *p = make_double2(p->x - acc[a][b].x, p->y - acc[a][b].y);
            }
        }
    }
}

// The panel width for n: 32 where ceil(n/16) rows of 33 entries fit the
// shared memory, else 16; 0 (column path) beyond.
static int zpanel_width(int64_t n)
{
    const int64_t rpc = ceil_div(n, kZPanelCtas);
    if ((size_t)rpc * 33 * sizeof(double2) <= kZPanelSmemMax) return 32;
    if ((size_t)rpc * 17 * sizeof(double2) <= kZPanelSmemMax) return 16;
    return 0;
}

// Whether the 16-CTA panel cluster of width KB can run here with the most
// shared memory it may ask for (checked once per context and width).
template <int KB>
static bool zpanel_cluster_ok(Context* c)
{
    static_assert(kZPanelCtas == 16, "non-portable cluster size");
    int& ok = c->zpanel_ok[KB == 32 ? 0 : 1];
    if (ok >= 0) return ok == 1;
    ok = 0;
    if (cudaFuncSetAttribute(zlu_panel_smem_kernel<KB>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess ||
        cudaFuncSetAttribute(zlu_panel_smem_kernel<KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kZPanelSmemMax) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kZPanelCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(kZPanelCtas);
    cfg.blockDim = dim3(kZPanelThreads);
    cfg.dynamicSmemBytes = kZPanelSmemMax;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, zlu_panel_smem_kernel<KB>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ok = clusters >= 1 ? 1 : 0;
    return ok == 1;
}

// Look-ahead: panel k+1 runs on the high-priority side stream as soon as
// step k has updated its columns (the "narrow" update: interchanges, U12 and
// the product for those KB columns, on the main stream), beside step k's
// update of every other column (the "wide" update); the main stream waits for
// panel k+1 before step k+1.  The panel and the wide update touch disjoint
// columns.
template <int KB>
static tmvg_status zlu_factor_blocked(Context* c, int64_t n, double2* A, int64_t lda, int64_t* P)
{
    tmvg_status st = ensure_side_stream(c);
    if (st) return st;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kZPanelCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(kZPanelCtas);
    cfg.blockDim = dim3(kZPanelThreads);
    cfg.stream = c->side;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    auto panel = [&](int64_t k) -> tmvg_status {
        const int kb = (int)std::min<int64_t>(KB, n - k);
        const int rpc = (int)ceil_div(n - k, kZPanelCtas);
        cfg.dynamicSmemBytes = (size_t)rpc * (KB + 1) * sizeof(double2);
        ++c->launches;
        return check_cuda(c, cudaLaunchKernelEx(&cfg, zlu_panel_smem_kernel<KB>, n, A, lda, k, kb, P, rpc),
                          "lu_z: panel launch");
    };
    auto swap = [&](int64_t c0, int64_t c1, int64_t k, int kb) {
        if (c1 <= c0) return;
        zlu_swap_rest_kernel<<<(unsigned)ceil_div(c1 - c0, 128), 128, 0, c->stream>>>(c0, c1, A, lda, k, kb, P);
        ++c->launches;
    };
    // step k's U12 and product for the columns [c0, c1) (k + KB <= c0)
    auto update = [&](int64_t k, int64_t c0, int64_t c1) {
        if (c1 <= c0 || k + KB >= n) return;
        zlu_trsm_kernel<KB><<<(unsigned)ceil_div(c1 - c0, kZTrsmWarps), 32 * kZTrsmWarps, 0, c->stream>>>(
            c1, A, lda, k, c0);
        const dim3 grid((unsigned)ceil_div(n - k - KB, kZgBM), (unsigned)ceil_div(c1 - c0, kZgBN));
        zlu_gemm_kernel<KB><<<grid, 256, 0, c->stream>>>(n, A, lda, k, c0, c1);
        c->launches += 2;
    };
    if ((st = check_cuda(c, cudaEventRecord(c->ev_fork, c->stream), "lu_z: fork"))) return st;
    if ((st = check_cuda(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0), "lu_z: fork wait"))) return st;
    if ((st = panel(0))) return st;
    if ((st = check_cuda(c, cudaEventRecord(c->ev_panel, c->side), "lu_z: panel event"))) return st;
    for (int64_t k = 0; k < n; k += KB) {
        const int kb = (int)std::min<int64_t>(KB, n - k);
        if ((st = check_cuda(c, cudaStreamWaitEvent(c->stream, c->ev_panel, 0), "lu_z: panel wait"))) return st;
        const int64_t kn = k + kb, kn1 = std::min<int64_t>(n, kn + KB);
        if (kn < n) {
            // narrow: the next panel's columns, then that panel on the side stream
            swap(kn, kn1, k, kb);
            update(k, kn, kn1);
            if ((st = check_cuda(c, cudaGetLastError(), "lu_z: narrow update"))) return st;
            if ((st = check_cuda(c, cudaEventRecord(c->ev_wide, c->stream), "lu_z: narrow event"))) return st;
            if ((st = check_cuda(c, cudaStreamWaitEvent(c->side, c->ev_wide, 0), "lu_z: narrow wait"))) return st;
            if ((st = panel(kn))) return st;
            if ((st = check_cuda(c, cudaEventRecord(c->ev_panel, c->side), "lu_z: panel event"))) return st;
        }
        // wide: the factored columns before the panel and the columns beyond
        // the next panel
        swap(0, k, k, kb);
        swap(kn1, n, k, kb);
        update(k, kn1, n);
        if ((st = check_cuda(c, cudaGetLastError(), "lu_z: wide update"))) return st;
    }
    return TMVG_OK;
}

tmvg_status zlu_factor(Context* c, int64_t n, double2* A, int64_t lda, int64_t* P)
{
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "lu_z: bad n/lda");
    if (n == 0) return TMVG_OK;
    if (n >= kZBlockedMin) {
        const int w = zpanel_width(n);
        if (w == 32 && zpanel_cluster_ok<32>(c)) return zlu_factor_blocked<32>(c, n, A, lda, P);
        if (w == 16 && zpanel_cluster_ok<16>(c)) return zlu_factor_blocked<16>(c, n, A, lda, P);
    }
    int* flag = (int*)workspace(c, 256);
    if (!flag) return TMVG_OOM;
    const unsigned gcols = (unsigned)std::min<int64_t>(ceil_div(n, kZThreads), 4 * c->num_sms);
    for (int64_t k = 0; k < n; ++k) {
        zlu_pivot_kernel<<<1, kZPivThreads, 0, c->stream>>>(n, A, lda, k, P, flag);
        zlu_swap_kernel<<<gcols, kZThreads, 0, c->stream>>>(n, A, lda, k, P);
        zlu_scale_kernel<<<gcols, kZThreads, 0, c->stream>>>(n, A, lda, k, flag);
        c->launches += 3;
        const int64_t rest = n - k - 1;
        if (rest > 0) {
            const dim3 g((unsigned)ceil_div(rest, kZTile), (unsigned)ceil_div(rest, kZTile));
            zlu_update_kernel<<<g, dim3(kZTile, kZTile), 0, c->stream>>>(n, A, lda, k);
            ++c->launches;
        }
        const tmvg_status st = check_cuda(c, cudaGetLastError(), "lu_z: launch");
        if (st) return st;
    }
    return TMVG_OK;
}

// One right-hand side per CTA: b := U^-1 L^-1 (P b) in place.
__global__ void __launch_bounds__(kZThreads)
zlu_solve_kernel(int64_t n, const double2* __restrict__ LU, int64_t lda, const int64_t* __restrict__ P,
                 double2* B, int64_t ldb, int* err)
{
    __shared__ double2 s_bj;
    __shared__ int s_stop;
    double2* b = B + blockIdx.x * ldb;
    const int tid = threadIdx.x;
    if (tid == 0) {
        s_stop = 0;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t p = P[i];
            if (p != i && p >= 0 && p < n) {
                const double2 t = b[i];
                b[i] = b[p];
                b[p] = t;
            }
        }
    }
    __syncthreads();
    // unit lower L, columns in order
    for (int64_t j = 0; j + 1 < n; ++j) {
        if (tid == 0) s_bj = b[j];
        __syncthreads();
        const double2 bj = s_bj;
        if (znonzero(bj))
            for (int64_t i = j + 1 + tid; i < n; i += kZThreads) b[i] = zsub(b[i], zmul(bj, LU[i + j * lda]));
        __syncthreads();
    }
    // upper U, columns from the last
    for (int64_t j = n - 1; j >= 0; --j) {
        if (tid == 0) {
            double2 v = b[j];
            if (znonzero(v)) {
                const double2 d = LU[j + j * lda];
                if (!znonzero(d)) {
                    atomicCAS(err, (int)kDevOk, (int)kDevSingular);
                    s_stop = 1;
                } else {
                    v = zmul(v, tmv_inverse_of(d));
                    b[j] = v;
                }
            }
            s_bj = v;
        }
        __syncthreads();
        if (s_stop) return;
        const double2 bj = s_bj;
        if (znonzero(bj))
            for (int64_t i = tid; i < j; i += kZThreads) b[i] = zsub(b[i], zmul(bj, LU[i + j * lda]));
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Blocked left solve (n >= kZBlockedMin): B is gathered into a scratch copy in
// the pivoted row order, then solved by 64-row blocks: each diagonal block by
// one CTA per 4 right-hand sides, a thread per (row, column) and one barrier
// per step (the column-oriented solve: a zero entry is skipped; a nonzero
// entry meeting a zero U(j,j) is singular; division as b * TMV_InverseOf(d),
// the inverses taken once for the whole diagonal), the rows beyond the block
// updated by a complex product; then the result is copied back.  Values agree
// with the column-by-column solve to rounding.
// ---------------------------------------------------------------------------
constexpr int kZSolveBlock = 64;
constexpr int kZSolveCols = 4;

__global__ void zlu_gather_rows_kernel(int64_t n, int64_t nrhs, const int* __restrict__ perm,
                                       const double2* __restrict__ B, int64_t ldb, double2* __restrict__ X)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * nrhs) return;
    const int64_t i = t % n, q = t / n;
    X[i + q * n] = B[(int64_t)perm[i] + q * ldb];
}

__global__ void zlu_copy_back_kernel(int64_t n, int64_t nrhs, const double2* __restrict__ X,
                                     double2* __restrict__ B, int64_t ldb)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * nrhs) return;
    const int64_t i = t % n, q = t / n;
    B[i + q * ldb] = X[i + q * n];
}

__global__ void zlu_diag_inverse_kernel(int64_t n, const double2* __restrict__ LU, int64_t lda,
                                        double2* __restrict__ dinv)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double2 d = LU[j + j * lda];
    dinv[j] = znonzero(d) ? tmv_inverse_of(d) : make_double2(0.0, 0.0);
}

// One 64-row diagonal block [k, k+w) of the unit lower (upper = false) or
// non-unit upper triangle for columns [q0, q0 + 4) of X (n x nrhs, ld n); the
// block's triangle is staged in shared memory first (dynamic, 64 x 65
// entries), so that the 64 steps read it at shared-memory latency.
__global__ void __launch_bounds__(kZSolveBlock * kZSolveCols)
zlu_diag_solve_kernel(int64_t n, const double2* __restrict__ LU, int64_t lda, const double2* __restrict__ dinv,
                      int64_t k, int w, bool upper, int64_t nrhs, double2* X, int* err)
{
    __shared__ double2 xs[kZSolveBlock][kZSolveCols];
    extern __shared__ double2 s_tri[];  // [kZSolveBlock][kZSolveBlock + 1]
    const int i = threadIdx.x % kZSolveBlock, ql = threadIdx.x / kZSolveBlock;
    const int64_t q = (int64_t)blockIdx.x * kZSolveCols + ql;
    const bool mine = i < w && q < nrhs;
    double2* x = X + k + q * n;
    xs[i][ql] = mine ? x[i] : make_double2(0.0, 0.0);
    for (int t = threadIdx.x; t < w * w; t += kZSolveBlock * kZSolveCols) {
        const int r = t % w, cc = t / w;
        s_tri[r * (kZSolveBlock + 1) + cc] = LU[(k + r) + (k + cc) * lda];
    }
    bool sing = false;
    __syncthreads();
    for (int s = 0; s < w; ++s) {
        const int j = upper ? w - 1 - s : s;
        if (upper) {
            if (i == j && mine) {
                const double2 v = xs[j][ql];
                if (znonzero(v)) {
                    const double2 d = s_tri[j * (kZSolveBlock + 1) + j];
                    if (!znonzero(d)) sing = true;
                    else xs[j][ql] = zmul(v, dinv[k + j]);
                }
            }
            __syncthreads();
        }
        const double2 xj = xs[j][ql];
        const bool below = upper ? i < j : i > j;
        if (mine && below && znonzero(xj))
            xs[i][ql] = zsub(xs[i][ql], zmul(xj, s_tri[i * (kZSolveBlock + 1) + j]));
        __syncthreads();
    }
    if (sing) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
    if (mine) x[i] = xs[i][ql];
}

// C -= A B for a few columns (N <= 16): a thread per entry of C.
__global__ void zlu_gemm_skinny_kernel(int64_t M, int64_t N, int K, const double2* __restrict__ A, int64_t lda,
                                       const double2* __restrict__ B, int64_t ldb, double2* __restrict__ C,
                                       int64_t ldc)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= M * N) return;
    const int64_t i = t % M, q = t / M;
    double re = 0.0, im = 0.0;
    for (int kk = 0; kk < K; ++kk) {
        const double2 a = A[i + kk * lda], b = B[kk + q * ldb];
        re = fma(a.x, b.x, re);
        re = fma(-a.y, b.y, re);
        im = fma(a.x, b.y, im);
        im = fma(a.y, b.x, im);
    }
    double2* cp = &C[i + q * ldc];
    *cp = make_double2(cp->x - re, cp->y - im);
}

// C -= A B, general: 64 x 64 tiles, each of the 256 threads a 4 x 4 block.
__global__ void __launch_bounds__(256)
zlu_gemm_tiled_kernel(int64_t M, int64_t N, int K, const double2* __restrict__ A, int64_t lda,
                      const double2* __restrict__ B, int64_t ldb, double2* __restrict__ C, int64_t ldc)
{
    __shared__ double2 s_a[kZgBK][kZgBM];
    __shared__ double2 s_b[kZgBK][kZgBN + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t r0 = (int64_t)blockIdx.x * kZgBM, c0 = (int64_t)blockIdx.y * kZgBN;
    double2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);
    for (int kk = 0; kk < K; kk += kZgBK) {
        for (int t = tid; t < kZgBK * kZgBM; t += 256) {
            const int r = t % kZgBM, q = t / kZgBM;
            s_a[q][r] = (r0 + r < M && kk + q < K) ? A[(r0 + r) + (kk + q) * lda] : make_double2(0.0, 0.0);
        }
        for (int t = tid; t < kZgBK * kZgBN; t += 256) {
            const int q = t % kZgBK, cc = t / kZgBK;
            s_b[q][cc] = (c0 + cc < N && kk + q < K) ? B[(kk + q) + (c0 + cc) * ldb] : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kZgBK; ++q) {
            double2 av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = s_a[q][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = s_b[q][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    acc[a][b].x = fma(av[a].x, bv[b].x, acc[a][b].x);
                    acc[a][b].x = fma(-av[a].y, bv[b].y, acc[a][b].x);
                    acc[a][b].y = fma(av[a].x, bv[b].y, acc[a][b].y);
                    acc[a][b].y = fma(av[a].y, bv[b].x, acc[a][b].y);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int64_t gj = c0 + ty + 16 * b;
        if (gj >= N) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int64_t gi = r0 + tx + 16 * a;
            if (gi < M) {
                double2* cp = &C[gi + gj * ldc];
                *cp = make_double2(cp->x - acc[a][b].x, cp->y - acc[a][b].y);
            }
        }
    }
}

static tmvg_status zgemm_sub(Context* c, int64_t M, int64_t N, int K, const double2* A, int64_t lda,
                             const double2* B, int64_t ldb, double2* C, int64_t ldc)
{
    if (M <= 0 || N <= 0 || K <= 0) return TMVG_OK;
    if (N <= 16) {
        zlu_gemm_skinny_kernel<<<(unsigned)ceil_div(M * N, 128), 128, 0, c->stream>>>(M, N, K, A, lda, B, ldb, C,
                                                                                        ldc);
    } else {
        const dim3 grid((unsigned)ceil_div(M, kZgBM), (unsigned)ceil_div(N, kZgBN));
        zlu_gemm_tiled_kernel<<<grid, 256, 0, c->stream>>>(M, N, K, A, lda, B, ldb, C, ldc);
    }
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "lu_ldiveq_z: product");
}

static tmvg_status zlu_ldiveq_blocked(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P,
                                      int64_t nrhs, double2* B, int64_t ldb)
{
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_perm = 0, o_dinv = al(sizeof(int) * n), o_x = o_dinv + al(sizeof(double2) * n);
    unsigned char* ws = (unsigned char*)workspace(c, o_x + sizeof(double2) * (size_t)n * nrhs);
    if (!ws) return set_error(c, TMVG_OOM, "lu_ldiveq_z: workspace");
    int* perm = (int*)(ws + o_perm);
    double2* dinv = (double2*)(ws + o_dinv);
    double2* X = (double2*)(ws + o_x);
    tmvg_status st = pivots_to_perm(c, n, P, perm);
    if (st) return st;
    const unsigned ge = (unsigned)ceil_div(n * nrhs, 256);
    zlu_gather_rows_kernel<<<ge, 256, 0, c->stream>>>(n, nrhs, perm, B, ldb, X);
    zlu_diag_inverse_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, c->stream>>>(n, LU, lda, dinv);
    c->launches += 2;
    if ((st = check_cuda(c, cudaGetLastError(), "lu_ldiveq_z: gather"))) return st;
    const unsigned gq = (unsigned)ceil_div(nrhs, kZSolveCols);
    const size_t tri_smem = sizeof(double2) * kZSolveBlock * (kZSolveBlock + 1);
    if ((st = check_cuda(c, cudaFuncSetAttribute(zlu_diag_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)tri_smem),
                         "lu_ldiveq_z: smem attribute")))
        return st;
    // L (unit lower), blocks in order
    for (int64_t k = 0; k < n; k += kZSolveBlock) {
        const int w = (int)std::min<int64_t>(kZSolveBlock, n - k);
        zlu_diag_solve_kernel<<<gq, kZSolveBlock * kZSolveCols, tri_smem, c->stream>>>(n, LU, lda, dinv, k, w,
                                                                                        false, nrhs, X, c->dflags);
        ++c->launches;
        if ((st = check_cuda(c, cudaGetLastError(), "lu_ldiveq_z: diagonal block"))) return st;
        if ((st = zgemm_sub(c, n - k - w, nrhs, w, LU + (k + w) + k * lda, lda, X + k, n, X + k + w, n))) return st;
    }
    // U (non-unit upper), blocks from the last
    for (int64_t k = ((n - 1) / kZSolveBlock) * kZSolveBlock; k >= 0; k -= kZSolveBlock) {
        const int w = (int)std::min<int64_t>(kZSolveBlock, n - k);
        zlu_diag_solve_kernel<<<gq, kZSolveBlock * kZSolveCols, tri_smem, c->stream>>>(n, LU, lda, dinv, k, w,
                                                                                        true, nrhs, X, c->dflags);
        ++c->launches;
        if ((st = check_cuda(c, cudaGetLastError(), "lu_ldiveq_z: diagonal block"))) return st;
        if ((st = zgemm_sub(c, k, nrhs, w, LU + k * lda, lda, X + k, n, X, n))) return st;
    }
    zlu_copy_back_kernel<<<ge, 256, 0, c->stream>>>(n, nrhs, X, B, ldb);
    ++c->launches;
    if ((st = check_cuda(c, cudaGetLastError(), "lu_ldiveq_z: copy back"))) return st;
    return collect_device_error(c, "lu_ldiveq_z");
}

tmvg_status zlu_ldiveq(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, int64_t nrhs,
                       double2* B, int64_t ldb)
{
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "lu_ldiveq_z: bad sizes");
    if (n == 0 || nrhs == 0) return TMVG_OK;
    if (n >= kZBlockedMin && n <= (int64_t)INT32_MAX) return zlu_ldiveq_blocked(c, n, LU, lda, P, nrhs, B, ldb);
    if (nrhs > 65535) return set_error(c, TMVG_UNSUPPORTED, "lu_ldiveq_z: too many right-hand sides");
    zlu_solve_kernel<<<(unsigned)nrhs, kZThreads, 0, c->stream>>>(n, LU, lda, P, B, ldb, c->dflags);
    ++c->launches;
    const tmvg_status st = check_cuda(c, cudaGetLastError(), "lu_ldiveq_z: launch");
    if (st) return st;
    return collect_device_error(c, "lu_ldiveq_z");
}

// One row of B per CTA: b := b (P L U)^-1 (LU_RDivEq, src/TMV_LUDiv.cpp:370-411:
// m %= U, m %= L, m.reversePermuteCols(P)).  m %= T is T^T.LDivEq(m^T), and
// U^T and L^T of a column-major LU are row-major, so TMV takes its
// row-oriented vector solves (src/TMV_TriDiv_V.cpp:59-146, 237-320) after
// trimming the leading (lower) or trailing (upper) zeros of b (:401-462): each
// entry's terms subtracted one by one in index order, a zero U(i,i) singular.
// One thread substitutes the row in that order.
__global__ void zlu_rsolve_kernel(int64_t n, const double2* __restrict__ LU, int64_t lda,
                                  const int64_t* __restrict__ P, double2* B, int64_t ldb, int* err)
{
    if (threadIdx.x != 0) return;
    double2* x = B + blockIdx.x;  // row r: entry j at x[j * ldb]
#define X(i) x[(i) * ldb]
    int64_t i1 = 0;
    while (i1 < n && !znonzero(X(i1))) ++i1;
    for (int64_t i = i1; i < n; ++i) {
        double2 v = X(i);
        for (int64_t j = i1; j < i; ++j) v = zsub(v, zmul(X(j), LU[j + i * lda]));
        const double2 d = LU[i + i * lda];
        if (!znonzero(d)) {
            atomicCAS(err, (int)kDevOk, (int)kDevSingular);
            return;
        }
        X(i) = zmul(v, tmv_inverse_of(d));
    }
    int64_t i2 = n;
    while (i2 > 0 && !znonzero(X(i2 - 1))) --i2;
    for (int64_t i = i2 - 1; i >= 0; --i) {
        double2 v = X(i);
        for (int64_t j = i + 1; j < i2; ++j) v = zsub(v, zmul(X(j), LU[j + i * lda]));
        X(i) = v;
    }
    for (int64_t i = n - 1; i >= 0; --i) {
        const int64_t p = P[i];
        if (p != i && p >= 0 && p < n) {
            const double2 t = X(i);
            X(i) = X(p);
            X(p) = t;
        }
    }
#undef X
}

tmvg_status zlu_rdiveq(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, int64_t nrows,
                       double2* B, int64_t ldb)
{
    if (n < 0 || nrows < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(nrows, 1))
        return set_error(c, TMVG_BAD_ARG, "lu_rdiveq_z: bad sizes");
    if (n == 0 || nrows == 0) return TMVG_OK;
    if (nrows > 65535) return set_error(c, TMVG_UNSUPPORTED, "lu_rdiveq_z: too many rows");
    zlu_rsolve_kernel<<<(unsigned)nrows, 32, 0, c->stream>>>(n, LU, lda, P, B, ldb, c->dflags);
    ++c->launches;
    const tmvg_status st = check_cuda(c, cudaGetLastError(), "lu_rdiveq_z: launch");
    if (st) return st;
    return collect_device_error(c, "lu_rdiveq_z");
}

__global__ void zlu_identity_kernel(int64_t n, double2* M, int64_t ldm)
{
    const int64_t total = n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, j = t / n;
        M[i + j * ldm] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    }
}

// m.inverse() from the factors (LUDiv::doMakeInverse -> LU_Inverse,
// src/TMV_LUInverse.cpp:236): M = (P L U)^-1, which is TMV's U^-1 L^-1 with
// its columns reverse-permuted, here as the left division of the identity
// (one column per CTA, TMV's vector solves); values agree to rounding.  A
// zero U(j,j) met by a column is TMVG_SINGULAR, as TMV's triangular inverse
// throws.
tmvg_status zlu_inverse(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, double2* M,
                        int64_t ldm)
{
    if (n < 0 || lda < std::max<int64_t>(n, 1) || ldm < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "inverse_z: bad sizes");
    if (n == 0) return TMVG_OK;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n * n, kZThreads), 8 * c->num_sms);
    zlu_identity_kernel<<<blocks, kZThreads, 0, c->stream>>>(n, M, ldm);
    ++c->launches;
    const tmvg_status st = check_cuda(c, cudaGetLastError(), "inverse_z: launch");
    if (st) return st;
    return zlu_ldiveq(c, n, LU, lda, P, n, M, ldm);
}

}  // namespace tmvg
