// lu.cu -- partial-pivoting LU factorisation and LU solves on sm_103a.
//
// Algorithm (right-looking, blocked; the reference is recursive,
// src/TMV_LUDecompose.cpp:217-407, and produces the same factors up to the
// rounding of the trailing updates):
//   for each panel of kPanel columns starting at k:
//     1. lu_panel_kernel: factor A[k:n, k:k+nb] column by column with TMV's
//        pivot rule; the panel lives in the shared memory of up to one CTA
//        per SM, one bounded grid barrier per column;
//     2. laswp_kernel: apply the panel's interchanges to the other columns
//        (TMV: A1.permuteRows(P,0,N1) and A0.permuteRows(P,N1,R));
//     3. tri_diag_kernel: U12 = L11^-1 A12 (TMV: A01 /= A00.lowerTri(UnitDiag));
//     4. gemm: A22 -= L21 U12 (TMV: A11 -= A10*A01 -> MultMM<true>(-1,...)).
//
// Pivot rule (src/TMV_Vector.cpp:474-503, src/TMV_LUDecompose.cpp:274-383):
// first index of the strict maximum |a| over the sub-column, NaN handling as
// described at pivot_key(); a maximum |a| < DBL_MIN (TMV_Underflow,
// include/tmv/TMV_Base.h:692-696) zeroes the sub-column and records P[j] = j.
// The L column is scaled by the reciprocal of the pivot, as TMV's v /= x does
// (include/tmv/TMV_VectorArith.h:104-106).
#include "async.cuh"
#include "gemm_tc.cuh"
#include "lu.cuh"
#include "pivots.cuh"
#include "trsv.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

namespace tmvg {

constexpr int kPanelThreads = 256;
constexpr int kPanelMax = 128;  // largest panel width (scratch layout)
constexpr int kTriBlock = 64;   // diagonal block of the blocked triangular solves

// Panel width: 64 columns in FP64, 128 in FP32 (same shared-memory
// footprint, 256 rows x ~33 KB per CTA; wider FP32 panels halve the number
// of trailing updates and so the trailing-matrix traffic).
template <typename T>
constexpr int panel_width() { return sizeof(T) == 8 ? 64 : 128; }

// ---------------------------------------------------------------------
// Columns that TMV factors as the second column of a two-column leaf of its
// recursion (split N1 = R/2, rounded down to a multiple of 64 above 64,
// src/TMV_LUDecompose.cpp:241-245).  Their pivot scan starts from max = 0,
// which only matters for NaN input.
// ---------------------------------------------------------------------
static void leaf_modes(int64_t off, int64_t R, std::vector<unsigned char>& modes)
{
    if (R > 2) {
        int64_t N1 = R / 2;
        if (N1 > 64) N1 = (N1 / 64) * 64;
        leaf_modes(off, N1, modes);
        leaf_modes(off + N1, R - N1, modes);
    } else if (R == 2) {
        modes[off + 1] = 1;
    }
}

// ---------------------------------------------------------------------
// Panel factorisation.
// ---------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
lu_panel_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int nb,
                int64_t* __restrict__ P, const unsigned char* __restrict__ modes,
                int rows_per_cta, double* cand_key, long long* cand_idx,
                T* cand_rows, T* diag_row, unsigned* bar, int* err, int* pairs)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* rows = reinterpret_cast<T*>(smem_raw);
    const int ldp = nb + 1;
    __shared__ double s_key[kPanelThreads / 32];
    __shared__ long long s_idx[kPanelThreads / 32];
    __shared__ double w_key;
    __shared__ long long w_idx;
    __shared__ T urow[kPanelMax];
    __shared__ int s_piv[kPanelMax];

    const int G = gridDim.x;
    const int cta = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t m = n - k;
    const int64_t r0 = (int64_t)cta * rows_per_cta;
    const int nr = (int)max((int64_t)0, min((int64_t)rows_per_cta, m - r0));

    for (int t = tid; t < nr * nb; t += kPanelThreads) {
        const int r = t % nr, cc = t / nr;
        rows[r * ldp + cc] = A[(k + r0 + r) + (k + cc) * lda];
    }
    __syncthreads();

    bool prev_uf = false;
    for (int jj = 0; jj < nb; ++jj) {
        const int par = jj & 1;
        const bool r2 = modes[jj] && !prev_uf;

        // 1. this CTA's best candidate among panel rows >= jj
        double bk = -INFINITY;
        long long bi = LLONG_MAX;
        for (int r = tid; r < nr; r += kPanelThreads) {
            const int64_t pr = r0 + r;
            if (pr < jj) continue;
            pivot_combine(bk, bi, pivot_key(rows[r * ldp + jj], pr == jj, r2), (long long)pr);
        }
        warp_pivot_reduce(bk, bi);
        if (lane == 0) { s_key[warp] = bk; s_idx[warp] = bi; }
        __syncthreads();
        if (warp == 0) {
            bk = lane < kPanelThreads / 32 ? s_key[lane] : -INFINITY;
            bi = lane < kPanelThreads / 32 ? s_idx[lane] : LLONG_MAX;
            warp_pivot_reduce(bk, bi);
            if (lane == 0) {
                __stcg(&cand_key[par * G + cta], bk);
                __stcg(&cand_idx[par * G + cta], bi);
                w_idx = bi;  // local use below
            }
        }
        __syncthreads();
        // 2. publish the candidate row and (owner only) the diagonal row
        {
            const long long mine = w_idx;
            if (mine != LLONG_MAX) {
                const int r = (int)(mine - r0);
                for (int cc = tid; cc < nb; cc += kPanelThreads)
                    __stcg(&cand_rows[((int64_t)par * G + cta) * kPanelMax + cc], rows[r * ldp + cc]);
            }
            if (jj >= r0 && jj < r0 + nr) {
                const int r = (int)(jj - r0);
                for (int cc = tid; cc < nb; cc += kPanelThreads)
                    __stcg(&diag_row[par * kPanelMax + cc], rows[r * ldp + cc]);
            }
        }
        if (!grid_barrier(bar, (unsigned)(jj + 1) * (unsigned)G, err)) return;

        // 3. global winner
        if (warp == 0) {
            double kk = -INFINITY;
            long long ii = LLONG_MAX;
            for (int g = lane; g < G; g += 32)
                pivot_combine(kk, ii, __ldcg(&cand_key[par * G + g]), __ldcg(&cand_idx[par * G + g]));
            warp_pivot_reduce(kk, ii);
            if (lane == 0) { w_key = kk; w_idx = ii; }
        }
        __syncthreads();
        const double wk = w_key;
        const long long wi = w_idx;  // panel row of the pivot

        if (underflows<T>(wk)) {
            if (tid == 0) s_piv[jj] = (int)(k + jj);
            if (cta == 0 && tid == 0) P[k + jj] = k + jj;
            for (int r = tid; r < nr; r += kPanelThreads)
                if (r0 + r >= jj) rows[r * ldp + jj] = T(0);
            prev_uf = true;
        } else {
            prev_uf = false;
            if (tid == 0) s_piv[jj] = (int)(k + wi);
            if (cta == 0 && tid == 0) P[k + jj] = k + wi;
            const int wc = (int)(wi / rows_per_cta);
            for (int cc = tid; cc < nb; cc += kPanelThreads)
                urow[cc] = __ldcg(&cand_rows[((int64_t)par * G + wc) * kPanelMax + cc]);
            __syncthreads();
            if (wi != jj) {
                if (jj >= r0 && jj < r0 + nr) {
                    const int r = (int)(jj - r0);
                    for (int cc = tid; cc < nb; cc += kPanelThreads) rows[r * ldp + cc] = urow[cc];
                }
                if (wi >= r0 && wi < r0 + nr) {
                    const int r = (int)(wi - r0);
                    for (int cc = tid; cc < nb; cc += kPanelThreads)
                        rows[r * ldp + cc] = __ldcg(&diag_row[par * kPanelMax + cc]);
                }
            }
            __syncthreads();
            const T inv = T(1) / urow[jj];
            for (int r = tid; r < nr; r += kPanelThreads) {
                if (r0 + r <= jj) continue;
                T* rw = rows + r * ldp;
                const T l = rw[jj] * inv;
                rw[jj] = l;
                for (int cc = jj + 1; cc < nb; ++cc) rw[cc] -= l * urow[cc];
            }
        }
        __syncthreads();
    }

    for (int t = tid; t < nr * nb; t += kPanelThreads) {
        const int r = t % nr, cc = t / nr;
        A[(k + r0 + r) + (k + cc) * lda] = rows[r * ldp + cc];
    }
    if (cta == 0 && warp == 0) panel_row_pairs(k, nb, s_piv, pairs);
}


// ---------------------------------------------------------------------
// Panel factorisation on one 16-CTA thread-block cluster.
//
// When the panel's rows fit in the shared memory of 16 SMs, one cluster
// holds the whole panel in distributed shared memory and the CTAs exchange
// pivot candidates and the pivot row through DSMEM, synchronising with the
// hardware cluster barrier once per column: each CTA publishes its candidate
// (key, index and a copy of the row) and the owner of row j publishes a copy
// of row j; after the barrier every CTA reduces the candidates itself and
// the two owners complete the interchange from the copies.  There is no
// global-memory traffic or spinning per column.
// The pivot rule and the arithmetic are those of lu_panel_kernel.
// ---------------------------------------------------------------------
constexpr int kClusterCtas = 16;

template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
lu_panel_cluster_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int nb,
                        int64_t* __restrict__ P, const unsigned char* __restrict__ modes,
                        int rows_per_cta, int* pairs)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* rows = reinterpret_cast<T*>(smem_raw);
    const int ldp = nb + 1;
    __shared__ double s_key[kPanelThreads / 32];
    __shared__ long long s_idx[kPanelThreads / 32];
    // per-column candidates published to the cluster, double-buffered by
    // column parity so one cluster barrier per column separates each write
    // from the remote reads of the same buffer
    __shared__ double cand_key[2];
    __shared__ long long cand_idx[2];
    __shared__ T cand_row[2][kPanelMax];
    __shared__ T diag_row[2][kPanelMax];
    __shared__ T urow[kPanelMax];
    __shared__ int s_piv[kPanelMax];

    const int G = (int)cluster.num_blocks();
    const int cta = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t m = n - k;
    const int64_t r0 = (int64_t)cta * rows_per_cta;
    const int nr = (int)max((int64_t)0, min((int64_t)rows_per_cta, m - r0));

    for (int t = tid; t < nr * nb; t += kPanelThreads) {
        const int r = t % nr, cc = t / nr;
        rows[r * ldp + cc] = A[(k + r0 + r) + (k + cc) * lda];
    }
    __syncthreads();

    bool prev_uf = false;
    for (int jj = 0; jj < nb; ++jj) {
        const int par = jj & 1;
        const bool r2 = modes[jj] && !prev_uf;
        const int owner_j = jj / rows_per_cta;
        // each thread scans (and later updates) the rows tid, tid + 256, ...
        double bk = -INFINITY;
        long long bi = LLONG_MAX;
        for (int r = tid; r < nr; r += kPanelThreads) {
            const int64_t pr = r0 + r;
            if (pr < jj) continue;
            pivot_combine(bk, bi, pivot_key(rows[r * ldp + jj], pr == jj, r2), (long long)pr);
        }
        warp_pivot_reduce(bk, bi);
        if (lane == 0) { s_key[warp] = bk; s_idx[warp] = bi; }
        __syncthreads();
        if (warp == 0) {
            bk = lane < kPanelThreads / 32 ? s_key[lane] : -INFINITY;
            bi = lane < kPanelThreads / 32 ? s_idx[lane] : LLONG_MAX;
            warp_pivot_reduce(bk, bi);
            if (lane == 0) { cand_key[par] = bk; cand_idx[par] = bi; }
            if (bi != LLONG_MAX) {
                const T* src = rows + (bi - r0) * ldp;
                for (int cc = lane; cc < nb; cc += 32) cand_row[par][cc] = src[cc];
            }
        } else if (warp == 1 && cta == owner_j) {
            const T* src = rows + (jj - r0) * ldp;
            for (int cc = lane; cc < nb; cc += 32) diag_row[par][cc] = src[cc];
        }
        cluster.sync();  // the only cluster barrier of this column
        double wk = -INFINITY;
        long long wi = LLONG_MAX;
        if (lane < G) {
            wk = *cluster.map_shared_rank(&cand_key[par], lane);
            wi = *cluster.map_shared_rank(&cand_idx[par], lane);
        }
        warp_pivot_reduce(wk, wi);  // every warp reaches the same winner
        if (underflows<T>(wk)) {
            if (tid == 0) s_piv[jj] = (int)(k + jj);
            if (cta == 0 && tid == 0) P[k + jj] = k + jj;
            for (int r = tid; r < nr; r += kPanelThreads)
                if (r0 + r >= jj) rows[r * ldp + jj] = T(0);
            prev_uf = true;
            continue;
        }
        prev_uf = false;
        if (tid == 0) s_piv[jj] = (int)(k + wi);
        if (cta == 0 && tid == 0) P[k + jj] = k + wi;
        const int owner_w = (int)(wi / rows_per_cta);
        {
            const T* wrow = cluster.map_shared_rank(&cand_row[par][0], owner_w);
            for (int cc = tid; cc < nb; cc += kPanelThreads) {
                const T v = wrow[cc];
                urow[cc] = v;
                if (cta == owner_j) rows[(jj - r0) * ldp + cc] = v;
            }
            if (wi != jj && cta == owner_w) {
                const T* jrow = cluster.map_shared_rank(&diag_row[par][0], owner_j);
                for (int cc = tid; cc < nb; cc += kPanelThreads) rows[(wi - r0) * ldp + cc] = jrow[cc];
            }
        }
        __syncthreads();
        const T inv = T(1) / urow[jj];
        for (int r = tid; r < nr; r += kPanelThreads) {
            if (r0 + r <= jj) continue;
            T* rw = rows + r * ldp;
            const T l = rw[jj] * inv;
            rw[jj] = l;
            for (int cc = jj + 1; cc < nb; ++cc) rw[cc] -= l * urow[cc];
        }
    }
    __syncthreads();

    for (int t = tid; t < nr * nb; t += kPanelThreads) {
        const int r = t % nr, cc = t / nr;
        A[(k + r0 + r) + (k + cc) * lda] = rows[r * ldp + cc];
    }
    if (cta == 0 && warp == 0) panel_row_pairs(k, nb, s_piv, pairs);
    cluster.sync();  // keep every CTA's shared memory alive until all reads are done
}

// ---------------------------------------------------------------------
// Register-resident cluster panel.
//
// Every thread holds panel rows in registers (two: lu_panel_cluster_reg2_kernel),
// so the rank-1 update of column j costs a thread NB-j-1 FMAs per row against
// the pivot row read from shared memory.  Register indices must be static, so the row is kept
// rotated: columns are processed in blocks of 4 (unrolled), the active
// columns of block q sit at positions 0.. of the register array, and after
// each block the array rotates left by 4 (finished columns wrap to the end,
// where the update skips them).  Rows exchanged between threads travel in the
// same rotated order, which every thread shares.
//
// The cluster exchange has no cluster barrier.  Each CTA reduces its
// candidate and publishes it in its own shared memory (the row, double-
// buffered by column parity; the CTA holding row j publishes row j the same
// way), then stores the 16-byte candidate record (key, index) into a slot of
// every CTA and arrives, with cluster-scope release, on that CTA's mbarrier
// for the column's parity.  A CTA's warp 0 waits (acquire) until all 16
// records are in, reduces them, pulls the pivot row from the CTA that holds
// it (and, in the CTA that holds the pivot row, the old row j), and hands
// both to the block through shared memory: one DSMEM round trip per column.
// A CTA rewrites a parity's published rows and remote slots only two columns
// later, after every CTA has arrived for the column in between, which each
// does after its pulls of the column before.  The waits are bounded: on a
// timeout the CTA records kDevTimeout and stops, and the others time out in
// turn.  Used while a 16-CTA cluster covers the panel's rows with two rows
// per thread (m <= 16 * 512); a panel of at most 512 rows runs in one CTA,
// which takes its own candidate with no exchange.
// ---------------------------------------------------------------------
constexpr int kRegBlock = 4;

template <typename T>
struct RegPanel {
    static constexpr int NB = sizeof(T) == 8 ? 32 : 64;  // columns a thread holds
};

// Pivot key as an unsigned integer with the same order: -1 (a NaN that is
// not the first element) -> 0, key k >= 0 -> bits(k) + 1.  Empty slots are 0
// with index INT_MAX, so they lose to every row.
__device__ __forceinline__ unsigned long long pivot_key_bits(double k)
{
    return k < 0 ? 0ull : (unsigned long long)__double_as_longlong(k) + 1ull;
}

__device__ __forceinline__ double pivot_key_value(unsigned long long b)
{
    return b == 0 ? -1.0 : __longlong_as_double((long long)(b - 1));
}

// Warp-wide (key desc, index asc) reduction with three redux.sync steps;
// every lane receives the result.
__device__ __forceinline__ void warp_key_reduce(unsigned long long& key, int& idx)
{
    const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    const unsigned mi = __reduce_min_sync(0xffffffffu, (hi == mhi && lo == mlo) ? (unsigned)idx : 0x7fffffffu);
    key = ((unsigned long long)mhi << 32) | mlo;
    idx = (int)mi;
}

// Pivot key of a panel element with integer operations only: the IEEE bits
// of |v| plus 1 (non-negative floats order like their bit patterns, and the
// conversion of a float to double is exact, so this is the order of the FP64
// comparison of pivot_key()); 0 for a NaN that is not the first element; the
// first element's NaN counts as +inf, or as 0 in the second column of a
// two-column leaf.  FP64 instructions run at 1/64 of the FP32 rate on this
// part, and every thread of the panel computes a key per column.
__device__ __forceinline__ unsigned long long reg_pivot_key(float v, bool first, bool r2mode)
{
    const unsigned a = __float_as_uint(v) & 0x7fffffffu;
    if (a > 0x7f800000u) return first ? (r2mode ? 1ull : 0x7f800001ull) : 0ull;
    return (unsigned long long)a + 1ull;
}
__device__ __forceinline__ unsigned long long reg_pivot_key(double v, bool first, bool r2mode)
{
    const unsigned long long a = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    if (a > 0x7ff0000000000000ull) return first ? (r2mode ? 1ull : 0x7ff0000000000001ull) : 0ull;
    return a + 1ull;
}

// |pivot| < numeric_limits<T>::min() on a reg_pivot_key (key 0 included).
template <typename T>
__device__ __forceinline__ bool reg_key_underflows(unsigned long long key)
{
    return sizeof(T) == 4 ? key <= 0x00800000ull : key <= 0x0010000000000000ull;
}

// warp_key_reduce for reg_pivot_key: FP32 keys fit 32 bits (two redux steps).
template <typename T>
__device__ __forceinline__ void reg_key_reduce(unsigned long long& key, int& idx)
{
    if constexpr (sizeof(T) == 4) {
        const unsigned k32 = (unsigned)key;
        const unsigned mk = __reduce_max_sync(0xffffffffu, k32);
        const unsigned mi = __reduce_min_sync(0xffffffffu, k32 == mk ? (unsigned)idx : 0x7fffffffu);
        key = mk;
        idx = (int)mi;
    } else {
        warp_key_reduce(key, idx);
    }
}

// 16-byte vectors of a row held in registers (4 floats or 2 doubles).
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int E = 4;
    __device__ static float get(const float4& v, int e)
    {
        return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
    }
    __device__ static float4 make(const float* x) { return make_float4(x[0], x[1], x[2], x[3]); }
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int E = 2;
    __device__ static double get(const double2& v, int e) { return e == 0 ? v.x : v.y; }
    __device__ static double2 make(const double* x) { return make_double2(x[0], x[1]); }
};

template <typename T, int NB>
__device__ __forceinline__ void store_row(T* dst, const T (&x)[NB])
{
    using V = Vec16<T>;
#pragma unroll
    for (int v = 0; v < NB / V::E; ++v)
        reinterpret_cast<typename V::type*>(dst)[v] = V::make(&x[v * V::E]);
}

template <typename T, int NB>
__device__ __forceinline__ void load_row(T (&x)[NB], const T* src)
{
    using V = Vec16<T>;
#pragma unroll
    for (int v = 0; v < NB / V::E; ++v) {
        const typename V::type t = reinterpret_cast<const typename V::type*>(src)[v];
#pragma unroll
        for (int e = 0; e < V::E; ++e) x[v * V::E + e] = V::get(t, e);
    }
}

__device__ __forceinline__ float recip_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip_rn(double x) { return __drcp_rn(x); }


// ---------------------------------------------------------------------
// Register panel, two rows per thread: 256 threads per CTA, each holding
// panel rows r0 + t and r0 + t + 256 in registers (16 CTAs: m <= 8192).  Per
// column a thread reads the pivot row's active part from shared memory once and
// updates both rows with it; with one row per thread (512 threads) those
// broadcast reads and the per-warp key reduction, candidate store and
// barrier work cost 5-7 % more per column (measured).
// ---------------------------------------------------------------------
constexpr int kReg2Threads = 256;
constexpr int kReg2Warps = kReg2Threads / 32;

// The rank-1 update of one column on both of a thread's rows: x[c] -= lx *
// ur[c] (when ux) and y[c] -= ly * ur[c] (when uy) for the positions this
// step updates, u < c < lim.  lim is a multiple of kRegBlock, so the vectors
// below it are whole and the finished columns above it are skipped with one
// uniform branch per vector; u < kRegBlock folds to a constant in the
// unrolled column loop, so the positions up to u in the first vector drop
// out at compile time.  Only those positions are touched, as in TMV, so a
// non-finite multiplier needs no separate path.  One shared-memory read of
// each pivot-row vector serves both rows.
template <typename T, int NB>
__device__ __forceinline__ void reg2_update(T (&x)[NB], T lx, bool ux, T (&y)[NB], T ly, bool uy,
                                            const T* __restrict__ ur, int u, int lim)
{
    using V = Vec16<T>;
    static_assert(V::E <= kRegBlock && kRegBlock % V::E == 0, "vectors within a block");
#pragma unroll
    for (int v = 0; v < NB / V::E; ++v) {
        if (v * V::E >= lim) break;
        const typename V::type uv = reinterpret_cast<const typename V::type*>(ur)[v];
        if constexpr (std::is_same<T, float>::value) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = 4 * v + 2 * h;
                const float2 up = h == 0 ? make_float2(uv.x, uv.y) : make_float2(uv.z, uv.w);
                if (c > u) {
                    if (ux) {
                        const float2 r = __ffma2_rn(make_float2(-lx, -lx), up, make_float2(x[c], x[c + 1]));
                        x[c] = r.x;
                        x[c + 1] = r.y;
                    }
                    if (uy) {
                        const float2 r = __ffma2_rn(make_float2(-ly, -ly), up, make_float2(y[c], y[c + 1]));
                        y[c] = r.x;
                        y[c + 1] = r.y;
                    }
                } else if (c + 1 > u) {
                    if (ux) x[c + 1] = fmaf(-lx, up.y, x[c + 1]);
                    if (uy) y[c + 1] = fmaf(-ly, up.y, y[c + 1]);
                }
            }
        } else {
#pragma unroll
            for (int e = 0; e < V::E; ++e) {
                const int c = v * V::E + e;
                if (c > u) {
                    if (ux) x[c] = fma(-lx, V::get(uv, e), x[c]);
                    if (uy) y[c] = fma(-ly, V::get(uv, e), y[c]);
                }
            }
        }
    }
}

template <typename T, int NB>
__global__ void __launch_bounds__(kReg2Threads, 1)
lu_panel_cluster_reg2_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int nb,
                             int64_t* __restrict__ P, const unsigned char* __restrict__ modes,
                             int rows_per_cta, int* pairs, int* err, float* __restrict__ ahi,
                             float* __restrict__ alo, const T* __restrict__ Sp, int64_t lds)
{
    // Sp: the panel's columns come from this scratch panel (row i, column c
    // at Sp[i + c lds]) instead of A
    static_assert(NB % kRegBlock == 0, "whole blocks");
    static_assert(NB * sizeof(T) == 256, "a row is 16 vectors of 16 bytes");
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ unsigned long long s_key[kReg2Warps];
    __shared__ int s_idx[kReg2Warps];
    __shared__ __align__(16) T warp_row[kReg2Warps][NB];  // each warp's candidate row
    // published for remote pulls, double-buffered by column parity
    __shared__ __align__(16) T pub_row[2][NB];   // this CTA's candidate row
    __shared__ __align__(16) T pub_diag[2][NB];  // row j, in the CTA that holds it
    __shared__ __align__(16) uint4 slot[2][kClusterCtas];  // records stored by every CTA
    __shared__ __align__(8) uint64_t mbar[2];
    // the column's outcome, handed from warp 0 to the block
    __shared__ __align__(16) T urow[NB];
    __shared__ __align__(16) T drow[NB];
    __shared__ unsigned long long s_wk;
    __shared__ int s_wi;
    __shared__ unsigned char s_mode[kPanelMax];
    __shared__ int s_piv[kPanelMax];
    __shared__ int s_abort;

    const int G = (int)cluster.num_blocks();
    const int cta = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // row indices within the panel fit an int (m <= 16 * 512)
    const int m = (int)(n - k);
    const int r0 = cta * rows_per_cta;
    const int nr = max(0, min(rows_per_cta, m - r0));
    const bool ha = tid < nr, hb = tid + kReg2Threads < nr;
    const int pa = r0 + tid, pb = r0 + tid + kReg2Threads;  // this thread's rows
    T* Ap = A + k + k * lda;

    if (tid == 0) {
        mbar_init(&mbar[0], (uint32_t)G);
        mbar_init(&mbar[1], (uint32_t)G);
        s_abort = 0;
        mbar_fence_init();
    }
    for (int j = tid; j < nb; j += kReg2Threads) s_mode[j] = modes[j];
    const T* Xp = Sp ? Sp : Ap;
    const int64_t ldx = Sp ? lds : lda;
    T x[NB], y[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        x[c] = (ha && c < nb) ? Xp[pa + c * ldx] : T(0);
        y[c] = (hb && c < nb) ? Xp[pb + c * ldx] : T(0);
    }
    cluster.sync();  // every CTA's mbarriers are initialised before any arrival

    bool prev_uf = false;
    int rot = 0;  // x[p], y[p] hold column (p + rot) mod NB
    for (int jb = 0; jb < nb; jb += kRegBlock) {
        const int lim = NB - jb;  // positions >= lim hold finished columns 0..jb-1
#pragma unroll
        for (int u = 0; u < kRegBlock; ++u) {
            const int jj = jb + u;
            if (jj >= nb) break;
            const int par = jj & 1;
            const bool r2 = s_mode[jj] && !prev_uf;
            const int owner_j = jj < rows_per_cta ? 0 : jj / rows_per_cta;
            // 1. this warp's candidate (the better of each thread's two rows,
            //    the lower row on a tie); its row, and row jj, into shared memory
            unsigned long long bk = 0;
            int bi = INT_MAX;
            if (ha && pa >= jj) {
                bk = reg_pivot_key(x[u], pa == jj, r2);
                bi = pa;
            }
            if (hb && pb >= jj) {
                const unsigned long long kb = reg_pivot_key(y[u], pb == jj, r2);
                if (bi == INT_MAX || kb > bk) {
                    bk = kb;
                    bi = pb;
                }
            }
            reg_key_reduce<T>(bk, bi);
            if (bi == pa) store_row<T, NB>(warp_row[warp], x);
            else if (bi == pb) store_row<T, NB>(warp_row[warp], y);
            if (lane == 0) { s_key[warp] = bk; s_idx[warp] = bi; }
            if (ha && pa == jj) store_row<T, NB>(pub_diag[par], x);
            else if (hb && pb == jj) store_row<T, NB>(pub_diag[par], y);
            __syncthreads();
            if (warp == 0) {
                // 2. this CTA's candidate
                bk = lane < kReg2Warps ? s_key[lane] : 0ull;
                bi = lane < kReg2Warps ? s_idx[lane] : INT_MAX;
                reg_key_reduce<T>(bk, bi);
                if (G == 1) {
                    // one CTA: its candidate is the pivot, taken without the
                    // cluster exchange
                    if (lane == 0) { s_wk = bk; s_wi = bi; }
                    if (!reg_key_underflows<T>(bk)) {
                        if (lane < 16)
                            reinterpret_cast<uint4*>(urow)[lane] = reinterpret_cast<const uint4*>(
                                warp_row[((bi - r0) & (kReg2Threads - 1)) >> 5])[lane];
                        else if (bi != jj)
                            reinterpret_cast<uint4*>(drow)[lane - 16] =
                                reinterpret_cast<const uint4*>(pub_diag[par])[lane - 16];
                    }
                } else {
                    // publish it, store its record into every CTA and arrive
                    // there (release)
                    if (bi != INT_MAX && lane < 16)
                        reinterpret_cast<uint4*>(pub_row[par])[lane] =
                            reinterpret_cast<const uint4*>(warp_row[((bi - r0) & (kReg2Threads - 1)) >> 5])[lane];
                    __syncwarp();
                    if (lane < G) {
                        st_cluster16(cluster_addr(&slot[par][cta], lane),
                                     make_uint4((unsigned)bk, (unsigned)(bk >> 32), (unsigned)bi, 0u));
                        mbar_arrive_remote_release(cluster_addr(&mbar[par], lane));
                    }
                    // 3. wait for every CTA's record (bounded), reduce, pull rows
                    const bool got = __all_sync(0xffffffffu, mbar_wait_cluster(&mbar[par], (uint32_t)((jj >> 1) & 1)));
                    if (!got) {
                        if (lane == 0) {
                            s_abort = 1;
                            atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                        }
                    } else {
                        const uint4 mt = lane < G ? slot[par][lane] : make_uint4(0u, 0u, (unsigned)INT_MAX, 0u);
                        unsigned long long wk = ((unsigned long long)mt.y << 32) | mt.x;
                        int wi = (int)mt.z;
                        reg_key_reduce<T>(wk, wi);
                        if (lane == 0) { s_wk = wk; s_wi = wi; }
                        if (!reg_key_underflows<T>(wk)) {
                            // the winning record's lane is the CTA that holds row wi
                            const int owner_w = __ffs(__ballot_sync(0xffffffffu, lane < G && (int)mt.z == wi)) - 1;
                            if (lane < 16)
                                reinterpret_cast<uint4*>(urow)[lane] =
                                    ld_cluster16(cluster_addr(&pub_row[par][0], owner_w) + 16 * lane);
                            else if (cta == owner_w && wi != jj)
                                reinterpret_cast<uint4*>(drow)[lane - 16] =
                                    ld_cluster16(cluster_addr(&pub_diag[par][0], owner_j) + 16 * (lane - 16));
                        }
                    }
                }
            }
            __syncthreads();
            if (s_abort) break;
            const unsigned long long wk = s_wk;
            const int wi = s_wi;
            if (reg_key_underflows<T>(wk)) {
                if (tid == 0) s_piv[jj] = (int)(k + jj);
                if (ha && pa >= jj) x[u] = T(0);
                if (hb && pb >= jj) y[u] = T(0);
                prev_uf = true;
                continue;
            }
            prev_uf = false;
            if (tid == 0) s_piv[jj] = (int)(k + wi);
            // the interchange: row jj takes the pivot row, row wi the old row jj
            if (ha && pa == jj) load_row<T, NB>(x, urow);
            else if (ha && pa == wi) load_row<T, NB>(x, drow);
            if (hb && pb == jj) load_row<T, NB>(y, urow);
            else if (hb && pb == wi) load_row<T, NB>(y, drow);
            // TMV scales the column by the reciprocal of the pivot
            const T rp = recip_rn(urow[u]);
            const bool ux = ha && pa > jj, uy = hb && pb > jj;
            const T lx = x[u] * rp, ly = y[u] * rp;
            if (ux) x[u] = lx;
            if (uy) y[u] = ly;
            reg2_update<T, NB>(x, lx, ux, y, ly, uy, urow, u, lim);
        }
        if (s_abort) break;
        if (jb + kRegBlock < nb) {
            T t[kRegBlock], t2[kRegBlock];
#pragma unroll
            for (int c = 0; c < kRegBlock; ++c) {
                t[c] = x[c];
                t2[c] = y[c];
            }
#pragma unroll
            for (int c = 0; c < NB - kRegBlock; ++c) {
                x[c] = x[c + kRegBlock];
                y[c] = y[c + kRegBlock];
            }
#pragma unroll
            for (int c = 0; c < kRegBlock; ++c) {
                x[NB - kRegBlock + c] = t[c];
                y[NB - kRegBlock + c] = t2[c];
            }
            rot += kRegBlock;
        }
    }

    if (!s_abort) {
        // with ahi (FP32 factorisation) the rows below the panel block are
        // also written as the TF32 hi/lo split of L21 (row-major, nb wide)
        // that the step's tensor-core update reads
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const bool have = h == 0 ? ha : hb;
            const int pr = h == 0 ? pa : pb;
            if (!have) continue;
            const bool split = std::is_same<T, float>::value && ahi != nullptr && pr >= nb;
#pragma unroll
            for (int p = 0; p < NB; ++p) {
                const int col = (p + rot) % NB;
                if (col < nb) {
                    const T v = h == 0 ? x[p] : y[p];
                    Ap[pr + col * lda] = v;
                    if (split) {
                        const float f = (float)v;
                        const float hi = tf32_round(f);
                        ahi[(int64_t)(pr - nb) * nb + col] = hi;
                        alo[(int64_t)(pr - nb) * nb + col] = tf32_round(f - hi);
                    }
                }
            }
        }
        __syncthreads();
        if (cta == 0) {
            for (int j = tid; j < nb; j += kReg2Threads) P[k + j] = s_piv[j];
            if (warp == 0) panel_row_pairs(k, nb, s_piv, pairs);
        }
    }
    cluster.sync();  // no CTA leaves while another may still store into it
}

// ---------------------------------------------------------------------
// Register panel with leaves: the same cluster, row partition and pivot rule
// as lu_panel_cluster_reg2_kernel, and bitwise the same factors, organised
// so that a column's critical chain carries only what the next pivot
// decision needs; everything else runs in the shadow of the cluster
// exchange, while warp 0 waits for the other CTAs.
//
// * One panel row per thread, 512 threads per CTA (16 CTAs: m <= 8192).
// * Columns are factored in leaves of kLeaf = 8; the step loop is not
//   unrolled (every column runs the same instructions: a large unrolled body
//   misses in the instruction cache), and the leaf's eight registers rotate
//   by one position per step so that column j is always x[0].  After a pivot
//   decision a thread scales its row's column j and updates column j+1 (the next key);
//   the rest of the step's rank-1 update on the leaf is owed and paid in the
//   next column's shadow.  A leaf's effect on the later columns is a rank-8
//   update A2 -= L1 U12 at the end of the leaf, with U12 = L11^-1 A12 solved
//   from the leaf's pivot rows.  Every entry still receives TMV's
//   subtractions in TMV's order, one fused multiply-add each.
// * Rows never move: each thread tracks its row's current position; an
//   interchange swaps two positions, a pivot row is marked done, and rows
//   are written to their final positions at the end.  Ties go to the lowest
//   position, the NaN rule looks at the element at position j.
// * The exchange of a column is one message per CTA and destination (key,
//   position, location and the candidate row's leaf part) stored with
//   st.async, whose arrival completes the receiver's mbarrier; every CTA
//   reduces the 16 messages itself.
// * A pivot row's other columns are needed only at the end of its leaf: its
//   owner stages them in shared memory and bulk-copies them to every CTA in
//   the next column's shadow.
// Bounded waits as in lu_panel_cluster_reg2_kernel.
// ---------------------------------------------------------------------
constexpr int kLeaf = 8;
constexpr int kLeafThreads = 512;
constexpr int kLeafWarps = kLeafThreads / 32;

template <typename T>
struct LeafMsg {
    unsigned long long key;
    int pos;
    int loc;  // cta << 16 | thread
    T leaf[kLeaf];
};

template <typename T, int NB>
__device__ __forceinline__ void leaf_stage_row(T* __restrict__ dst, const T (&x)[NB], int pw)
{
    using V = Vec16<T>;
#pragma unroll
    for (int v = 0; v < NB / V::E; ++v) {
        if (v * V::E >= pw) break;
        reinterpret_cast<typename V::type*>(dst)[v] = V::make(&x[v * V::E]);
    }
}

// Rank-8 update of positions [kLeaf, pend) of a row: x[p] -= x[LP + t] *
// U[t][p + SHIFT] for the leaf's steps t in order (steps whose column
// underflowed did no update and are skipped).
template <typename T, int NB, int LP, int SHIFT, int PMAX>
__device__ __forceinline__ void leaf_rank8(T (&x)[NB], const T* __restrict__ U, unsigned ufmask, int pend)
{
    using V = Vec16<T>;
#pragma unroll
    for (int v = kLeaf / V::E; v < PMAX / V::E; ++v) {
        const int p = v * V::E;
        if (p >= pend) break;
#pragma unroll
        for (int t = 0; t < kLeaf; ++t) {
            if ((ufmask >> t) & 1u) continue;
            const T l = x[LP + t];
            const typename V::type uv = *reinterpret_cast<const typename V::type*>(U + t * NB + p + SHIFT);
            if constexpr (std::is_same<T, float>::value) {
                const float2 a = __ffma2_rn(make_float2(-l, -l), make_float2(uv.x, uv.y), make_float2(x[p], x[p + 1]));
                const float2 b = __ffma2_rn(make_float2(-l, -l), make_float2(uv.z, uv.w), make_float2(x[p + 2], x[p + 3]));
                x[p] = a.x;
                x[p + 1] = a.y;
                x[p + 2] = b.x;
                x[p + 3] = b.y;
            } else {
                x[p] = fma(-l, uv.x, x[p]);
                x[p + 1] = fma(-l, uv.y, x[p + 1]);
            }
        }
    }
}

// Positions [kLeaf, pend) of a row that became a pivot row in the leaf take
// their final (U) values.
template <typename T, int NB>
__device__ __forceinline__ void leaf_take_u(T (&x)[NB], const T* __restrict__ ut, int pend)
{
    using V = Vec16<T>;
#pragma unroll
    for (int v = kLeaf / V::E; v < NB / V::E; ++v) {
        const int p = v * V::E;
        if (p >= pend) break;
        const typename V::type uv = reinterpret_cast<const typename V::type*>(ut)[v];
#pragma unroll
        for (int e = 0; e < V::E; ++e) x[p + e] = V::get(uv, e);
    }
}

template <typename T, int NB>
__device__ __forceinline__ void leaf_rotate(T (&x)[NB])
{
    T t[kLeaf];
#pragma unroll
    for (int c = 0; c < kLeaf; ++c) t[c] = x[c];
#pragma unroll
    for (int c = 0; c < NB - kLeaf; ++c) x[c] = x[c + kLeaf];
#pragma unroll
    for (int c = 0; c < kLeaf; ++c) x[NB - kLeaf + c] = t[c];
}

// The leaf part by one position: x[q] <- x[q + 1], x[kLeaf - 1] <- x[0].
template <typename T, int NB>
__device__ __forceinline__ void leaf_rotate1(T (&x)[NB])
{
    const T t = x[0];
#pragma unroll
    for (int q = 0; q < kLeaf - 1; ++q) x[q] = x[q + 1];
    x[kLeaf - 1] = t;
}

// A pivot row's columns [0, pw) into every CTA's receive buffer `dst_row`
// (one CTA: written there directly); its leaf part is rotated by `rot`
// (position q holds leaf column (rot + q) mod kLeaf).
template <typename T, int NB>
__device__ __forceinline__ void leaf_send_row(const T (&x)[NB], int rot, int pw, int G, T* stage, T* dst_row,
                                              uint64_t* bar)
{
    T* buf = G == 1 ? dst_row : stage;
#pragma unroll
    for (int q = 0; q < kLeaf; ++q) buf[(rot + q) & (kLeaf - 1)] = x[q];
    using V = Vec16<T>;
#pragma unroll
    for (int v = kLeaf / V::E; v < NB / V::E; ++v) {
        if (v * V::E >= pw) break;
        reinterpret_cast<typename V::type*>(buf)[v] = V::make(&x[v * V::E]);
    }
    if (G == 1) return;
    fence_proxy_async_smem();
    for (int d = 0; d < G; ++d)
        bulk_s2cluster(cluster_addr(dst_row, d), stage, (uint32_t)(pw * sizeof(T)), cluster_addr(bar, d));
}

template <typename T, int NB>
__global__ void __launch_bounds__(kLeafThreads, 1)
lu_panel_leaf_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int nb,
                     int64_t* __restrict__ P, const unsigned char* __restrict__ modes,
                     int rows_per_cta, int* pairs, int* err, float* __restrict__ ahi,
                     float* __restrict__ alo, const T* __restrict__ Sp, int64_t lds)
{
    static_assert(NB % kLeaf == 0 && NB >= 2 * kLeaf, "whole leaves");
    static_assert(NB * sizeof(T) == 256, "a row is 16 vectors of 16 bytes");
    using V = Vec16<T>;
    constexpr int kMsgVecs = (int)(sizeof(LeafMsg<T>) / 16);
    static_assert(sizeof(LeafMsg<T>) % 16 == 0, "message in 16-byte pieces");
    constexpr int kLast = kLeaf - 1;
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();

    __shared__ unsigned long long s_key[kLeafWarps];
    __shared__ int s_idx[kLeafWarps];
    __shared__ int s_loc[kLeafWarps];
    __shared__ __align__(16) T warp_leaf[kLeafWarps][kLeaf];     // each warp's candidate's leaf part
    __shared__ __align__(16) LeafMsg<T> msg[2][kClusterCtas];   // messages, by column parity
    __shared__ __align__(16) T s_urow[kLeaf][kLeaf];             // the leaf's pivot rows, leaf part
    __shared__ __align__(16) T s_rem[2][kLeaf][NB];              // pivot rows, then U (by leaf parity)
    __shared__ __align__(16) T s_stage[kLeaf][NB];               // this CTA's pivot rows, staged
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ __align__(8) uint64_t mbar_leaf;
    __shared__ unsigned long long s_wk;
    __shared__ int s_wi, s_wloc;
    __shared__ unsigned char s_mode[kPanelMax];
    __shared__ int s_piv[kPanelMax];
    __shared__ int s_npairs;  // row pairs written so far (used in CTA 0)
    __shared__ int s_abort;

    const int G = (int)cluster.num_blocks();
    const int cta = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m = (int)(n - k);
    const int r0 = cta * rows_per_cta;
    const int nr = max(0, min(rows_per_cta, m - r0));
    const bool have = tid < nr;
    T* Ap = A + k + k * lda;

    if (tid == 0) {
        mbar_init(&mbar[0], 1u);
        mbar_init(&mbar[1], 1u);
        mbar_init(&mbar_leaf, 1u);
        s_abort = 0;
        s_npairs = 0;
        mbar_fence_init();
    }
    for (int j = tid; j < nb; j += kLeafThreads) s_mode[j] = modes[j];
    const T* Xp = Sp ? Sp : Ap;
    const int64_t ldx = Sp ? lds : lda;
    T x[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) x[c] = (have && c < nb) ? Xp[r0 + tid + c * ldx] : T(0);
    int pos = r0 + tid;  // this row's current position
    bool act = have;     // still a candidate (not yet a pivot row)
    const int loc = (cta << 16) | tid;
    cluster.sync();  // every CTA's mbarriers are initialised before any message

    bool prev_uf = false;
    unsigned leaf_uses = 0;
    for (int jb = 0, leaf = 0; jb < nb; jb += kLeaf, ++leaf) {
        const int lpar = leaf & 1;
        const int steps = min(kLeaf, nb - jb);
        const int rc = max(0, nb - jb - kLeaf);          // columns after the leaf still to factor
        const int rcv = (rc + V::E - 1) / V::E * V::E;   // in whole vectors
        const int pw = kLeaf + rcv;                      // positions a pivot row sends
        const bool block = rc > 0;
        if (block && G > 1 && tid == 0)
            mbar_expect_tx(&mbar_leaf, (uint32_t)(steps * pw * (int)sizeof(T)));
        int dstep = -1;       // leaf step at which this row became a pivot row
        int send_step = -1;   // this thread's pivot row, not yet sent
        unsigned ufmask = 0;
        T lprev = T(0);       // the previous step's multiplier, owed on positions > step + 1
        bool owe = false;
#pragma unroll 1
        for (int u = 0; u < steps; ++u) {
            // the leaf's registers are rotated one position per step:
            // position q holds column (u + q) mod kLeaf of the leaf
            const int j = jb + u;
            const int par = j & 1;
            const bool r2 = s_mode[j] && !prev_uf;
            // 1. this warp's candidate; the winner's leaf part with the owed update applied
            unsigned long long bk = act ? reg_pivot_key(x[0], pos == j, r2) : 0ull;
            int bi = act ? pos : INT_MAX;
            reg_key_reduce<T>(bk, bi);
            if (act && pos == bi) {
                // (in position order; positions 1..7-u owe step u-1's update,
                // whose pivot row s_urow[u-1] is in step u-1's position order)
                T lp[kLeaf];
#pragma unroll
                for (int q = 0; q < kLeaf; ++q)
                    lp[q] = (owe && q >= 1 && q <= kLast - u) ? fma(-lprev, s_urow[u - 1][q + 1 < kLeaf ? q + 1 : q], x[q]) : x[q];
#pragma unroll
                for (int q = 0; q < kLeaf / V::E; ++q)
                    reinterpret_cast<typename V::type*>(warp_leaf[warp])[q] = V::make(&lp[q * V::E]);
                s_loc[warp] = loc;
            }
            if (lane == 0) {
                s_key[warp] = bk;
                s_idx[warp] = bi;
            }
            __syncthreads();
            if (warp == 0) {
                // 2. this CTA's candidate; with a cluster, one message into every CTA
                bk = lane < kLeafWarps ? s_key[lane] : 0ull;
                bi = lane < kLeafWarps ? s_idx[lane] : INT_MAX;
                reg_key_reduce<T>(bk, bi);
                const unsigned wm = __ballot_sync(0xffffffffu, lane < kLeafWarps && bi != INT_MAX && s_idx[lane] == bi);
                const int ww = wm ? __ffs(wm) - 1 : -1;
                if (G == 1) {
                    if (lane == 0) {
                        s_wk = bk;
                        s_wi = bi;
                        s_wloc = ww >= 0 ? s_loc[ww] : -1;
                    }
                    if (ww >= 0 && lane < kLeaf / V::E)
                        reinterpret_cast<typename V::type*>(s_urow[u])[lane] =
                            reinterpret_cast<const typename V::type*>(warp_leaf[ww])[lane];
                } else {
                    if (lane == 0) mbar_expect_tx(&mbar[par], (uint32_t)(G * sizeof(LeafMsg<T>)));
                    if (lane < G) {
                        const uint32_t dst = cluster_addr(&msg[par][cta], lane);
                        const uint32_t bar = cluster_addr(&mbar[par], lane);
                        const int wl = ww >= 0 ? s_loc[ww] : -1;
                        st_async16(dst, make_uint4((unsigned)bk, (unsigned)(bk >> 32), (unsigned)bi, (unsigned)wl), bar);
#pragma unroll
                        for (int q = 1; q < kMsgVecs; ++q) {
                            const uint4 v = ww >= 0 ? reinterpret_cast<const uint4*>(warp_leaf[ww])[q - 1]
                                                    : make_uint4(0u, 0u, 0u, 0u);
                            st_async16(dst + 16 * q, v, bar);
                        }
                    }
                }
            }
            // 3. the shadow: work this row owes, while the messages travel
            if (owe) {
#pragma unroll
                for (int q = 1; q < kLeaf; ++q)
                    if (q <= kLast - u) x[q] = fma(-lprev, s_urow[u - 1][q + 1 < kLeaf ? q + 1 : q], x[q]);
            }
            owe = false;
            if (send_step >= 0) {
                leaf_send_row<T, NB>(x, u, pw, G, s_stage[send_step], s_rem[lpar][send_step], &mbar_leaf);
                send_step = -1;
            }
            if (warp == 0 && G > 1) {
                // 4. every CTA's message (bounded wait), reduced here
                const bool got = __all_sync(0xffffffffu, mbar_wait(&mbar[par], (uint32_t)((j >> 1) & 1)));
                if (!got) {
                    if (lane == 0) {
                        s_abort = 1;
                        atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                    }
                } else {
                    unsigned long long wk = lane < G ? msg[par][lane].key : 0ull;
                    int wi = lane < G ? msg[par][lane].pos : INT_MAX;
                    reg_key_reduce<T>(wk, wi);
                    const unsigned om = __ballot_sync(0xffffffffu, lane < G && wi != INT_MAX && msg[par][lane].pos == wi);
                    const int wo = om ? __ffs(om) - 1 : -1;
                    if (lane == 0) {
                        s_wk = wk;
                        s_wi = wi;
                        s_wloc = wo >= 0 ? msg[par][wo].loc : -1;
                    }
                    if (wo >= 0 && lane < kLeaf / V::E)
                        reinterpret_cast<typename V::type*>(s_urow[u])[lane] =
                            reinterpret_cast<const typename V::type*>(msg[par][wo].leaf)[lane];
                }
            }
            __syncthreads();
            if (s_abort) break;
            // 5. the decision: bookkeeping, the column's scaling and the next column
            const bool uf = reg_key_underflows<T>(s_wk);
            bool own;
            if (uf) {
                own = act && pos == j;
                if (act) x[0] = T(0);
                if (tid == 0) s_piv[j] = (int)(k + j);
                ufmask |= 1u << u;
                prev_uf = true;
            } else {
                const int wi = s_wi;
                own = act && loc == s_wloc;
                if (tid == 0) s_piv[j] = (int)(k + wi);
                prev_uf = false;
                if (act && !own && pos == j) pos = wi;  // the interchange
            }
            if (own) {
                act = false;
                pos = j;
                dstep = u;
                if (block) send_step = u;
            }
            if (!uf && act) {
                // TMV scales the column by the reciprocal of the pivot
                const T l = x[0] * recip_rn(s_urow[u][0]);
                x[0] = l;
                if (u < kLast) x[1] = fma(-l, s_urow[u][1], x[1]);
                if (u + 2 < kLeaf) {
                    lprev = l;
                    owe = true;
                }
            }
            leaf_rotate1<T, NB>(x);
        }
        if (s_abort) break;
        for (int r = steps; r < kLeaf; ++r) leaf_rotate1<T, NB>(x);  // back to column order
        if (block) {
            // 6. the leaf's end: the last pivot row out, the leaf's U12 (every
            //    CTA the same), the rank-8 update of the columns after the
            //    leaf, and the final values of the leaf's pivot rows
            if (send_step >= 0) {
                leaf_send_row<T, NB>(x, 0, pw, G, s_stage[send_step], s_rem[lpar][send_step], &mbar_leaf);
                send_step = -1;
            }
            if (G > 1) {
                if (!mbar_wait(&mbar_leaf, leaf_uses & 1u)) {
                    if (tid == 0) atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                    s_abort = 1;  // every thread of the CTA reaches this
                }
                ++leaf_uses;
            }
            __syncthreads();
            if (s_abort) break;
            T(*Ur)[NB] = s_rem[lpar];
            for (int p = kLeaf + tid; p < pw; p += kLeafThreads) {
                T uc[kLeaf];
#pragma unroll
                for (int t = 0; t < kLeaf; ++t) uc[t] = Ur[t][p];
#pragma unroll
                for (int t = 1; t < kLeaf; ++t) {
#pragma unroll
                    for (int q = 0; q < t; ++q)
                        if (!((ufmask >> q) & 1u)) uc[t] = fma(-Ur[t][q], uc[q], uc[t]);
                }
#pragma unroll
                for (int t = 0; t < kLeaf; ++t) Ur[t][p] = uc[t];
            }
            __syncthreads();
            if (act) leaf_rank8<T, NB, 0, 0, NB>(x, &Ur[0][0], ufmask, pw);
            else if (dstep >= 0) leaf_take_u<T, NB>(x, Ur[dstep], pw);
        }
        if (jb + kLeaf < nb) leaf_rotate<T, NB>(x);
    }

    if (!s_abort) {
        // rows to their final positions (the TF32 split of L21 that the
        // tensor-core update reads is made by its own kernel; ahi and alo are
        // not written here)
        const int rot = ((nb - 1) / kLeaf) * kLeaf;  // x[p] holds column (p + rot) mod NB
        if (have) {
#pragma unroll
            for (int p = 0; p < NB; ++p) {
                const int col = (p + rot) % NB;
                if (col < nb) Ap[pos + col * lda] = x[p];
            }
            // the interchanges as a row gather: a row that moved is one pair,
            // "row k + pos receives the old row k + r0 + tid" (slots handed
            // out by a counter in CTA 0's shared memory; consumers read the
            // pairs as a set)
            if (pos != r0 + tid) {
                int* cnt = cluster.map_shared_rank(&s_npairs, 0);
                const int q = atomicAdd(cnt, 1);
                pairs[1 + q] = (int)(k + pos);
                pairs[1 + kMaxPairs + q] = (int)(k + r0 + tid);
            }
        }
        if (cta == 0)
            for (int j = tid; j < nb; j += kLeafThreads) P[k + j] = s_piv[j];
    }
    cluster.sync();  // no CTA leaves while another may still store into it
    if (cta == 0 && tid == 0 && !s_abort) pairs[0] = s_npairs;
}

// ---------------------------------------------------------------------
// Row interchanges.
// ---------------------------------------------------------------------
// Interchanges P[k..k+nb) applied to columns [0, ncols) except [skip0, skip1).
template <typename T>
__global__ void laswp_kernel(T* __restrict__ A, int64_t lda, int64_t ncols, int64_t k, int nb,
                             const int64_t* __restrict__ P, int64_t skip0, int64_t skip1)
{
    __shared__ int64_t sp[kPanelMax];
    for (int t = threadIdx.x; t < nb; t += blockDim.x) sp[t] = P[k + t];
    __syncthreads();
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= ncols || (c >= skip0 && c < skip1)) return;
    T* col = A + c * lda;
    for (int t = 0; t < nb; ++t) {
        const int64_t i = k + t, p = sp[t];
        if (p != i) {
            const T a = col[i];
            col[i] = col[p];
            col[p] = a;
        }
    }
}

// The panel's row pairs applied to columns [0, ncols) outside [skip0, skip1):
// one warp per column loads every source value, then stores them.
template <typename T>
__global__ void laswp_pairs_kernel(T* __restrict__ A, int64_t lda, int64_t ncols, int64_t skip0,
                                   int64_t skip1, const int* __restrict__ pairs)
{
    const int lane = threadIdx.x & 31;
    const int64_t col = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    if (col >= ncols || (col >= skip0 && col < skip1)) return;
    const int np = pairs[0];
    const int* dst = pairs + 1;
    const int* src = pairs + 1 + kMaxPairs;
    T* a = A + col * lda;
    T v[kMaxPairs / 32];
#pragma unroll
    for (int t = 0; t < kMaxPairs / 32; ++t) {
        const int q = lane + 32 * t;
        if (q < np) v[t] = a[src[q]];
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < kMaxPairs / 32; ++t) {
        const int q = lane + 32 * t;
        if (q < np) a[dst[q]] = v[t];
    }
}

// U12 = L11^-1 A12 for a panel: each CTA solves 64 columns of A12 in shared
// memory, all threads sweeping the rows together (one barrier per row of
// L11), instead of one thread per column.
constexpr int kU12Cols = 64;
template <typename T>
__global__ void __launch_bounds__(256)
panel_u12_kernel(int nb, const T* __restrict__ L, int64_t lda, T* __restrict__ A12, int64_t ncols)
{
    extern __shared__ __align__(16) unsigned char u12_smem[];
    T* Ls = reinterpret_cast<T*>(u12_smem);  // [nb][nb+1]
    T* X = Ls + nb * (nb + 1);               // [nb][kU12Cols+1]
    const int tid = threadIdx.x;
    const int64_t c0 = (int64_t)blockIdx.x * kU12Cols;
    const int nc = (int)min((int64_t)kU12Cols, ncols - c0);
    for (int t = tid; t < nb * nb; t += 256) {
        const int i = t % nb, j = t / nb;
        Ls[i * (nb + 1) + j] = j < i ? L[i + j * lda] : T(0);
    }
    for (int t = tid; t < nb * nc; t += 256) {
        const int i = t % nb, c = t / nb;
        X[i * (kU12Cols + 1) + c] = A12[i + (c0 + c) * lda];
    }
    __syncthreads();
    for (int j = 0; j < nb - 1; ++j) {
        const int rowsleft = nb - 1 - j;
        for (int t = tid; t < rowsleft * nc; t += 256) {
            const int i = j + 1 + t % rowsleft, c = t / rowsleft;
            X[i * (kU12Cols + 1) + c] -= Ls[i * (nb + 1) + j] * X[j * (kU12Cols + 1) + c];
        }
        __syncthreads();
    }
    for (int t = tid; t < nb * nc; t += 256) {
        const int i = t % nb, c = t / nb;
        A12[i + (c0 + c) * lda] = X[i * (kU12Cols + 1) + c];
    }
}

// ---------------------------------------------------------------------
// U12 = L11^-1 A12 with one column per thread held in registers.
//
// L11 (unit lower, nb <= NB) is staged transposed in shared memory so that the
// multipliers of column j are read as 16-byte broadcast vectors; a CTA's
// columns of A12 are staged through shared memory so that global reads and
// writes stay coalesced.  Each column's substitution runs in the same order
// as the scalar kernel (j ascending), so results are bitwise the same.  With
// SPLIT the kernel also writes the TF32 hi/lo split of U12 (column-major,
// leading dimension nb) for the tensor-core trailing update.
// ---------------------------------------------------------------------
constexpr int kU12RegThreads = 64;   // columns per CTA (wide launches), one per computing thread
constexpr int kU12NarrowCols = 8;    // columns per CTA when only a panel's width is solved
constexpr int kU12RegBlock = 256;    // threads per CTA: all of them stage, COLS compute

template <typename T, int NB, bool SPLIT, int COLS>
__global__ void __launch_bounds__(kU12RegBlock)
u12_reg_kernel(int nb, const T* __restrict__ L, int64_t lda, T* __restrict__ A12, int64_t ncols,
               float* __restrict__ Bhi, float* __restrict__ Blo, const int* __restrict__ pairs, int64_t k)
{
    using V = Vec16<T>;
    constexpr int XP = NB + V::E;  // padded staging row: conflict-free vector access
    __shared__ __align__(16) T LsT[NB][NB];  // LsT[j][i] = L(i, j) for i > j, else 0
    __shared__ __align__(16) T Xs[COLS][XP];
    const int tid = threadIdx.x;
    const int64_t c0 = (int64_t)blockIdx.x * COLS;

    if (pairs) {
        // the step's row interchanges on this CTA's columns first (over all
        // rows: a warp per column, a lane per row pair; A12 - k is row 0)
        const int lane = tid & 31, w = tid >> 5;
        const int np = pairs[0];
        const int* dst = pairs + 1;
        const int* src = pairs + 1 + kMaxPairs;
        for (int cc = w; cc < COLS; cc += kU12RegBlock / 32) {
            if (c0 + cc >= ncols) break;
            T* a = A12 - k + (c0 + cc) * lda;
            T v[kMaxPairs / 32];
#pragma unroll
            for (int t = 0; t < kMaxPairs / 32; ++t) {
                const int q = lane + 32 * t;
                if (q < np) v[t] = a[src[q]];
            }
            __syncwarp();
#pragma unroll
            for (int t = 0; t < kMaxPairs / 32; ++t) {
                const int q = lane + 32 * t;
                if (q < np) a[dst[q]] = v[t];
            }
        }
        __syncthreads();
    }

    // stage L11 and this CTA's columns, eight independent loads in flight
    constexpr int LU = 8;
    for (int t0 = tid; t0 < NB * NB; t0 += kU12RegBlock * LU) {
        T v[LU];
#pragma unroll
        for (int q = 0; q < LU; ++q) {
            const int t = t0 + q * kU12RegBlock;
            const int i = t % NB, j = t / NB;
            v[q] = (t < NB * NB && i < nb && j < nb && i > j) ? L[i + (int64_t)j * lda] : T(0);
        }
#pragma unroll
        for (int q = 0; q < LU; ++q) {
            const int t = t0 + q * kU12RegBlock;
            if (t < NB * NB) LsT[t / NB][t % NB] = v[q];
        }
    }
    for (int t0 = tid; t0 < COLS * NB; t0 += kU12RegBlock * LU) {
        T v[LU];
#pragma unroll
        for (int q = 0; q < LU; ++q) {
            const int t = t0 + q * kU12RegBlock;
            const int i = t % NB, c = t / NB;
            v[q] = (t < COLS * NB && i < nb && c0 + c < ncols) ? A12[i + (c0 + c) * lda] : T(0);
        }
#pragma unroll
        for (int q = 0; q < LU; ++q) {
            const int t = t0 + q * kU12RegBlock;
            if (t < COLS * NB) Xs[t / NB][t % NB] = v[q];
        }
    }
    __syncthreads();

    if (tid < COLS) {
    T x[NB];
    load_row<T, NB>(x, Xs[tid]);
#pragma unroll
    for (int j = 0; j < NB - 1; ++j) {
#pragma unroll
        for (int v = (j + 1) / V::E; v < NB / V::E; ++v) {
            const typename V::type lv = reinterpret_cast<const typename V::type*>(LsT[j])[v];
#pragma unroll
            for (int e = 0; e < V::E; ++e) {
                const int i = v * V::E + e;
                if (i > j) x[i] -= V::get(lv, e) * x[j];
            }
        }
    }
    store_row<T, NB>(Xs[tid], x);
    }
    __syncthreads();

    for (int t0 = tid; t0 < COLS * NB; t0 += kU12RegBlock) {
        const int i = t0 % NB, c = t0 / NB;
        if (i < nb && c0 + c < ncols) {
            const T val = Xs[c][i];
            A12[i + (c0 + c) * lda] = val;
            if constexpr (SPLIT) {
                const float h = tf32_round((float)val);
                Bhi[(c0 + c) * nb + i] = h;
                Blo[(c0 + c) * nb + i] = tf32_round((float)val - h);
            }
        }
    }
}

// ---------------------------------------------------------------------
// FP32 register path: the update of the next panel's columns [c0, c0+nc)
// with step k (the "narrow" update on the chain between two panels) in one
// kernel, out of place.  Each CTA takes kNarrowRows trailing rows:
//   1. the step's row pairs give every row its source row (row r of the new
//      columns is old row src(r));
//   2. U12 = L11^-1 A12' for the gathered block rows k..k+63, solved in the
//      CTA (64 threads, one column each, L11 transposed in shared memory;
//      every CTA solves the same small block, which costs no more time than
//      one);
//   3. its rows: S = A(src(r), c0..) - L21(r, :) U12, FP32 FMAs (kNarrowRows/32
//      rows x 8 columns per thread).
// CTA 0 also writes U12.  The results go to the scratch panel S (row r at
// S[(r - k) + c lds]) and not into A, because a row's source may be a row
// another CTA overwrites; the next panel kernel reads its columns from S,
// and U12 is copied into A on the main stream, off the chain.
// ---------------------------------------------------------------------
constexpr int kNarrowRows = 64;
constexpr int kNarrowThreads = 256;
constexpr int kNarrowNB = 64;  // the step's width: the FP32 register panel's
constexpr int kNarrowXP = kNarrowNB + 4;
constexpr size_t kNarrowSmem =
    sizeof(float) * ((size_t)kNarrowNB * kNarrowNB + (size_t)kNarrowNB * kNarrowXP + (size_t)kNarrowRows * (kNarrowNB + 1));

__global__ void __launch_bounds__(kNarrowThreads)
narrow_update_f32_kernel(const float* __restrict__ A, int64_t lda, int64_t n, int64_t k, int64_t c0, int nc,
                         const int* __restrict__ pairs, float* __restrict__ S, int64_t lds)
{
    constexpr int NB = kNarrowNB, XP = kNarrowXP;
    using V = Vec16<float>;
    extern __shared__ __align__(16) float nsm[];
    float (*LsT)[NB] = reinterpret_cast<float (*)[NB]>(nsm);          // LsT[j][i] = L(i, j), i > j
    float (*Us)[XP] = reinterpret_cast<float (*)[XP]>(nsm + NB * NB);  // Us[c][i]: column c of A12'
    float (*UT)[XP] = Us;                                              // then UT[t][c] = U12(t, c)
    float (*Ls)[NB + 1] = reinterpret_cast<float (*)[NB + 1]>(nsm + NB * NB + NB * XP);  // this CTA's L21 rows
    __shared__ int s_dst[2 * NB], s_src[2 * NB];
    __shared__ int map_blk[NB], map_row[kNarrowRows];
    const int tid = threadIdx.x;
    const int64_t r0 = k + NB + (int64_t)blockIdx.x * kNarrowRows;  // this CTA's first row
    const int R = (int)min((int64_t)kNarrowRows, n - r0);
    constexpr int RQ = kNarrowRows / 32;
    const int rg = tid & 31, cg = tid >> 5;  // outputs: rows rg + 32 q (q < RQ), columns 8 cg + e
    // loads that need no row map first (L11, this CTA's L21 rows), in flight
    // together with the pair list; every load of a batch is issued before
    // its values are stored
    {
        constexpr int QB = NB * NB / kNarrowThreads;           // 16
        constexpr int QL = kNarrowRows * NB / kNarrowThreads;  // 32
        float lv[QB], v[QL];
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int t = tid + q * kNarrowThreads;
            const int i = t % NB, j = t / NB;
            lv[q] = i > j ? A[(k + i) + (k + j) * lda] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < QL; ++q) {
            const int t = tid + q * kNarrowThreads;
            const int r = t % kNarrowRows, j = t / kNarrowRows;
            v[q] = r < R ? A[(r0 + r) + (k + j) * lda] : 0.f;
        }
        const int np = min(pairs[0], 2 * NB);
        if (tid < np) {
            s_dst[tid] = pairs[1 + tid];
            s_src[tid] = pairs[1 + kMaxPairs + tid];
        }
        if (tid < NB) map_blk[tid] = (int)(k + tid);
        if (tid < kNarrowRows) map_row[tid] = (int)(r0 + tid);
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int t = tid + q * kNarrowThreads;
            LsT[t / NB][t % NB] = lv[q];
        }
#pragma unroll
        for (int q = 0; q < QL; ++q) {
            const int t = tid + q * kNarrowThreads;
            Ls[t % kNarrowRows][t / kNarrowRows] = v[q];
        }
        __syncthreads();
        if (tid < np) {
            const int64_t d = s_dst[tid];
            if (d >= k && d < k + NB) map_blk[d - k] = s_src[tid];
            else if (d >= r0 && d < r0 + R) map_row[d - r0] = s_src[tid];
        }
        __syncthreads();
    }
    // the gathered A12' and this thread's outputs (their source rows)
    float acc[RQ][8];
    {
        constexpr int QB = NB * NB / kNarrowThreads;
        float uv[QB];
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int t = tid + q * kNarrowThreads;
            const int i = t % NB, j = t / NB;
            uv[q] = j < nc ? A[map_blk[i] + (c0 + j) * lda] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < RQ; ++q)
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int r = rg + 32 * q, cc = 8 * cg + e;
                acc[q][e] = (r < R && cc < nc) ? A[map_row[r] + (c0 + cc) * lda] : 0.f;
            }
#pragma unroll
        for (int q = 0; q < QB; ++q) {
            const int t = tid + q * kNarrowThreads;
            Us[t / NB][t % NB] = uv[q];
        }
    }
    __syncthreads();
    // U12 = L11^-1 A12', a column per thread; written transposed over the
    // staged columns once every solving thread has read its own
    float x[NB];
    if (tid < nc) load_row<float, NB>(x, Us[tid]);
    __syncthreads();
    if (tid < nc) {
#pragma unroll
        for (int j = 0; j < NB - 1; ++j) {
#pragma unroll
            for (int v = (j + 1) / V::E; v < NB / V::E; ++v) {
                const float4 lv = reinterpret_cast<const float4*>(LsT[j])[v];
#pragma unroll
                for (int e = 0; e < V::E; ++e) {
                    const int i = v * V::E + e;
                    if (i > j) x[i] -= V::get(lv, e) * x[j];
                }
            }
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) UT[i][tid] = x[i];
    } else if (tid < NB) {
#pragma unroll
        for (int i = 0; i < NB; ++i) UT[i][tid] = 0.f;
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        // U12 into the scratch panel's first rows (copied into A later)
        for (int t = tid; t < NB * nc; t += kNarrowThreads) {
            const int i = t % NB, j = t / NB;
            S[i + j * lds] = UT[i][j];
        }
    }
#pragma unroll 4
    for (int t = 0; t < NB; ++t) {
        float l[RQ];
#pragma unroll
        for (int q = 0; q < RQ; ++q) l[q] = Ls[rg + 32 * q][t];
        const float4 u0 = reinterpret_cast<const float4*>(&UT[t][8 * cg])[0];
        const float4 u1 = reinterpret_cast<const float4*>(&UT[t][8 * cg])[1];
        const float u[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
        for (int q = 0; q < RQ; ++q)
#pragma unroll
            for (int e = 0; e < 8; ++e) acc[q][e] = fmaf(-l[q], u[e], acc[q][e]);
    }
#pragma unroll
    for (int q = 0; q < RQ; ++q)
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int r = rg + 32 * q, cc = 8 * cg + e;
            if (r < R && cc < nc) S[(r0 + r - k) + cc * lds] = acc[q][e];
        }
}

static tmvg_status narrow_update_f32(Context* c, const float* A, int64_t lda, int64_t n, int64_t k, int64_t c0,
                                     int nc, const int* pairs, float* S, int64_t lds)
{
    const int64_t rest = n - k - kNarrowNB;
    const double fr = (double)rest, fc = (double)nc;
    ScopedTimer timer(c, kClsTrailingUpdate, sizeof(float) * (2.0 * fr * fc + fr * kNarrowNB + kNarrowNB * fc),
                      2.0 * fr * fc * kNarrowNB);
    cudaFuncSetAttribute(narrow_update_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNarrowSmem);
    const unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(rest, kNarrowRows));
    narrow_update_f32_kernel<<<grid, kNarrowThreads, kNarrowSmem, c->stream>>>(A, lda, n, k, c0, nc, pairs, S, lds);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "lu: narrow update launch");
}

// General interchanges on a strided matrix (one thread per column).
template <typename T>
__global__ void pivot_rows_kernel(int64_t ncols, T* __restrict__ B, int64_t bsi, int64_t bsj,
                                  const int64_t* __restrict__ P, int64_t i1, int64_t i2, bool reverse)
{
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    T* col = B + c * bsj;
    if (!reverse) {
        for (int64_t i = i1; i < i2; ++i) {
            const int64_t p = P[i];
            if (p != i) { const T a = col[i * bsi]; col[i * bsi] = col[p * bsi]; col[p * bsi] = a; }
        }
    } else {
        for (int64_t i = i2; i > i1;) {
            --i;
            const int64_t p = P[i];
            if (p != i) { const T a = col[i * bsi]; col[i * bsi] = col[p * bsi]; col[p * bsi] = a; }
        }
    }
}

// ---------------------------------------------------------------------
// Triangular solve of one diagonal block (w <= kTriBlock rows) for many
// right-hand sides: each thread substitutes one column, held in shared
// memory.  Lower: x_i = (b_i - sum_{j<i} T_ij x_j) / T_ii; upper the mirror,
// with the sums taken in the order TMV's column-oriented vector solve applies
// its updates (src/TMV_TriDiv_V.cpp:148-236, 322-398).
// skip_zero reproduces that solve's "if (*bj != 0)" test: a zero diagonal
// only raises SINGULAR where it would divide a nonzero; the division is then
// a true division.  Otherwise (TMV's row-major leaves,
// src/TMV_TriDiv_M.cpp:58-188) every zero diagonal is singular and the row
// is multiplied by the reciprocal.
// ---------------------------------------------------------------------
constexpr int kTriCols = 64;     // right-hand sides per CTA of the diagonal-block solve
constexpr int kTriThreads = 256; // threads per CTA of the diagonal-block solve
template <typename T>
__global__ void __launch_bounds__(kTriThreads)
tri_diag_kernel(int w, const T* __restrict__ tri, int64_t tsi, int64_t tsj, bool upper,
                bool unit, int64_t nrhs, T* __restrict__ B, int64_t bsi, int64_t bsj,
                bool skip_zero, int* err)
{
    // dynamic shared memory: Ts[w][w+1] then Xs[w][kTriCols+1]
    extern __shared__ __align__(16) unsigned char tri_smem[];
    T* Tsb = reinterpret_cast<T*>(tri_smem);
    T* Xsb = Tsb + w * (w + 1);
#define Ts(i, j) Tsb[(i) * (w + 1) + (j)]
#define Xs(i, j) Xsb[(i) * (kTriCols + 1) + (j)]
    const int tid = threadIdx.x;
    const int64_t c0 = (int64_t)blockIdx.x * kTriCols;
    const int ncb = (int)min((int64_t)kTriCols, nrhs - c0);

    // staging: eight loads in flight per thread before their stores
    constexpr int QS = 8;
    for (int t0 = tid; t0 < w * w; t0 += kTriThreads * QS) {
        T v[QS];
#pragma unroll
        for (int u = 0; u < QS; ++u) {
            const int t = t0 + u * kTriThreads;
            const int i = t % w, j = t / w;
            const bool need = t < w * w && (upper ? (j >= i) : (i >= j));
            v[u] = need ? tri[i * tsi + j * tsj] : T(0);
        }
#pragma unroll
        for (int u = 0; u < QS; ++u) {
            const int t = t0 + u * kTriThreads;
            if (t < w * w) Ts(t % w, t / w) = v[u];
        }
    }
    for (int t0 = tid; t0 < w * ncb; t0 += kTriThreads * QS) {
        T v[QS];
#pragma unroll
        for (int u = 0; u < QS; ++u) {
            const int t = t0 + u * kTriThreads;
            if (t < w * ncb) {
                // a unit row step reads down the columns, otherwise along the rows
                const int i = bsi == 1 ? t % w : t / ncb, cl = bsi == 1 ? t / w : t % ncb;
                v[u] = B[i * bsi + (c0 + cl) * bsj];
            } else {
                v[u] = T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < QS; ++u) {
            const int t = t0 + u * kTriThreads;
            if (t < w * ncb) {
                const int i = bsi == 1 ? t % w : t / ncb, cl = bsi == 1 ? t / w : t % ncb;
                Xs(i, cl) = v[u];
            }
        }
    }
    __syncthreads();

    // Column-oriented substitution, one step per diagonal entry: the thread
    // owning (j, col) divides x_j, then every (i, col) below (above) takes
    // x_i -= T(i, j) x_j.  Each x_i receives its subtractions in the order
    // j = 0, 1, ... (upper: w-1, w-2, ...), as the row-by-row dot product
    // does, so the results are the same.
    bool sing = false;
    for (int s = 0; s < w; ++s) {
        const int j = upper ? w - 1 - s : s;
        if (!unit) {
            for (int cl = tid; cl < ncb; cl += kTriThreads) {
                T v = Xs(j, cl);
                const T d = Ts(j, j);
                if (skip_zero) {
                    if (v != T(0)) {
                        if (d == T(0)) sing = true;
                        else v = v / d;
                    }
                } else {
                    if (d == T(0)) sing = true;
                    else v = v * (T(1) / d);
                }
                Xs(j, cl) = v;
            }
            __syncthreads();
        }
        const int r0 = upper ? 0 : j + 1, r1 = upper ? j : w;
        const int rows = r1 - r0;
        for (int t = tid; t < rows * ncb; t += kTriThreads) {
            const int i = r0 + t % rows, cl = t / rows;
            Xs(i, cl) -= Ts(i, j) * Xs(j, cl);
        }
        __syncthreads();
    }
    if (sing) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
    if (bsi == 1) {
        for (int t = tid; t < w * ncb; t += kTriThreads) {
            const int i = t % w, cl = t / w;
            B[i + (c0 + cl) * bsj] = Xs(i, cl);
        }
    } else {
        for (int t = tid; t < w * ncb; t += kTriThreads) {
            const int cl = t % ncb, i = t / ncb;
            B[i * bsi + (c0 + cl) * bsj] = Xs(i, cl);
        }
    }
}
#undef Ts
#undef Xs

// Strided copy out(i, j) = in(i, j).
template <typename T>
__global__ void copy_kernel(int64_t m, int64_t n, const T* __restrict__ in, int64_t isi,
                            int64_t isj, T* __restrict__ out, int64_t osi, int64_t osj)
{
    const int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % m, j = t / m;
        out[i * osi + j * osj] = in[i * isi + j * isj];
    }
}

template <typename T>
tmvg_status copy_matrix(Context* c, int64_t m, int64_t n, const T* in, int64_t isi, int64_t isj,
                        T* out, int64_t osi, int64_t osj)
{
    if (m <= 0 || n <= 0) return TMVG_OK;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(m * n, 256), 8 * c->num_sms);
    copy_kernel<T><<<blocks, 256, 0, c->stream>>>(m, n, in, isi, isj, out, osi, osj);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "copy launch");
}

// ---------------------------------------------------------------------
// Host drivers.
// ---------------------------------------------------------------------
template <typename T>
static tmvg_status launch_tri_diag(Context* c, int w, const T* tri, int64_t tsi, int64_t tsj,
                                   bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi,
                                   int64_t bsj, bool skip_zero)
{
    if (nrhs <= 0 || w <= 0) return TMVG_OK;
    const int64_t blocks = ceil_div(nrhs, kTriCols);
    if (blocks > INT_MAX) return set_error(c, TMVG_UNSUPPORTED, "tri solve: too many columns");
    const size_t smem = sizeof(T) * ((size_t)w * (w + 1) + (size_t)w * (kTriCols + 1));
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(tri_diag_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(T) * (kTriBlock * (kTriBlock + 1) + kTriBlock * (kTriCols + 1))));
    tri_diag_kernel<T><<<(unsigned)blocks, kTriThreads, smem, c->stream>>>(
        w, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip_zero, c->dflags);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "tri_diag launch");
}

template <typename T>
tmvg_status tri_solve(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                      bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi, int64_t bsj,
                      bool skip_zero)
{
    if (n <= 0 || nrhs <= 0) return TMVG_OK;
    tmvg_status st;
    if (!upper) {
        for (int64_t kb = 0; kb < n; kb += kTriBlock) {
            const int w = (int)std::min<int64_t>(kTriBlock, n - kb);
            st = launch_tri_diag<T>(c, w, tri + kb * tsi + kb * tsj, tsi, tsj, false, unit, nrhs,
                                    B + kb * bsi, bsi, bsj, skip_zero);
            if (st) return st;
            if (kb + w < n) {
                st = gemm<T>(c, n - kb - w, nrhs, w, T(-1),
                             Mat<const T>{tri + (kb + w) * tsi + kb * tsj, tsi, tsj},
                             Mat<const T>{B + kb * bsi, bsi, bsj}, T(1),
                             Mat<T>{B + (kb + w) * bsi, bsi, bsj});
                if (st) return st;
            }
        }
    } else {
        const int64_t last = ((n - 1) / kTriBlock) * kTriBlock;
        for (int64_t kb = last; kb >= 0; kb -= kTriBlock) {
            const int w = (int)std::min<int64_t>(kTriBlock, n - kb);
            st = launch_tri_diag<T>(c, w, tri + kb * tsi + kb * tsj, tsi, tsj, true, unit, nrhs,
                                    B + kb * bsi, bsi, bsj, skip_zero);
            if (st) return st;
            if (kb > 0) {
                st = gemm<T>(c, kb, nrhs, w, T(-1), Mat<const T>{tri + kb * tsj, tsi, tsj},
                             Mat<const T>{B + kb * bsi, bsi, bsj}, T(1), Mat<T>{B, bsi, bsj});
                if (st) return st;
            }
        }
    }
    return TMVG_OK;
}

template <typename T>
tmvg_status apply_pivots(Context* c, int64_t ncols, T* B, int64_t bsi, int64_t bsj,
                         const int64_t* P, int64_t i1, int64_t i2, bool reverse)
{
    if (ncols <= 0 || i2 <= i1) return TMVG_OK;
    pivot_rows_kernel<T><<<(unsigned)ceil_div(ncols, 128), 128, 0, c->stream>>>(
        ncols, B, bsi, bsj, P, i1, i2, reverse);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "pivot_rows launch");
}

// After the panel at k: its interchanges on the other columns (row pairs),
// U12 = L11^-1 A12, and the trailing update A22 -= L21 U12.
// Multiply-adds x 2 of factoring an m x nb panel: column j scales m-j-1
// entries and updates (m-j-1) x (nb-j-1) of them.
static double panel_flops(int64_t m, int nb)
{
    double f = 0.0;
    for (int j = 0; j < nb; ++j) f += (double)(m - j - 1) * (1.0 + 2.0 * (nb - j - 1));
    return f;
}

// Trailing updates of at least this many rows and columns use the tensor
// cores in the FP32 factorisation; smaller ones stay on the SIMT kernel.
constexpr int64_t kTcMinRest = 256;

// The panel's interchanges on every other column of A (stream order: after
// the panel, before any update that reads those rows).
template <typename T>
static tmvg_status laswp_step(Context* c, int64_t n, T* A, int64_t lda, int64_t k, int nb, const int* pairs)
{
    if (n <= nb) return TMVG_OK;
    const int cols_per_cta = 8;  // one warp per column
    laswp_pairs_kernel<T><<<(unsigned)ceil_div(n, cols_per_cta), 32 * cols_per_cta, 0, c->stream>>>(
        A, lda, n, k, k + nb, pairs);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "lu: laswp launch");
}

// The panel's interchanges on columns [c0, c1) except [skip0, skip1).
template <typename T>
static tmvg_status laswp_cols(Context* c, T* A, int64_t lda, int64_t c0, int64_t c1, int64_t skip0,
                              int64_t skip1, const int* pairs)
{
    if (c1 <= c0) return TMVG_OK;
    const int cols_per_cta = 8;  // one warp per column
    laswp_pairs_kernel<T><<<(unsigned)ceil_div(c1 - c0, cols_per_cta), 32 * cols_per_cta, 0, c->stream>>>(
        A + c0 * lda, lda, c1 - c0, skip0 - c0, skip1 - c0, pairs);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "lu: laswp launch");
}

// Whether the FP32 trailing updates of step (k, nb) run on the tensor cores;
// if so, the step's split copies are set up and L21 is split into them.
template <typename T>
static tmvg_status tc_step_setup(Context* c, int64_t n, T* A, int64_t lda, int64_t k, int nb, bool* tc,
                                 Tf32x3Buffers* b)
{
    *tc = false;
    if constexpr (std::is_same<T, float>::value) {
        const int64_t rest = n - k - nb;
        if (rest >= kTcMinRest && tf32x3_supported(nb)) {
            tmvg_status st = tf32x3_buffers(c, rest, rest, nb, b);
            if (st) return st;
            st = tf32x3_split_a(c, rest, nb, A + (k + nb) + k * lda, lda, *b);
            if (st) return st;
            *tc = true;
        }
    }
    return TMVG_OK;
}

// For the columns [c0, c0 + nc) right of panel (k, nb): U12 = L11^-1 A12, then
// A22 -= L21 U12 on those columns (tensor cores when tc, with U12's split
// copy written by the U12 kernel at its offset in b).
template <typename T>
static tmvg_status update_columns(Context* c, int64_t n, T* A, int64_t lda, int64_t k, int nb, int64_t c0,
                                  int64_t nc, bool tc, const Tf32x3Buffers& b, const int* pairs = nullptr)
{
    // pairs: the step's row interchanges, still to be applied to these
    // columns (fused into the U12 kernel for the next panel's columns)
    if (nc <= 0) return TMVG_OK;
    const bool fuse_swaps = pairs && nb <= RegPanel<T>::NB && nc <= RegPanel<T>::NB;
    if (pairs && !fuse_swaps) {
        tmvg_status st0 = laswp_cols<T>(c, A, lda, c0, c0 + nc, 0, 0, pairs);
        if (st0) return st0;
    }
    const int64_t rest = n - k - nb;  // rows below the panel
    const T* L11 = A + k + k * lda;
    T* A12 = A + k + c0 * lda;
    const double fr = (double)rest, fc = (double)nc;
    ScopedTimer timer(c, kClsTrailingUpdate, sizeof(T) * (2.0 * fr * fc + fr * nb + nb * fc), 2.0 * fr * fc * nb);
    Tf32x3Buffers bc = b;  // B copies of these columns
    if (tc) {
        bc.Bhi = b.Bhi + (c0 - k - nb) * nb;
        bc.Blo = b.Blo + (c0 - k - nb) * nb;
    }
    tmvg_status st;
    if (nb <= RegPanel<T>::NB) {
        constexpr int NB = RegPanel<T>::NB;
        // a few columns (the next panel's): spread over more CTAs, since
        // each one's latency is staging L11 and the substitution chain
        const int* sp = fuse_swaps ? pairs : nullptr;
        if (nc <= NB) {
            const unsigned grid = (unsigned)ceil_div(nc, kU12NarrowCols);
            if (tc)
                u12_reg_kernel<T, NB, true, kU12NarrowCols><<<grid, kU12RegBlock, 0, c->stream>>>(
                    nb, L11, lda, A12, nc, bc.Bhi, bc.Blo, sp, k);
            else
                u12_reg_kernel<T, NB, false, kU12NarrowCols><<<grid, kU12RegBlock, 0, c->stream>>>(
                    nb, L11, lda, A12, nc, nullptr, nullptr, sp, k);
        } else {
            const unsigned grid = (unsigned)ceil_div(nc, kU12RegThreads);
            if (tc)
                u12_reg_kernel<T, NB, true, kU12RegThreads><<<grid, kU12RegBlock, 0, c->stream>>>(
                    nb, L11, lda, A12, nc, bc.Bhi, bc.Blo, nullptr, k);
            else
                u12_reg_kernel<T, NB, false, kU12RegThreads><<<grid, kU12RegBlock, 0, c->stream>>>(
                    nb, L11, lda, A12, nc, nullptr, nullptr, nullptr, k);
        }
        ++c->launches;
        st = check_cuda(c, cudaGetLastError(), "lu: u12 launch");
        if (st) return st;
    } else {
        const size_t smem = sizeof(T) * ((size_t)nb * (nb + 1) + (size_t)nb * (kU12Cols + 1));
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(panel_u12_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        panel_u12_kernel<T><<<(unsigned)ceil_div(nc, kU12Cols), 256, smem, c->stream>>>(nb, L11, lda, A12, nc);
        ++c->launches;
        st = check_cuda(c, cudaGetLastError(), "lu: u12 launch");
        if (st) return st;
        if constexpr (std::is_same<T, float>::value) {
            if (tc) {
                st = tf32x3_split_b(c, nc, nb, A12, lda, bc);
                if (st) return st;
            }
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        // FP32 factor: 3xTF32 on the tensor cores keeps FP32 accuracy
        if (tc) return tf32x3_apply(c, rest, nc, nb, bc, A + (k + nb) + c0 * lda, lda);
    }
    return gemm<T>(c, rest, nc, nb, T(-1), Mat<const T>{A + (k + nb) + k * lda, 1, lda},
                   Mat<const T>{A12, 1, lda}, T(1), Mat<T>{A + (k + nb) + c0 * lda, 1, lda});
}

// Everything of step (k, nb) after its panel: interchanges, U12, update.
template <typename T>
static tmvg_status panel_update(Context* c, int64_t n, T* A, int64_t lda, int64_t k, int nb,
                                const int* pairs)
{
    tmvg_status st = laswp_step<T>(c, n, A, lda, k, nb, pairs);
    if (st || k + nb >= n) return st;
    bool tc;
    Tf32x3Buffers b{};
    st = tc_step_setup<T>(c, n, A, lda, k, nb, &tc, &b);
    if (st) return st;
    return update_columns<T>(c, n, A, lda, k, nb, k + nb, n - k - nb, tc, b);
}

constexpr size_t kClusterSmemMax = 200 * 1024;

// Can this device run the 16-CTA panel cluster with the largest shared
// memory the kernel may ask for?  Checked once per context and type.
template <typename T>
static bool cluster_panel_ok(Context* c)
{
    int& ok = c->cluster_ok[sizeof(T) == 8 ? 0 : 1];
    if (ok >= 0) return ok == 1;
    ok = 0;
    if (cudaFuncSetAttribute(lu_panel_cluster_kernel<T>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(lu_panel_cluster_kernel<T>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClusterSmemMax) !=
            cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = kClusterSmemMax;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, lu_panel_cluster_kernel<T>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ok = clusters >= 1 ? 1 : 0;
    return ok == 1;
}

// Panel width for the cluster path: the widest of 128/64/32 (FP32) or
// 64/32 (FP64) whose ceil(n/16) rows fit a CTA's shared memory; 0 if none.
template <typename T>
static int cluster_panel_width(int64_t n)
{
    const int64_t rows = ceil_div(n, kClusterCtas);
    const int cands[3] = {sizeof(T) == 8 ? 64 : 128, sizeof(T) == 8 ? 32 : 64, 32};
    for (int w : cands)
        if ((size_t)rows * (w + 1) * sizeof(T) <= kClusterSmemMax) return w;
    return 0;
}

template <typename T>
static tmvg_status launch_panel_cluster(Context* c, cudaStream_t s, T* A, int64_t lda, int64_t n, int64_t k,
                                        int nb, int64_t* P, const unsigned char* modes, int* pairs)
{
    const int64_t m = n - k;
    const int rpc = (int)ceil_div(m, kClusterCtas);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = (size_t)rpc * (nb + 1) * sizeof(T);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    ++c->launches;
    return check_cuda(c,
                      cudaLaunchKernelEx(&cfg, lu_panel_cluster_kernel<T>, A, lda, n, k, nb, P,
                                         modes, rpc, pairs),
                      "lu: cluster panel launch");
}

// Can this device run the 16-CTA cluster of the register-resident panel?
template <typename T>
static bool reg_panel_ok(Context* c)
{
    int& ok = c->reg_cluster_ok[sizeof(T) == 8 ? 0 : 1];
    if (ok >= 0) return ok == 1;
    ok = 0;
    // both register panels (the launcher picks one per handle) need the
    // 16-CTA cluster
    auto kern = c->panel_reg2 ? lu_panel_cluster_reg2_kernel<T, RegPanel<T>::NB>
                              : lu_panel_leaf_kernel<T, RegPanel<T>::NB>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(c->panel_reg2 ? kReg2Threads : kLeafThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ok = clusters >= 1 ? 1 : 0;
    return ok == 1;
}

template <typename T>
static tmvg_status launch_panel_cluster_reg(Context* c, cudaStream_t s, T* A, int64_t lda, int64_t n,
                                            int64_t k, int nb, int64_t* P, const unsigned char* modes,
                                            int* pairs, float* ahi, float* alo, const T* Sp = nullptr,
                                            int64_t lds = 0)
{
    // FP32 leaf panel: one row per thread, in the smallest power-of-two
    // cluster whose CTAs hold the panel's rows (16 at m = 8192, 8 from 4096
    // rows down, ... one CTA, with no cluster exchange, at 512 rows): the
    // exchange of a column costs less with fewer CTAs.  FP64 panels spread
    // their rows over 16 CTAs from 128 rows up: their in-panel products run
    // on the FP64 pipe (2 per SM per clock), which fewer SMs would make the
    // limit (n = 2048: 12.4 ms for the LU with the FP32 rule).  The
    // two-rows-per-thread panel keeps 16 CTAs (a panel of at most 512 rows in
    // one CTA).
    const int64_t m = n - k;
    int G = m <= 2 * kReg2Threads ? 1 : kClusterCtas;
    if (!c->panel_reg2) {
        if (sizeof(T) == 4)
            while (G > 1 && (int64_t)(G / 2) * kLeafThreads >= m) G /= 2;
        else
            G = m <= 128 ? 1 : kClusterCtas;
    }
    const int rpc = (int)ceil_div(m, G);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(c->panel_reg2 ? kReg2Threads : kLeafThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    ++c->launches;
    if (c->panel_reg2)
        return check_cuda(c,
                          cudaLaunchKernelEx(&cfg, lu_panel_cluster_reg2_kernel<T, RegPanel<T>::NB>, A,
                                             lda, n, k, nb, P, modes, rpc, pairs, c->dflags, ahi, alo, Sp,
                                             lds),
                          "lu: register panel launch");
    return check_cuda(c,
                      cudaLaunchKernelEx(&cfg, lu_panel_leaf_kernel<T, RegPanel<T>::NB>, A, lda, n, k,
                                         nb, P, modes, rpc, pairs, c->dflags, ahi, alo, Sp, lds),
                      "lu: leaf register panel launch");
}

template <typename T>
tmvg_status lu_factor(Context* c, int64_t n, T* A, int64_t lda, int64_t* P)
{
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "lu: bad n/lda");
    if (n == 0) return TMVG_OK;
    // one panel row per thread of a 16-CTA cluster while the rows fit
    const bool reg = n <= (int64_t)kClusterCtas * 2 * kReg2Threads && reg_panel_ok<T>(c);
    const int cl_nb = reg ? RegPanel<T>::NB : cluster_panel_ok<T>(c) ? cluster_panel_width<T>(n) : 0;
    const int nbmax = cl_nb > 0 ? cl_nb : panel_width<T>();

    // Panel geometry: one CTA per 256 rows up to one per SM.
    const int64_t G_full = std::min<int64_t>(c->num_sms, ceil_div(n, kPanelThreads));
    const int64_t rows_full = ceil_div(n, G_full);
    const size_t smem_full = (size_t)rows_full * (nbmax + 1) * sizeof(T);
    if (smem_full > 200 * 1024)
        return set_error(c, TMVG_UNSUPPORTED, "lu: matrix too tall for the shared-memory panel");

    // Workspace: modes (n bytes), candidate keys/indices/rows, diag rows.
    const size_t off_key = 0;
    const size_t off_idx = off_key + sizeof(double) * 2 * G_full;
    const size_t off_rows = (off_idx + sizeof(long long) * 2 * G_full + 255) & ~size_t(255);
    const size_t off_diag = off_rows + sizeof(T) * 2 * G_full * kPanelMax;
    const size_t off_modes = (off_diag + sizeof(T) * 2 * kPanelMax + 255) & ~size_t(255);
    const size_t off_pairs = (off_modes + (size_t)n + 255) & ~size_t(255);
    // two pair lists: with look-ahead, step s+1's panel writes its list while
    // step s's interchanges still read theirs
    const size_t pairs_len = 1 + 2 * (size_t)kMaxPairs;
    const size_t bytes = off_pairs + sizeof(int) * 2 * pairs_len;
    unsigned char* ws = (unsigned char*)workspace(c, bytes);
    if (!ws) return TMVG_OOM;
    double* cand_key = (double*)(ws + off_key);
    long long* cand_idx = (long long*)(ws + off_idx);
    T* cand_rows = (T*)(ws + off_rows);
    T* diag_row = (T*)(ws + off_diag);
    unsigned char* modes = ws + off_modes;
    int* pairs = (int*)(ws + off_pairs);
    {
        std::vector<unsigned char> hm((size_t)n, 0);
        leaf_modes(0, n, hm);
        tmvg_status st = check_cuda(
            c, cudaMemcpyAsync(modes, hm.data(), (size_t)n, cudaMemcpyHostToDevice, c->stream),
            "lu: modes upload");
        if (st) return st;
        // the host vector must outlive the copy
        st = check_cuda(c, cudaStreamSynchronize(c->stream), "lu: modes sync");
        if (st) return st;
    }

    static bool attr_set[2] = {false, false};
    const int ai = sizeof(T) == 8 ? 0 : 1;
    if (!attr_set[ai]) {
        cudaFuncSetAttribute(lu_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        attr_set[ai] = true;
    }

    if (cl_nb > 0) {
        // Look-ahead: panel k+1 runs on the high-priority side stream as soon
        // as its own columns are updated, while the rest of step k's update
        // runs on the main stream.
        tmvg_status st = ensure_side_stream(c);
        if (st) return st;
        cudaStream_t side = c->side;
        // FP32: split copies for the tensor-core updates, U12 (B) once and
        // L21 (A) double-buffered by step parity, since the panel kernel of
        // step s+1 writes its L21 split while step s's update still reads.
        bool tc_any = false;
        Tf32x3Buffers arena[2] = {};
        // FP32 register path: the narrow update writes the next panel's
        // columns into a scratch panel (n x 64, double-buffered by step
        // parity) that the panel kernel reads
        T* Sbuf[2] = {nullptr, nullptr};
        if constexpr (std::is_same<T, float>::value) {
            const bool tc = n - nbmax >= kTcMinRest && tf32x3_supported(nbmax);
            const bool fused = reg && nbmax == kNarrowNB;
            const size_t part = ((size_t)n * nbmax * sizeof(float) + 255) & ~size_t(255);
            const int nparts = (tc ? 6 : 0) + (fused ? 2 : 0);
            if (nparts > 0) {
                unsigned char* w3 = (unsigned char*)workspace3(c, nparts * part);
                if (!w3) return TMVG_OOM;
                if (tc) {
                    for (int q = 0; q < 2; ++q) {
                        arena[q].Bhi = (float*)w3;
                        arena[q].Blo = (float*)(w3 + part);
                        arena[q].Ahi = (float*)(w3 + (2 + 2 * q) * part);
                        arena[q].Alo = (float*)(w3 + (3 + 2 * q) * part);
                    }
                    tc_any = true;
                }
                if (fused) {
                    Sbuf[0] = (T*)(w3 + (nparts - 2) * part);
                    Sbuf[1] = (T*)(w3 + (nparts - 1) * part);
                }
            }
        }
        auto tc_for = [&](int64_t kk, int w) {
            return tc_any && n - kk - w >= kTcMinRest && tf32x3_supported(w);
        };
        auto pairs_of = [&](int64_t step) { return pairs + (step & 1) * pairs_len; };
        // from_scratch: the panel's columns are in the scratch panel of the
        // step before (row r at Sbuf[(step - 1) & 1][r - (kk - nbmax)]),
        // written by its fused narrow update
        auto panel = [&](int64_t kk, int w, int64_t step, bool from_scratch = false) -> tmvg_status {
            ScopedTimer timer(c, kClsPanel, 2.0 * sizeof(T) * (n - kk) * w, panel_flops(n - kk, w), side);
            // (the register panel writes no L21 split: tf32x3_split_a makes it
            // below, on the main stream, off the chain of panels)
            float* ahi = nullptr;
            float* alo = nullptr;
            int* pp = pairs_of(step);
            tmvg_status s2 =
                reg ? (from_scratch
                           ? launch_panel_cluster_reg<T>(c, side, A, lda, n, kk, w, P, modes + kk, pp, ahi, alo,
                                                         Sbuf[(step - 1) & 1] + nbmax, n)
                           : launch_panel_cluster_reg<T>(c, side, A, lda, n, kk, w, P, modes + kk, pp, ahi, alo))
                    : launch_panel_cluster<T>(c, side, A, lda, n, kk, w, P, modes + kk, pp);
            if (!s2 && c->serialize_lookahead) s2 = check_cuda(c, cudaStreamSynchronize(side), "lu: serialize");
            return s2;
        };
        // The chain of the factorisation runs on the side stream with no
        // hand-off between streams: panel k, the update of the next panel's
        // columns with step k (interchanges inside the U12 kernel, U12, the
        // narrow update), panel k+1, ...  The main stream applies step k to
        // every other column (the wide update) once the narrow update of step
        // k is done (event ev_fork), overlapping panel k+1, and the side
        // stream's narrow update of step k+1 waits for that wide update (it
        // covers the same columns with step k first; event ev_wide), which
        // is normally finished by then.  The event waits are enqueued before
        // the events are recorded again, so each refers to its own step.
        st = check_cuda(c, cudaEventRecord(c->ev_fork, c->stream), "lu: fork");
        if (!st) st = check_cuda(c, cudaStreamWaitEvent(side, c->ev_fork, 0), "lu: fork");
        if (!st) st = panel(0, (int)std::min<int64_t>(nbmax, n), 0);
        if (!st) st = check_cuda(c, cudaEventRecord(c->ev_panel, side), "lu: panel event");
        cudaStream_t main_stream = c->stream;
        for (int64_t k = 0, step = 0; k < n && !st; k += nbmax, ++step) {
            const int nb = (int)std::min<int64_t>(nbmax, n - k);
            const int* pk = pairs_of(step);
            if (k + nb >= n) {
                st = check_cuda(c, cudaStreamWaitEvent(c->stream, c->ev_panel, 0), "lu: join");
                if (!st) st = laswp_step<T>(c, n, A, lda, k, nb, pk);
                break;
            }
            const int64_t rest = n - k - nb;
            const int nb2 = (int)std::min<int64_t>(nbmax, rest);
            const bool tc = tc_for(k, nb);
            const Tf32x3Buffers& b = arena[step & 1];
            // side: the next panel's columns (after the previous step's wide
            // update, event ev_wide), then the next panel
            if (step > 0) st = check_cuda(c, cudaStreamWaitEvent(side, c->ev_wide, 0), "lu: wide wait");
            c->stream = side;
            // the fused narrow update (FP32 register path, 64-wide step) writes
            // the next panel's columns into Sp; otherwise they are updated in A
            T* Sk = Sbuf[step & 1];
            const bool fused = Sk != nullptr && nb == kNarrowNB;
            if constexpr (std::is_same<T, float>::value) {
                // the L21 split here when the narrow update reads it; with the
                // fused narrow update (exact FP32) only the wide update does,
                // and the main stream makes it
                if (!st && tc && !fused) st = tf32x3_split_a(c, rest, nb, A + (k + nb) + k * lda, lda, b);
                if (!st && fused) st = narrow_update_f32(c, A, lda, n, k, k + nb, nb2, pk, Sk, n);
            }
            if (!st && !fused) st = update_columns<T>(c, n, A, lda, k, nb, k + nb, nb2, tc, b, pk);
            c->stream = main_stream;
            // the wide update starts after the narrow one, not beside it: the
            // narrow update, on the chain, gets the whole GPU
            if (!st) st = check_cuda(c, cudaEventRecord(c->ev_fork, side), "lu: narrow done");
            if (!st) st = check_cuda(c, cudaStreamWaitEvent(c->stream, c->ev_fork, 0), "lu: join");
            if (!st) st = panel(k + nb, nb2, step + 1, fused);
            if (!st) st = check_cuda(c, cudaEventRecord(c->ev_panel, side), "lu: panel event");
            // main: everything else of step k, overlapping the next panel;
            // with the fused narrow update first its U12 (the scratch panel's
            // first nb rows) into A: the next panel reads the scratch panel
            // and writes only rows below these, and the scratch panel is
            // reused two steps later, after this step's wide update
            if constexpr (std::is_same<T, float>::value)
                if (!st && tc && fused) st = tf32x3_split_a(c, rest, nb, A + (k + nb) + k * lda, lda, b);
            if (!st && fused)
                st = check_cuda(c,
                                cudaMemcpy2DAsync(A + k + (k + nb) * lda, sizeof(T) * lda, Sk, sizeof(T) * n,
                                                  sizeof(T) * nb, nb2, cudaMemcpyDeviceToDevice, c->stream),
                                "lu: U12 copy");
            if (!st) st = laswp_cols<T>(c, A, lda, 0, n, k, k + nb + nb2, pk);
            if (!st) st = update_columns<T>(c, n, A, lda, k, nb, k + nb + nb2, rest - nb2, tc, b);
            if (!st) st = check_cuda(c, cudaEventRecord(c->ev_wide, c->stream), "lu: wide event");
        }
        c->stream = main_stream;
        if (st) {
            // leave no side work unordered after an error
            cudaStreamSynchronize(side);
            return st;
        }
        return collect_device_error(c, "lu_factor");
    }

    for (int64_t k = 0; k < n; k += nbmax) {
        const int nb = (int)std::min<int64_t>(nbmax, n - k);
        const int64_t m = n - k;
        const int G = (int)std::min<int64_t>(c->num_sms, ceil_div(m, kPanelThreads));
        const int rows_per_cta = (int)ceil_div(m, G);
        const size_t smem = (size_t)rows_per_cta * (nb + 1) * sizeof(T);
        tmvg_status st = check_cuda(c, cudaMemsetAsync(c->dbar, 0, sizeof(unsigned), c->stream),
                                    "lu: barrier reset");
        if (st) return st;
        T* Ap = A;
        int64_t* Pp = P;
        const unsigned char* mp = modes + k;
        int64_t ldav = lda, nv = n, kv = k;
        int nbv = nb, rpc = rows_per_cta;
        unsigned* bar = c->dbar;
        int* err = c->dflags;
        void* args[] = {&Ap, &ldav, &nv, &kv, &nbv, &Pp, &mp, &rpc, &cand_key, &cand_idx,
                        &cand_rows, &diag_row, &bar, &err, &pairs};
        {
            ScopedTimer timer(c, kClsPanel, 2.0 * sizeof(T) * m * nb, panel_flops(m, nb));
            st = check_cuda(c,
                            cudaLaunchCooperativeKernel((const void*)lu_panel_kernel<T>, dim3(G),
                                                        dim3(kPanelThreads), args, smem, c->stream),
                            "lu: panel launch");
        }
        if (st) return st;
        ++c->launches;
        st = panel_update<T>(c, n, A, lda, k, nb, pairs);
        if (st) return st;
    }
    return collect_device_error(c, "lu_factor");
}

// Triangular solve of the pivoted right-hand sides: the single-launch
// sync-free kernel (one CTA per 64-row block and group of right-hand sides)
// up to 256 columns, the blocked product-based solve for more.
template <typename T>
static tmvg_status tri_any(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                           bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi, int64_t bsj,
                           bool skip_zero)
{
    if (nrhs <= 256 && ceil_div(n, (int64_t)64) * ceil_div(nrhs, (int64_t)4) <= kTrsvFlagCap)
        return trsm_sync_free<T>(c, n, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip_zero);
    return tri_solve<T>(c, n, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip_zero);
}

// m /= T for a standalone triangle (TriLDivEq(GenUpper/LowerTriMatrix, MatrixView),
// src/TMV_TriDiv_M.cpp:583-710): one right-hand side takes TMV's vector path
// (a zero T(j,j) matters only where the entry it divides is nonzero), a
// column-major B the same column-by-column rule of NonBlasTriLDivEq's
// leaves; any other B treats every zero T(j,j) as singular.
template <typename T>
tmvg_status tri_ldiveq(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj, bool upper, bool unit,
                       int64_t nrhs, T* B, int64_t bsi, int64_t bsj)
{
    if (n <= 0 || nrhs <= 0) return TMVG_OK;
    const bool skip = nrhs == 1 || bsi == 1;
    tmvg_status st = tri_any<T>(c, n, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip);
    if (st) return st;
    return collect_device_error(c, "tri_ldiveq");
}

template <typename T>
tmvg_status lu_ldiveq(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                      int64_t nrhs, T* B, int64_t bsi, int64_t bsj)
{
    // src/TMV_LUDiv.cpp:186-226: m.permuteRows(P); m /= L(unit); m /= U.
    // The interchanges are applied as one gather into a dense column-major
    // scratch, which is solved and copied back.
    if (n <= 0 || nrhs <= 0) return TMVG_OK;
    const size_t pbytes = (sizeof(int) * (size_t)n + 255) & ~size_t(255);
    unsigned char* ws = (unsigned char*)workspace(c, pbytes + sizeof(T) * (size_t)n * nrhs);
    if (!ws) return TMVG_OOM;
    int* perm = (int*)ws;
    T* X = (T*)(ws + pbytes);
    tmvg_status st = pivots_to_perm(c, n, P, perm);
    if (st) return st;
    st = permute_rows<T>(c, n, nrhs, perm, B, bsi, bsj, X, 1, n, false);
    if (st) return st;
    // Column-major B (or one column) takes TMV's vector path: skip semantics.
    st = tri_any<T>(c, n, LU, 1, lda, false, true, nrhs, X, 1, n, true);
    if (st) return st;
    st = tri_any<T>(c, n, LU, 1, lda, true, false, nrhs, X, 1, n, true);
    if (st) return st;
    st = copy_matrix<T>(c, n, nrhs, X, 1, n, B, bsi, bsj);
    if (st) return st;
    return collect_device_error(c, "lu_ldiveq");
}

template <typename T>
tmvg_status lu_rdiveq(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                      int64_t nrows, T* B, int64_t bsi, int64_t bsj)
{
    // src/TMV_LUDiv.cpp:370-411: m %= U; m %= L; m.reversePermuteCols(P), with
    // m %= T computed as T^T.LDivEq(m^T) (include/tmv/TMV_TriMatrix.h:945-946).
    if (n <= 0 || nrows <= 0) return TMVG_OK;
    const size_t pbytes = (sizeof(int) * (size_t)n + 255) & ~size_t(255);
    unsigned char* ws = (unsigned char*)workspace(c, pbytes + sizeof(T) * (size_t)n * nrows);
    if (!ws) return TMVG_OOM;
    int* perm = (int*)ws;
    T* X = (T*)(ws + pbytes);  // m^T, n x nrows column-major
    // m^T: element (i, j) = B[j*bsi + i*bsj]
    tmvg_status st = copy_matrix<T>(c, n, nrows, B, bsj, bsi, X, 1, n);
    if (st) return st;
    // One row of m is one vector (skip semantics); otherwise m^T is
    // row-major in TMV and its row-major leaves check every diagonal.
    const bool skip = (nrows == 1);
    st = tri_any<T>(c, n, LU, lda, 1, false, false, nrows, X, 1, n, skip);
    if (st) return st;
    st = tri_any<T>(c, n, LU, lda, 1, true, true, nrows, X, 1, n, skip);
    if (st) return st;
    // reversePermuteCols(P): undo the interchanges, i.e. scatter by perm
    st = pivots_to_perm(c, n, P, perm);
    if (st) return st;
    st = permute_rows<T>(c, n, nrows, perm, X, 1, n, B, bsj, bsi, true);
    if (st) return st;
    return collect_device_error(c, "lu_rdiveq");
}

// ---------------------------------------------------------------------
// Inverse from the factors.
// ---------------------------------------------------------------------
template <typename T>
__global__ void identity_kernel(int64_t n, T* __restrict__ M, int64_t ldm)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, j = t / n;
        M[i + j * ldm] = i == j ? T(1) : T(0);
    }
}

// out[:, perm[j]] = in[:, j] (reversePermuteCols with perm from pivots_to_perm).
template <typename T>
__global__ void scatter_cols_kernel(int64_t n, const int* __restrict__ perm, const T* __restrict__ in,
                                    int64_t ldi, T* __restrict__ out, int64_t ldo)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, j = t / n;
        out[i + (int64_t)perm[j] * ldo] = in[i + j * ldi];
    }
}

// Y = U^-1 L^-1 into the dense n x n buffer Y (leading dimension n).
// L^-1 is the unit-lower solve of the identity: column block c of L^-1 is
// zero above row block c, so block step kb solves and updates only the
// columns [0, kb + w) (n^3/3 flops); U^-1 (L^-1) is the dense upper solve
// (n^3 flops).  A zero U(j,j) is reported as singular.
template <typename T>
static tmvg_status inverse_unpermuted(Context* c, int64_t n, const T* LU, int64_t lda, T* Y)
{
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n * n, 256), 8 * c->num_sms);
    identity_kernel<T><<<blocks, 256, 0, c->stream>>>(n, Y, n);
    ++c->launches;
    tmvg_status st = check_cuda(c, cudaGetLastError(), "inverse: identity launch");
    for (int64_t kb = 0; kb < n && !st; kb += kTriBlock) {
        const int w = (int)std::min<int64_t>(kTriBlock, n - kb);
        const int64_t cols = kb + w;
        st = launch_tri_diag<T>(c, w, LU + kb + kb * lda, 1, lda, false, true, cols, Y + kb, 1, n, false);
        if (!st && kb + w < n)
            st = gemm<T>(c, n - kb - w, cols, w, T(-1), Mat<const T>{LU + (kb + w) + kb * lda, 1, lda},
                         Mat<const T>{Y + kb, 1, n}, T(1), Mat<T>{Y + kb + w, 1, n});
    }
    if (!st) st = tri_solve<T>(c, n, LU, 1, lda, true, false, n, Y, 1, n, false);
    return st;
}

template <typename T>
tmvg_status lu_inverse(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P, T* M, int64_t ldm)
{
    // LU_Inverse (src/TMV_LUInverse.cpp:38-52, 236-299): A^-1 = U^-1 L^-1,
    // then minv.reversePermuteCols(P), here one column scatter.
    if (n <= 0) return TMVG_OK;
    const size_t pbytes = (sizeof(int) * (size_t)n + 255) & ~size_t(255);
    unsigned char* ws = (unsigned char*)workspace(c, pbytes + sizeof(T) * (size_t)n * n);
    if (!ws) return TMVG_OOM;
    int* perm = (int*)ws;
    T* Y = (T*)(ws + pbytes);
    tmvg_status st = inverse_unpermuted<T>(c, n, LU, lda, Y);
    if (!st) st = pivots_to_perm(c, n, P, perm);
    if (!st) {
        const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n * n, 256), 8 * c->num_sms);
        scatter_cols_kernel<T><<<blocks, 256, 0, c->stream>>>(n, perm, Y, n, M, ldm);
        ++c->launches;
        st = check_cuda(c, cudaGetLastError(), "inverse: scatter launch");
    }
    if (st) return st;
    return collect_device_error(c, "lu_inverse");
}

template <typename T>
tmvg_status lu_inverse_ata(Context* c, int64_t n, const T* LU, int64_t lda, T* M, int64_t ldm)
{
    // LUDiv::doMakeInverseATA (src/TMV_LUD.cpp:172-200): (A^T A)^-1 =
    // U^-1 L^-1 L^-T U^-T = Y Y^T with Y = U^-1 L^-1 (the permutation
    // cancels); TMV forms the same product as linv*linv^T, /= U, %= U^T.
    if (n <= 0) return TMVG_OK;
    T* Y = (T*)workspace(c, sizeof(T) * (size_t)n * n);
    if (!Y) return TMVG_OOM;
    tmvg_status st = inverse_unpermuted<T>(c, n, LU, lda, Y);
    if (!st)
        st = gemm<T>(c, n, n, n, T(1), Mat<const T>{Y, 1, n}, Mat<const T>{Y, n, 1}, T(0), Mat<T>{M, 1, ldm});
    if (st) return st;
    return collect_device_error(c, "lu_inverse_ata");
}

template tmvg_status lu_factor<double>(Context*, int64_t, double*, int64_t, int64_t*);
template tmvg_status lu_inverse<double>(Context*, int64_t, const double*, int64_t, const int64_t*, double*,
                                        int64_t);
template tmvg_status tri_ldiveq<double>(Context*, int64_t, const double*, int64_t, int64_t, bool, bool,
                                        int64_t, double*, int64_t, int64_t);
template tmvg_status lu_inverse_ata<double>(Context*, int64_t, const double*, int64_t, double*, int64_t);
template tmvg_status lu_factor<float>(Context*, int64_t, float*, int64_t, int64_t*);
template tmvg_status lu_inverse<float>(Context*, int64_t, const float*, int64_t, const int64_t*, float*,
                                       int64_t);
template tmvg_status lu_rdiveq<float>(Context*, int64_t, const float*, int64_t, const int64_t*,
                                      int64_t, float*, int64_t, int64_t);
template tmvg_status tri_solve<double>(Context*, int64_t, const double*, int64_t, int64_t, bool,
                                       bool, int64_t, double*, int64_t, int64_t, bool);
template tmvg_status tri_solve<float>(Context*, int64_t, const float*, int64_t, int64_t, bool,
                                      bool, int64_t, float*, int64_t, int64_t, bool);
template tmvg_status apply_pivots<double>(Context*, int64_t, double*, int64_t, int64_t,
                                          const int64_t*, int64_t, int64_t, bool);
template tmvg_status apply_pivots<float>(Context*, int64_t, float*, int64_t, int64_t,
                                         const int64_t*, int64_t, int64_t, bool);
template tmvg_status lu_ldiveq<double>(Context*, int64_t, const double*, int64_t, const int64_t*,
                                       int64_t, double*, int64_t, int64_t);
template tmvg_status lu_rdiveq<double>(Context*, int64_t, const double*, int64_t, const int64_t*,
                                       int64_t, double*, int64_t, int64_t);
template tmvg_status lu_ldiveq<float>(Context*, int64_t, const float*, int64_t, const int64_t*,
                                      int64_t, float*, int64_t, int64_t);
template tmvg_status copy_matrix<double>(Context*, int64_t, int64_t, const double*, int64_t,
                                         int64_t, double*, int64_t, int64_t);
template tmvg_status copy_matrix<float>(Context*, int64_t, int64_t, const float*, int64_t,
                                        int64_t, float*, int64_t, int64_t);

}  // namespace tmvg

// =====================================================================
// LU factorisation without device allocation.
//
// Some callers of this library cannot allocate device memory: programs whose
// device memory is owned entirely by another allocator (a framework's caching
// allocator or a fixed arena that must not see cudaMalloc behind its back),
// and code paths where an allocation's latency or failure is not acceptable.
// tmvg_lu_decompose_f64_noalloc serves them.  It applies the pivot rule of
// tmvg_lu_decompose_f64 and gives the same factors to rounding, but runs the
// simplest schedule: the cooperative grid-barrier panel (lu_panel_kernel)
// with no look-ahead, and every scratch word taken from the file-scope array
// below, which each GPU that loads this library holds until the process
// exits (kNoAllocBytes = 353,540 bytes, about 345 KiB).  It needs no
// tmvg_handle (creating one allocates).  Limits: n <= kNoAllocMaxN = 16384
// (larger n returns TMVG_UNSUPPORTED before any device work); at most
// kNoAllocMaxCtas = 160 panel CTAs are used, and a panel CTA's rows must fit
// in 200 KiB of shared memory (TMVG_UNSUPPORTED otherwise, also before any
// device work; on a GPU with at least 40 SMs every n <= 16384 fits).
// =====================================================================
namespace tmvg {
namespace {
constexpr int64_t kNoAllocMaxN = 16384;
constexpr int kNoAllocMaxCtas = 160;
constexpr size_t kNaOffErr = 0;    // int[2]: device error word + aux
constexpr size_t kNaOffBar = 64;   // unsigned: grid-barrier counter
constexpr size_t kNaOffKey = 256;  // double[2 * kNoAllocMaxCtas]
constexpr size_t kNaOffIdx = kNaOffKey + sizeof(double) * 2 * kNoAllocMaxCtas;
constexpr size_t kNaOffRows = kNaOffIdx + sizeof(long long) * 2 * kNoAllocMaxCtas;
constexpr size_t kNaOffDiag = kNaOffRows + sizeof(double) * 2 * kNoAllocMaxCtas * kPanelMax;
constexpr size_t kNaOffModes = kNaOffDiag + sizeof(double) * 2 * kPanelMax;
constexpr size_t kNaOffPairs = kNaOffModes + kNoAllocMaxN;  // int[1 + 2*kMaxPairs]
constexpr size_t kNoAllocBytes = kNaOffPairs + sizeof(int) * (1 + 2 * kMaxPairs);
constexpr size_t kNoAllocSmemMax = 200 * 1024;
}  // namespace

static __device__ __align__(256) unsigned char g_lu_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array in the current context.  The host-side
// name of a __device__ array is only a stand-in, so the address is asked of
// the runtime on every call: the lookup allocates nothing, and a cached value
// would go stale when the module is loaded again (after cudaDeviceReset, or
// in another context on the same device).
static unsigned char* noalloc_scratch(tmvg_status* st)
{
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_lu_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        *st = TMVG_CUDA_ERROR;
        return nullptr;
    }
    *st = TMVG_OK;
    return static_cast<unsigned char*>(p);
}

}  // namespace tmvg

extern "C" tmvg_status tmvg_lu_decompose_f64_noalloc(int64_t n, double* A, int64_t lda, int64_t* P,
                                                     void* stream)
{
    using namespace tmvg;
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return TMVG_BAD_ARG;
    if (n > kNoAllocMaxN) return TMVG_UNSUPPORTED;
    if (n == 0) return TMVG_OK;
    if (!A || !P) return TMVG_BAD_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return TMVG_NO_DEVICE;
    }
    // The first panel holds the most rows per CTA: refuse a size whose rows
    // do not fit in shared memory before any device work.
    const int nbmax = panel_width<double>();
    {
        const int G0 = (int)std::min<int64_t>(std::min(sms, kNoAllocMaxCtas), ceil_div(n, kPanelThreads));
        const size_t smem0 = (size_t)ceil_div(n, G0) * (std::min<int64_t>(nbmax, n) + 1) * sizeof(double);
        if (smem0 > kNoAllocSmemMax) return TMVG_UNSUPPORTED;
    }
    if (cudaFuncSetAttribute(lu_panel_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kNoAllocSmemMax) != cudaSuccess) {
        cudaGetLastError();
        return TMVG_CUDA_ERROR;
    }
    tmvg_status st = TMVG_OK;
    unsigned char* s = noalloc_scratch(&st);
    if (!s) return st;

    // A context on the stack: no workspace, flags and barrier in the scratch.
    Context c;
    c.device = dev;
    c.num_sms = std::min(sms, kNoAllocMaxCtas);
    c.stream = static_cast<cudaStream_t>(stream);
    c.dflags = reinterpret_cast<int*>(s + kNaOffErr);
    c.dbar = reinterpret_cast<unsigned*>(s + kNaOffBar);
    double* cand_key = reinterpret_cast<double*>(s + kNaOffKey);
    long long* cand_idx = reinterpret_cast<long long*>(s + kNaOffIdx);
    double* cand_rows = reinterpret_cast<double*>(s + kNaOffRows);
    double* diag_row = reinterpret_cast<double*>(s + kNaOffDiag);
    unsigned char* modes = s + kNaOffModes;
    int* pairs = reinterpret_cast<int*>(s + kNaOffPairs);

    // The array keeps the last call's contents: clear the error words.
    st = check_cuda(&c, cudaMemsetAsync(s, 0, 256, c.stream), "noalloc: clear");
    if (st) return st;
    {
        std::vector<unsigned char> hm((size_t)n, 0);
        leaf_modes(0, n, hm);
        st = check_cuda(&c, cudaMemcpyAsync(modes, hm.data(), (size_t)n, cudaMemcpyHostToDevice, c.stream),
                        "noalloc: modes");
        if (st) return st;
        st = check_cuda(&c, cudaStreamSynchronize(c.stream), "noalloc: modes sync");
        if (st) return st;
    }
    for (int64_t k = 0; k < n; k += nbmax) {
        const int nb = (int)std::min<int64_t>(nbmax, n - k);
        const int64_t m = n - k;
        const int G = (int)std::min<int64_t>(c.num_sms, ceil_div(m, kPanelThreads));
        const int rows_per_cta = (int)ceil_div(m, G);
        const size_t smem = (size_t)rows_per_cta * (nb + 1) * sizeof(double);
        st = check_cuda(&c, cudaMemsetAsync(c.dbar, 0, sizeof(unsigned), c.stream), "noalloc: barrier");
        if (st) return st;
        double* Ap = A;
        int64_t* Pp = P;
        const unsigned char* mp = modes + k;
        int64_t ldav = lda, nv = n, kv = k;
        int nbv = nb, rpc = rows_per_cta;
        unsigned* bar = c.dbar;
        int* err = c.dflags;
        void* args[] = {&Ap, &ldav, &nv, &kv, &nbv, &Pp, &mp, &rpc, &cand_key, &cand_idx,
                        &cand_rows, &diag_row, &bar, &err, &pairs};
        st = check_cuda(&c,
                        cudaLaunchCooperativeKernel((const void*)lu_panel_kernel<double>, dim3(G),
                                                    dim3(kPanelThreads), args, smem, c.stream),
                        "noalloc: panel launch");
        if (st) return st;
        st = panel_update<double>(&c, n, A, lda, k, nb, pairs);
        if (st) return st;
    }
    int code[2] = {0, 0};
    st = check_cuda(&c, cudaMemcpyAsync(code, c.dflags, sizeof(code), cudaMemcpyDeviceToHost, c.stream),
                    "noalloc: status");
    if (st) return st;
    st = check_cuda(&c, cudaStreamSynchronize(c.stream), "noalloc: sync");
    if (st) return st;
    if (code[0] == kDevTimeout) return TMVG_TIMEOUT;
    if (code[0] != kDevOk) return TMVG_CUDA_ERROR;
    return TMVG_OK;
}
