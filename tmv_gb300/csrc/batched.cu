// batched.cu -- thousands of uneven LU factor + solve problems in one
// persistent launch (FP64), replayed from a captured CUDA graph.
//
// Layout: system s has order n[s] and nrhs[s] right-hand sides; A_s is the
// column-major n x n block at A + a_off[s], B_s the column-major n x nrhs
// block at B + b_off[s] (overwritten by X_s = A_s^-1 B_s), the pivots go to
// P + p_off[s] and A_s is overwritten by its LU factors, as LU_Decompose and
// LU_LDivEq do for one matrix (src/TMV_LUDecompose.cpp:514,
// src/TMV_LUDiv.cpp:186).  status[s] = 1 when a zero U(j,j) met a nonzero
// (TMV's SingularUpperTriMatrix), else 0.
//
// Kernel: grid = SMs x resident CTAs (128 threads, four per SM, so that one
// CTA's barrier-bound phases overlap another's FMA work); each CTA repeatedly takes the next
// system from an atomic queue over `order` (largest n first, so the tail of
// the launch holds the small systems) and runs, for n <= 256:
//   for each panel of PW columns:
//     factor the panel in shared memory with TMV's pivot rule (pivot_key),
//     apply its interchanges to the other columns of A_s and to B_s,
//     U12 = L11^-1 A12 (one column per thread, in registers),
//     A22 -= L21 U12 (4x4 register tiles, FP64 FMA, U12 read back from A),
//   then forward/back substitution of B_s staged in shared memory.
// FP64 FMA throughput (about 2 per SM per clock on GB300) bounds the kernel.
// PW (8 or 16) is chosen per size class by the plan's tuner.
#include "batched.cuh"
#include "lu.cuh"
#include "pivots.cuh"

#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

namespace tmvg {

constexpr int kBatchThreads = 128;
constexpr int kBatchMaxN = 256;
constexpr int kBatchMaxRhs = 16;
constexpr int kNumClasses = 4;  // n <= 32, <= 64, <= 128, <= 256
constexpr int kSolveBlock = 32;  // columns per block of the substitutions

__host__ __device__ inline int size_class(int64_t n)
{
    return n <= 32 ? 0 : n <= 64 ? 1 : n <= 128 ? 2 : 3;
}

// Shared-memory doubles a panel width needs: the panel [256][PW+1].
__host__ __device__ constexpr int batch_smem_doubles(int pw)
{
    return kBatchMaxN * (pw + 1);
}

// Is column c of an n-column LU the second column of one of TMV's two-column
// recursion leaves (src/TMV_LUDecompose.cpp:241-245, 274-358)?
__device__ inline bool r2_column(int64_t n, int64_t c)
{
    int64_t off = 0, R = n;
    while (R > 2) {
        int64_t N1 = R / 2;
        if (N1 > 64) N1 = (N1 / 64) * 64;
        if (c < off + N1) R = N1;
        else { off += N1; R -= N1; }
    }
    return R == 2 && c == off + 1;
}

struct BatchDev {
    const int64_t* n;
    const int64_t* nrhs;
    const int64_t* a_off;
    const int64_t* b_off;
    const int64_t* p_off;
    const int* order;
    double* A;
    double* B;
    int64_t* P;
    int* status;
    int64_t count;
    int pw[kNumClasses];
    // mixed precision only: FP32 factors (at a_off), refinement limits and
    // optional per-system outputs
    float* As;
    int max_iter;
    double tol;
    int* iters;
    double* berr;
};

// FP32 factors stage U12 in shared memory for the trailing update (FP32 FMA
// is fast enough that streaming U12 from L1/L2 bounds it); FP64 reads it back
// from A (the FP64 FMA pipe is the bound there, and the smaller footprint
// keeps four CTAs per SM).
template <typename T>
constexpr bool kStageU12 = sizeof(T) == 4;

// The blocked LU of one system in place (A n x n column-major, element type
// T), pivots to P; the interchanges are also applied to the r columns of B
// (B may be null with r = 0).  Pivot keys compare in FP64 for either T.
// x != 0 on the integer pipe (a double comparison takes an FP64 issue slot,
// which the substitutions' products need): the bits without the sign.
__device__ __forceinline__ bool nz(double x) { return (__double_as_longlong(x) << 1) != 0; }
__device__ __forceinline__ bool nz(float x) { return (__float_as_uint(x) << 1) != 0u; }

template <typename T, int PW>
__device__ void factor_one(int64_t n, int64_t r, T* __restrict__ A, T* __restrict__ B,
                           int64_t* __restrict__ P, T* smem)
{
    constexpr int LDP = PW + 1;
    T* pan = smem;  // [256][LDP]
    T* u12s = smem + kBatchMaxN * LDP;  // FP32 only: U12 rows [PW][256]
    __shared__ long long s_key[kBatchThreads / 32];
    __shared__ long long s_idx[kBatchThreads / 32];
    __shared__ long long w_key;
    __shared__ long long w_idx;
    __shared__ int s_piv[PW];
    __shared__ int s_pairs[1 + 2 * kMaxPairs];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    bool prev_uf = false;

    for (int64_t k0 = 0; k0 < n; k0 += PW) {
        const int w = (int)min((int64_t)PW, n - k0);
        const int m = (int)(n - k0);
        // eight loads in flight per thread before their stores
        for (int t0 = tid; t0 < m * w; t0 += kBatchThreads * 8) {
            T v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int t = t0 + q * kBatchThreads;
                v[q] = t < m * w ? A[(k0 + t % m) + (k0 + t / m) * n] : T(0);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int t = t0 + q * kBatchThreads;
                if (t < m * w) pan[(t % m) * LDP + t / m] = v[q];
            }
        }
        __syncthreads();
        for (int j = 0; j < w; ++j) {
            const bool r2 = r2_column(n, k0 + j) && !prev_uf;
            long long bk = LLONG_MIN;
            long long bi = LLONG_MAX;
            for (int rr = j + tid; rr < m; rr += kBatchThreads)
                pivot_icombine(bk, bi, pivot_ikey(pan[rr * LDP + j], rr == j, r2), (long long)rr);
            warp_pivot_ireduce(bk, bi);
            if (lane == 0) { s_key[warp] = bk; s_idx[warp] = bi; }
            __syncthreads();
            if (warp == 0) {
                bk = lane < kBatchThreads / 32 ? s_key[lane] : LLONG_MIN;
                bi = lane < kBatchThreads / 32 ? s_idx[lane] : LLONG_MAX;
                warp_pivot_ireduce(bk, bi);
                if (lane == 0) { w_key = bk; w_idx = bi; }
            }
            __syncthreads();
            const int wi = (int)w_idx;
            // the winning key is the bits of |pivot| (0 or inf bits for a NaN
            // first element): TMV_Underflow is a comparison of bit patterns
            if (w_key < __double_as_longlong(std::is_same<T, double>::value ? 2.2250738585072014e-308
                                                                            : 1.1754943508222875e-38)) {
                if (tid == 0) s_piv[j] = (int)(k0 + j);
                for (int rr = j + tid; rr < m; rr += kBatchThreads) pan[rr * LDP + j] = T(0);
                prev_uf = true;
            } else {
                prev_uf = false;
                if (tid == 0) s_piv[j] = (int)(k0 + wi);
                if (wi != j && tid < w) {
                    const T t = pan[j * LDP + tid];
                    pan[j * LDP + tid] = pan[wi * LDP + tid];
                    pan[wi * LDP + tid] = t;
                }
                __syncthreads();
                const T inv = T(1) / pan[j * LDP + j];
                for (int rr = j + 1 + tid; rr < m; rr += kBatchThreads) {
                    T* row = pan + rr * LDP;
                    const T l = row[j] * inv;
                    row[j] = l;
                    for (int cc = j + 1; cc < w; ++cc) row[cc] -= l * pan[j * LDP + cc];
                }
            }
            __syncthreads();
        }
        for (int t = tid; t < m * w; t += kBatchThreads) {
            const int rr = t % m, cc = t / m;
            A[(k0 + rr) + (k0 + cc) * n] = pan[rr * LDP + cc];
        }
        for (int j = tid; j < w; j += kBatchThreads) P[k0 + j] = s_piv[j];
        // interchanges on the other columns of A and on B: the panel's swaps
        // as (dst, src) row pairs, applied per column as one gather
        if (warp == 0) panel_row_pairs(k0, w, s_piv, s_pairs);
        __syncthreads();
        {
            const int np = s_pairs[0];
            const int* dst = s_pairs + 1;
            const int* src = s_pairs + 1 + kMaxPairs;
            // a warp per column, a lane per pair: at most 2 PW <= 32 rows move
            static_assert(2 * PW <= 32, "one lane per row pair");
            for (int64_t col = warp; col < n + r; col += kBatchThreads / 32) {
                if (col >= k0 && col < k0 + w) continue;
                T* p = col < n ? A + col * n : B + (col - n) * n;
                T v = T(0);
                if (lane < np) v = p[src[lane]];
                __syncwarp();
                if (lane < np) p[dst[lane]] = v;
            }
        }
        __syncthreads();
        const int ncol = (int)(n - k0 - w);
        if (ncol > 0) {
            // U12 = L11^-1 A12, one column per thread in registers, written
            // back in place (the update below reads it from A12)
            for (int c = tid; c < ncol; c += kBatchThreads) {
                T* colp = A + k0 + (k0 + w + c) * n;
                T x[PW];
#pragma unroll
                for (int kk = 0; kk < PW; ++kk) x[kk] = kk < w ? colp[kk] : T(0);
#pragma unroll
                for (int kk = 1; kk < PW; ++kk) {
#pragma unroll
                    for (int jj = 0; jj < kk; ++jj) x[kk] -= pan[kk * LDP + jj] * x[jj];
                    asm volatile("" ::: "memory");  // keeps the loads of later rows from being hoisted
                }
#pragma unroll
                for (int kk = 0; kk < PW; ++kk)
                    if (kk < w) colp[kk] = x[kk];
                if constexpr (kStageU12<T>) {
                    // FP32: U12 also staged in shared memory (row kk at
                    // u12s[kk * kBatchMaxN]), the update below reads it there
#pragma unroll
                    for (int kk = 0; kk < PW; ++kk)
                        if (kk < w) u12s[kk * kBatchMaxN + c] = x[kk];
                }
            }
            __syncthreads();
            // A22 -= L21 U12: 4x4 tiles, a tile's rows strided by ti so that
            // consecutive threads read consecutive panel rows
            const int m2 = m - w;
            const int ti = (m2 + 3) / 4, tj = (ncol + 3) / 4;
            for (int t = tid; t < ti * tj; t += kBatchThreads) {
                const int iq = t % ti, j0 = (t / ti) * 4;
                T acc[4][4];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
                // FP32: the tile's C entries are loaded before the products,
                // so their latency overlaps them (each C entry is this
                // thread's alone, and the products read shared memory only)
                float cv[4][4];
                if constexpr (kStageU12<T>) {
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const T* cp = A + (k0 + w) + (k0 + w + j0 + b) * n;
#pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            const int ra = iq + a * ti;
                            cv[a][b] = (j0 + b < ncol && ra < m2) ? (float)cp[ra] : 0.f;
                        }
                    }
                }
                const T* u = A + k0 + (k0 + w + j0) * n;
                for (int kk = 0; kk < w; ++kk) {
                    T av[4], bv[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int ra = iq + a * ti;
                        av[a] = ra < m2 ? pan[(w + ra) * LDP + kk] : T(0);
                    }
                    if constexpr (kStageU12<T>) {
#pragma unroll
                        for (int b = 0; b < 4; ++b) bv[b] = (j0 + b < ncol) ? u12s[kk * kBatchMaxN + j0 + b] : T(0);
                    } else {
#pragma unroll
                        for (int b = 0; b < 4; ++b) bv[b] = (j0 + b < ncol) ? u[kk + b * n] : T(0);
                    }
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
                }
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    if (j0 + b >= ncol) continue;
                    T* cp = A + (k0 + w) + (k0 + w + j0 + b) * n;
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int ra = iq + a * ti;
                        if (ra < m2) {
                            if constexpr (kStageU12<T>) cp[ra] = (T)cv[a][b] - acc[a][b];
                            else cp[ra] -= acc[a][b];
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

// x := U^-1 L^-1 x for the r right-hand sides staged in shared memory (xs,
// stride XS) with the LU factors of one system (LU, n x n column-major), in
// the arithmetic and zero skipping of TMV's column-oriented vector solve
// (src/TMV_TriDiv_V.cpp:148-236, 322-398), blocked by kSolveBlock columns:
// one warp solves the diagonal block (staged in dg, a lane per right-hand
// side), then every thread updates its (row, rhs) entries below (or above)
// the block over the block's columns in TMV's order, streaming the factor
// from global memory.  A zero U(j,j) that divides a nonzero sets *sing.
template <typename T>
__device__ void lu_solve_staged(int64_t n, int64_t r, const T* __restrict__ LU, T* xs, int XS, T* dg,
                                int* sing)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int DS = kSolveBlock + 1;
    // factor entries a thread loads ahead of their (zero-skipping) use
    constexpr int PF = sizeof(T) == 8 ? 8 : 16;
    static_assert(kSolveBlock % PF == 0, "whole prefetch groups");
    // the diagonal block into dg, eight loads in flight per thread
    auto stage = [&](int j0, int jb) {
        for (int t0 = tid; t0 < jb * jb; t0 += kBatchThreads * 8) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int t = t0 + u * kBatchThreads;
                v[u] = t < jb * jb ? LU[(j0 + t % jb) + (int64_t)(j0 + t / jb) * n] : T(0);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int t = t0 + u * kBatchThreads;
                if (t < jb * jb) dg[(t % jb) * DS + t / jb] = v[u];
            }
        }
    };
        // forward: unit lower L
        for (int j0 = 0; j0 < n; j0 += kSolveBlock) {
            const int jb = (int)min((int64_t)kSolveBlock, n - j0);
            stage(j0, jb);
            __syncthreads();
            if (warp == 0 && lane < r) {
                T* xq = xs + lane * XS + j0;
                for (int k = 0; k < jb; ++k) {
                    const T xk = xq[k];
                    if (nz(xk))
                        for (int i = k + 1; i < jb; ++i) xq[i] -= dg[i * DS + k] * xk;
                }
            }
            __syncthreads();
            const int below = (int)(n - j0 - jb);
            for (int t = tid; t < below * r; t += kBatchThreads) {
                const int i = j0 + jb + t % below, q = t / below;
                const T* xq = xs + q * XS + j0;
                const T* lc = LU + i + (int64_t)j0 * n;
                T v = xs[q * XS + i];
                for (int k0 = 0; k0 < jb; k0 += PF) {
                    T lv[PF];
#pragma unroll
                    for (int u = 0; u < PF; ++u) lv[u] = k0 + u < jb ? lc[(int64_t)(k0 + u) * n] : T(0);
#pragma unroll
                    for (int u = 0; u < PF; ++u) {
                        const T xk = k0 + u < jb ? xq[k0 + u] : T(0);
                        if (nz(xk)) v -= lv[u] * xk;
                    }
                }
                xs[q * XS + i] = v;
            }
            __syncthreads();
        }
        // backward: upper U, columns from the last
        for (int j1 = (int)n; j1 > 0; j1 -= kSolveBlock) {
            const int j0 = max(0, j1 - kSolveBlock), jb = j1 - j0;
            stage(j0, jb);
            __syncthreads();
            if (warp == 0 && lane < r) {
                T* xq = xs + lane * XS + j0;
                for (int k = jb - 1; k >= 0; --k) {
                    T v = xq[k];
                    if (nz(v)) {
                        const T d = dg[k * DS + k];
                        if (!nz(d)) *sing = 1;
                        else xq[k] = v = v / d;
                    }
                    if (nz(v))
                        for (int i = 0; i < k; ++i) xq[i] -= dg[i * DS + k] * v;
                }
            }
            __syncthreads();
            for (int t = tid; t < j0 * r; t += kBatchThreads) {
                const int i = t % j0, q = t / j0;
                const T* xq = xs + q * XS + j0;
                const T* uc = LU + i + (int64_t)j0 * n;
                T v = xs[q * XS + i];
                // columns from the last, as before: groups of PF taken from
                // the top of the block down
                for (int kt = jb; kt > 0; kt -= PF) {
                    T uv[PF];
#pragma unroll
                    for (int u = 0; u < PF; ++u) {
                        const int k = kt - 1 - u;
                        uv[u] = k >= 0 ? uc[(int64_t)k * n] : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < PF; ++u) {
                        const int k = kt - 1 - u;
                        const T xk = k >= 0 ? xq[k] : T(0);
                        if (nz(xk)) v -= uv[u] * xk;
                    }
                }
                xs[q * XS + i] = v;
            }
            __syncthreads();
        }
}

template <int PW>
__device__ void factor_solve_one(int64_t n, int64_t r, double* __restrict__ A, double* __restrict__ B,
                                 int64_t* __restrict__ P, int* __restrict__ status, double* smem)
{
    __shared__ int s_sing;
    const int tid = threadIdx.x;
    if (tid == 0) s_sing = 0;
    factor_one<double, PW>(n, r, A, B, P, smem);

    // Solve: B holds P B; L (unit) then U (lu_solve_staged)
    if (r > 0) {
        constexpr int XS = kBatchMaxN + 1;                  // padded rhs stride
        double* xs = smem;                                   // [kBatchMaxRhs][XS]
        double* dg = smem + kBatchMaxRhs * XS;               // [kSolveBlock][kSolveBlock + 1]
        for (int t = tid; t < n * r; t += kBatchThreads) {
            const int i = t % n, q = t / n;
            xs[q * XS + i] = B[i + q * n];
        }
        __syncthreads();
        lu_solve_staged<double>(n, r, A, xs, XS, dg, &s_sing);
        for (int t = tid; t < n * r; t += kBatchThreads) {
            const int i = t % n, q = t / n;
            B[i + q * n] = xs[q * XS + i];
        }
    }
    __syncthreads();
    if (tid == 0) *status = s_sing;
}

__global__ void __launch_bounds__(kBatchThreads, 4)
batched_lu_kernel(const BatchDev* __restrict__ args, unsigned* queue)
{
    extern __shared__ __align__(16) double bsmem[];
    __shared__ int s_item;
    const BatchDev& a = *args;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= a.count) return;
        const int s = a.order[item];
        const int64_t n = a.n[s], r = a.nrhs[s];
        double* A = a.A + a.a_off[s];
        double* B = a.B + a.b_off[s];
        int64_t* P = a.P + a.p_off[s];
        int* st = a.status + s;
        if (a.pw[size_class(n)] == 8) factor_solve_one<8>(n, r, A, B, P, st, bsmem);
        else factor_solve_one<16>(n, r, A, B, P, st, bsmem);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------
// Mixed precision: FP32 factors, FP64 refinement, one persistent launch.
//
// Per system: As = (float) A together with ||A||_inf (TMV's norm: the
// largest row sum of |a_ij|); the blocked LU of As (factor_one<float>, pivot
// keys compared in FP64); then x = 0 and, until every column's normwise
// backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol:
// r = b - A x accumulated in FP64 (A, b and x in FP64), stored as FP32 in the
// pivoted order, d = U^-1 L^-1 r in FP32 (lu_solve_staged<float>), x += d in
// FP64.  A and b are not modified; x goes to B at the end.  status: 0
// converged, 1 a zero U(j,j) of the FP32 factors met a nonzero, 2 not
// converged within max_iter corrections (B holds the last iterate).
// ---------------------------------------------------------------------
__device__ __forceinline__ void smem_max_abs(unsigned long long* slot, double v)
{
    // non-negative doubles order like their bit patterns; a NaN is kept as NaN
    const double a = fabs(v);
    atomicMax(slot, (unsigned long long)__double_as_longlong(a != a ? __longlong_as_double(0x7ff8000000000000LL) : a));
}

// max(|a|, |b|) with a NaN kept
__device__ __forceinline__ double nan_max_abs(double a, double b)
{
    const double x = fabs(a), y = fabs(b);
    return (x != x || y != y) ? __longlong_as_double(0x7ff8000000000000LL) : fmax(x, y);
}

template <int PW>
__device__ void mixed_one(const BatchDev& d, int s, unsigned char* smem_raw)
{
    constexpr int XS = kBatchMaxN + 1;
    constexpr int RPT = kBatchMaxN / kBatchThreads;  // rows per thread in the residual
    static_assert(RPT == 2, "the residual loop handles two row blocks");
    __shared__ unsigned long long s_anorm;
    __shared__ unsigned long long s_bn[kBatchMaxRhs], s_rn[kBatchMaxRhs], s_xn[kBatchMaxRhs];
    __shared__ int s_inv[kBatchMaxN];  // row i of r goes to position s_inv[i] of P r
    __shared__ int s_sing, s_done;

    const int tid = threadIdx.x;
    const int64_t n = d.n[s], r = d.nrhs[s];
    const double* __restrict__ A = d.A + d.a_off[s];
    double* __restrict__ B = d.B + d.b_off[s];
    float* __restrict__ As = d.As + d.a_off[s];
    int64_t* __restrict__ P = d.P + d.p_off[s];

    // 1. FP32 copy and ||A||_inf
    if (tid == 0) { s_anorm = 0ull; s_sing = 0; s_done = 0; }
    __syncthreads();
    for (int i = tid; i < n; i += kBatchThreads) {
        double rs = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            const double v = A[i + j * n];
            As[i + j * n] = (float)v;
            rs += fabs(v);
        }
        smem_max_abs(&s_anorm, rs);
    }
    __syncthreads();
    // 2. FP32 factorisation (interchanges on As only: b stays in place)
    factor_one<float, PW>(n, 0, As, nullptr, P, reinterpret_cast<float*>(smem_raw));
    __syncthreads();
    // the gather of P r: apply the interchanges to the identity, invert
    if (tid == 0) {
        for (int i = 0; i < n; ++i) s_inv[i] = i;  // s_inv used as perm first
        for (int k = 0; k < n; ++k) {
            const int p = (int)P[k];
            const int t = s_inv[k];
            s_inv[k] = s_inv[p];
            s_inv[p] = t;
        }
    }
    __syncthreads();
    int perm_of[RPT];
#pragma unroll
    for (int u = 0; u < RPT; ++u) perm_of[u] = tid + u * kBatchThreads < n ? s_inv[tid + u * kBatchThreads] : 0;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < RPT; ++u)
        if (tid + u * kBatchThreads < n) s_inv[perm_of[u]] = tid + u * kBatchThreads;
    __syncthreads();

    double* xs = reinterpret_cast<double*>(smem_raw);          // x: [kBatchMaxRhs][XS] FP64
    float* ds = reinterpret_cast<float*>(xs + kBatchMaxRhs * XS);  // r, then d: [kBatchMaxRhs][XS] FP32
    float* dg = ds + kBatchMaxRhs * XS;                          // [kSolveBlock][kSolveBlock + 1]
    for (int t = tid; t < kBatchMaxRhs * XS; t += kBatchThreads) xs[t] = 0.0;
    if (tid < kBatchMaxRhs) s_bn[tid] = 0ull;
    __syncthreads();
    for (int t = tid; t < n * r; t += kBatchThreads) smem_max_abs(&s_bn[t / n], B[t % n + (t / n) * n]);
    const double anorm = __longlong_as_double((long long)s_anorm);
    int it = 0;
    for (;; ++it) {
        if (tid < kBatchMaxRhs) { s_rn[tid] = 0ull; s_xn[tid] = 0ull; }
        __syncthreads();
        // r = b - A x (FP64), into ds in the pivoted order, and its norms
        double acc[RPT][kBatchMaxRhs];
#pragma unroll
        for (int u = 0; u < RPT; ++u)
#pragma unroll
            for (int q = 0; q < kBatchMaxRhs; ++q) {
                const int i = tid + u * kBatchThreads;
                acc[u][q] = (q < r && i < n) ? B[i + q * n] : 0.0;
            }
        // warps whose rows all lie beyond n skip their FMAs (FP64 issue is
        // the bound here): the second row block only when n > 128
        if (it > 0 && (tid & ~31) < n) {
            const bool two = kBatchThreads + (tid & ~31) < n;
            for (int64_t j = 0; j < n; ++j) {
                const int i0 = tid, i1 = tid + kBatchThreads;
                const double a0 = i0 < n ? __ldg(A + i0 + j * n) : 0.0;
                if (two) {
                    const double a1 = i1 < n ? __ldg(A + i1 + j * n) : 0.0;
#pragma unroll
                    for (int q = 0; q < kBatchMaxRhs; ++q) {
                        if (q >= r) break;
                        const double xq = xs[q * XS + j];
                        acc[0][q] = fma(-a0, xq, acc[0][q]);
                        acc[1][q] = fma(-a1, xq, acc[1][q]);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < kBatchMaxRhs; ++q) {
                        if (q >= r) break;
                        acc[0][q] = fma(-a0, xs[q * XS + j], acc[0][q]);
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kBatchMaxRhs; ++q) {
            if (q >= r) break;
            double rm = 0.0, xm = 0.0;
#pragma unroll
            for (int u = 0; u < RPT; ++u) {
                const int i = tid + u * kBatchThreads;
                if (i >= n) continue;
                ds[q * XS + s_inv[i]] = (float)acc[u][q];
                rm = nan_max_abs(rm, acc[u][q]);
                xm = nan_max_abs(xm, xs[q * XS + i]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                rm = nan_max_abs(rm, __shfl_xor_sync(0xffffffffu, rm, o));
                xm = nan_max_abs(xm, __shfl_xor_sync(0xffffffffu, xm, o));
            }
            if ((tid & 31) == 0) {
                smem_max_abs(&s_rn[q], rm);
                smem_max_abs(&s_xn[q], xm);
            }
        }
        __syncthreads();
        // every column's backward error
        if (tid == 0) {
            double worst = 0.0;
            bool ok = true;
            for (int q = 0; q < r; ++q) {
                const double rn = __longlong_as_double((long long)s_rn[q]);
                const double den = anorm * __longlong_as_double((long long)s_xn[q]) +
                                   __longlong_as_double((long long)s_bn[q]);
                const double be = den > 0.0 ? rn / den : (rn > 0.0 ? INFINITY : 0.0);
                if (!(be <= d.tol)) ok = false;
                if (!(be <= worst)) worst = be;  // NaN propagates
            }
            if (d.berr) d.berr[s] = worst;
            s_done = (ok || s_sing || it >= d.max_iter) ? 1 : 0;
            if (!ok && !s_sing && it >= d.max_iter) s_done = 2;
        }
        __syncthreads();
        if (s_done) break;
        // d = U^-1 L^-1 (P r) in FP32; x += d in FP64
        lu_solve_staged<float>(n, r, As, ds, XS, dg, &s_sing);
        __syncthreads();
        for (int t = tid; t < n * r; t += kBatchThreads) {
            const int i = t % n, q = t / n;
            xs[q * XS + i] += (double)ds[q * XS + i];
        }
        __syncthreads();
    }
    for (int t = tid; t < n * r; t += kBatchThreads) {
        const int i = t % n, q = t / n;
        B[i + q * n] = xs[q * XS + i];
    }
    if (tid == 0) {
        d.status[s] = s_sing ? 1 : (s_done == 2 ? 2 : 0);
        if (d.iters) d.iters[s] = it;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kBatchThreads, 4)
batched_mixed_kernel(const BatchDev* __restrict__ args, unsigned* queue)
{
    extern __shared__ __align__(16) unsigned char bsmem_mixed[];
    __shared__ int s_item;
    const BatchDev& a = *args;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= a.count) return;
        const int s = a.order[item];
        if (a.pw[size_class(a.n[s])] == 8) mixed_one<8>(a, s, bsmem_mixed);
        else mixed_one<16>(a, s, bsmem_mixed);
    }
}

// ---------------------------------------------------------------------
// Plan: descriptors on the device, processing order, tile choice, graph.
// ---------------------------------------------------------------------
struct BatchPlan {
    Context* c = nullptr;
    int64_t count = 0;
    int64_t a_elems = 0, b_elems = 0, p_elems = 0;
    int64_t* d_desc = nullptr;  // n, nrhs, a_off, b_off, p_off (5 * count)
    int* d_order = nullptr;
    BatchDev* d_args = nullptr;
    BatchDev* h_args = nullptr;  // pinned
    unsigned* d_queue = nullptr;
    int grid = 0;
    size_t smem = 0;
    int pw[kNumClasses] = {16, 16, 16, 16};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // mixed precision: FP32 factors (a_elems floats), its own graph
    float* d_As = nullptr;
    cudaGraph_t graph_mixed = nullptr;
    cudaGraphExec_t exec_mixed = nullptr;
    int grid_mixed = 0;
    size_t smem_mixed = 0;
    double flops = 0;
    std::vector<int64_t> hn, hr;
};

static size_t smem_for(const int pw[kNumClasses])
{
    int mx = 8;
    for (int k = 0; k < kNumClasses; ++k) mx = std::max(mx, pw[k]);
    // the factorisation's panel and U12, or the solve's right-hand sides and
    // diagonal block, whichever is larger
    const int solve = kBatchMaxRhs * (kBatchMaxN + 1) + kSolveBlock * (kSolveBlock + 1);
    return sizeof(double) * (size_t)std::max(batch_smem_doubles(mx), solve);
}

static tmvg_status build_graph(BatchPlan* p)
{
    Context* c = p->c;
    if (p->exec) { cudaGraphExecDestroy(p->exec); p->exec = nullptr; }
    if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
    p->smem = smem_for(p->pw);
    tmvg_status st = check_cuda(
        c, cudaFuncSetAttribute(batched_lu_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)p->smem),
        "batched: smem attribute");
    if (st) return st;
    int per_sm = 0;
    st = check_cuda(c,
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_lu_kernel,
                                                                  kBatchThreads, p->smem),
                    "batched: occupancy");
    if (st) return st;
    per_sm = std::max(per_sm, 1);
    p->grid = (int)std::min<int64_t>((int64_t)per_sm * c->num_sms, std::max<int64_t>(p->count, 1));
    // capture: reset the queue, run the persistent kernel
    cudaStream_t cap;
    st = check_cuda(c, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "batched: stream");
    if (st) return st;
    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned), cap);
    batched_lu_kernel<<<p->grid, kBatchThreads, p->smem, cap>>>(p->d_args, p->d_queue);
    cudaError_t e = cudaStreamEndCapture(cap, &p->graph);
    cudaStreamDestroy(cap);
    st = check_cuda(c, e, "batched: capture");
    if (st) return st;
    return check_cuda(c, cudaGraphInstantiate(&p->exec, p->graph, 0), "batched: instantiate");
}

// Shared memory of the mixed kernel: the FP32 panel, or the refinement's
// FP64 iterate, FP32 correction and FP32 diagonal block.
static size_t smem_mixed_bytes()
{
    const size_t panel = sizeof(float) * ((size_t)batch_smem_doubles(16) + 16 * kBatchMaxN);
    const size_t refine = sizeof(double) * kBatchMaxRhs * (kBatchMaxN + 1) +
                          sizeof(float) * (kBatchMaxRhs * (kBatchMaxN + 1) + kSolveBlock * (kSolveBlock + 1));
    return std::max(panel, refine);
}

static tmvg_status build_graph_mixed(BatchPlan* p)
{
    Context* c = p->c;
    if (p->exec_mixed) { cudaGraphExecDestroy(p->exec_mixed); p->exec_mixed = nullptr; }
    if (p->graph_mixed) { cudaGraphDestroy(p->graph_mixed); p->graph_mixed = nullptr; }
    p->smem_mixed = smem_mixed_bytes();
    tmvg_status st = check_cuda(
        c, cudaFuncSetAttribute(batched_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)p->smem_mixed),
        "batched mixed: smem attribute");
    if (st) return st;
    int per_sm = 0;
    st = check_cuda(c,
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_mixed_kernel, kBatchThreads,
                                                                  p->smem_mixed),
                    "batched mixed: occupancy");
    if (st) return st;
    per_sm = std::max(per_sm, 1);
    p->grid_mixed = (int)std::min<int64_t>((int64_t)per_sm * c->num_sms, std::max<int64_t>(p->count, 1));
    cudaStream_t cap;
    st = check_cuda(c, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "batched mixed: stream");
    if (st) return st;
    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    cudaMemsetAsync(p->d_queue, 0, sizeof(unsigned), cap);
    batched_mixed_kernel<<<p->grid_mixed, kBatchThreads, p->smem_mixed, cap>>>(p->d_args, p->d_queue);
    cudaError_t e = cudaStreamEndCapture(cap, &p->graph_mixed);
    cudaStreamDestroy(cap);
    st = check_cuda(c, e, "batched mixed: capture");
    if (st) return st;
    return check_cuda(c, cudaGraphInstantiate(&p->exec_mixed, p->graph_mixed, 0), "batched mixed: instantiate");
}

static void fill_args(BatchPlan* p, double* A, double* B, int64_t* P, int* status)
{
    BatchDev& h = *p->h_args;
    h.n = p->d_desc;
    h.nrhs = p->d_desc + p->count;
    h.a_off = p->d_desc + 2 * p->count;
    h.b_off = p->d_desc + 3 * p->count;
    h.p_off = p->d_desc + 4 * p->count;
    h.order = p->d_order;
    h.A = A;
    h.B = B;
    h.P = P;
    h.status = status;
    h.count = p->count;
    for (int k = 0; k < kNumClasses; ++k) h.pw[k] = p->pw[k];
    h.As = nullptr;
    h.max_iter = 0;
    h.tol = 0.0;
    h.iters = nullptr;
    h.berr = nullptr;
}

static tmvg_status run_plan_mixed(BatchPlan* p, const double* A, double* B, int64_t* P, int* status,
                                  int max_iter, double tol, int* iters, double* berr)
{
    Context* c = p->c;
    if (!p->d_As) {
        if (cudaMalloc(&p->d_As, sizeof(float) * (size_t)std::max<int64_t>(p->a_elems, 1)) != cudaSuccess) {
            cudaGetLastError();
            p->d_As = nullptr;
            return set_error(c, TMVG_OOM, "batched mixed: FP32 factors");
        }
    }
    if (!p->exec_mixed) {
        tmvg_status st = build_graph_mixed(p);
        if (st) return st;
    }
    fill_args(p, const_cast<double*>(A), B, P, status);
    BatchDev& h = *p->h_args;
    h.As = p->d_As;
    h.max_iter = max_iter;
    h.tol = tol;
    h.iters = iters;
    h.berr = berr;
    tmvg_status st = check_cuda(
        c, cudaMemcpyAsync(p->d_args, p->h_args, sizeof(BatchDev), cudaMemcpyHostToDevice, c->stream),
        "batched mixed: args");
    if (st) return st;
    st = check_cuda(c, cudaGraphLaunch(p->exec_mixed, c->stream), "batched mixed: graph launch");
    if (st) return st;
    c->launches += 1;
    return check_cuda(c, cudaStreamSynchronize(c->stream), "batched mixed: sync");
}

static tmvg_status run_plan(BatchPlan* p, double* A, double* B, int64_t* P, int* status)
{
    Context* c = p->c;
    fill_args(p, A, B, P, status);
    tmvg_status st = check_cuda(
        c, cudaMemcpyAsync(p->d_args, p->h_args, sizeof(BatchDev), cudaMemcpyHostToDevice, c->stream),
        "batched: args");
    if (st) return st;
    st = check_cuda(c, cudaGraphLaunch(p->exec, c->stream), "batched: graph launch");
    if (st) return st;
    c->launches += 1;
    // the pinned argument block must not change before the copy has run
    return check_cuda(c, cudaStreamSynchronize(c->stream), "batched: sync");
}

// The tuner's results persist in a small text table keyed by the device
// (name and SM count) and the size class, so that a plan on the same kind of
// GPU takes its panel widths without timing them again: one line
// "<sms> <class> <width> <ms> <device name>" per entry.  The file is
// $TMVG_TUNE_CACHE ("off" or empty: no table), by default tmvg_tune_cache.txt
// beside this library.
static std::string tune_cache_path()
{
    if (const char* e = std::getenv("TMVG_TUNE_CACHE")) {
        if (!*e || std::strcmp(e, "off") == 0) return std::string();
        return std::string(e);
    }
    Dl_info info;
    if (dladdr((void*)&tune_cache_path, &info) && info.dli_fname) {
        std::string lib(info.dli_fname);
        const size_t slash = lib.rfind('/');
        return (slash == std::string::npos ? std::string(".") : lib.substr(0, slash)) + "/tmvg_tune_cache.txt";
    }
    return std::string();
}

struct TuneEntry {
    int sms, cls, width;
    float ms;
    std::string device;
};

static std::vector<TuneEntry> read_tune_cache(const std::string& path)
{
    std::vector<TuneEntry> out;
    if (path.empty()) return out;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return out;
    char line[512];
    while (std::fgets(line, sizeof(line), f)) {
        TuneEntry e;
        int used = 0;
        if (std::sscanf(line, "%d %d %d %f %n", &e.sms, &e.cls, &e.width, &e.ms, &used) < 4) continue;
        if (e.cls < 0 || e.cls >= kNumClasses || (e.width != 8 && e.width != 16)) continue;
        e.device = std::string(line + used);
        while (!e.device.empty() && (e.device.back() == '\n' || e.device.back() == '\r')) e.device.pop_back();
        out.push_back(e);
    }
    std::fclose(f);
    return out;
}

static void write_tune_cache(const std::string& path, const std::vector<TuneEntry>& es)
{
    if (path.empty()) return;
    const std::string tmp = path + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) return;  // a read-only location: the table is an optimisation only
    for (const TuneEntry& e : es) std::fprintf(f, "%d %d %d %.4f %s\n", e.sms, e.cls, e.width, e.ms, e.device.c_str());
    const bool ok = std::fclose(f) == 0;
    if (ok) std::rename(tmp.c_str(), path.c_str());
    else std::remove(tmp.c_str());
}

// Time each panel width on the systems of each size class (a sample of at
// most 256 of them, on scratch copies) and keep the fastest; a class already
// in the persisted table for this device takes its width from there.
static tmvg_status tune(BatchPlan* p)
{
    Context* c = p->c;
    const int cand[2] = {8, 16};
    const std::string cache = tune_cache_path();
    std::vector<TuneEntry> table = read_tune_cache(cache);
    cudaDeviceProp prop;
    std::string dev_name = "unknown";
    if (cudaGetDeviceProperties(&prop, c->device) == cudaSuccess) dev_name = prop.name;
    else cudaGetLastError();
    bool table_changed = false;
    std::vector<std::vector<int64_t>> members(kNumClasses);
    for (int64_t s = 0; s < p->count; ++s) members[size_class(p->hn[s])].push_back(s);
    for (int k = 0; k < kNumClasses; ++k) {
        if (members[k].empty()) continue;
        bool cached = false;
        for (const TuneEntry& e : table)
            if (e.sms == c->num_sms && e.cls == k && e.device == dev_name) {
                p->pw[k] = e.width;
                cached = true;
                break;
            }
        if (cached) continue;
        const size_t take = std::min<size_t>(members[k].size(), 256);
        // scratch sub-batch: packed copies of the sampled systems
        std::vector<int64_t> n(take), r(take), ao(take), bo(take), po(take);
        int64_t A_el = 0, B_el = 0, P_el = 0;
        for (size_t i = 0; i < take; ++i) {
            const int64_t s = members[k][i];
            n[i] = p->hn[s]; r[i] = p->hr[s];
            ao[i] = A_el; bo[i] = B_el; po[i] = P_el;
            A_el += n[i] * n[i]; B_el += n[i] * r[i]; P_el += n[i];
        }
        BatchPlan sub;
        sub.c = c;
        sub.count = (int64_t)take;
        tmvg_status st = TMVG_OK;
        double *dA = nullptr, *dB = nullptr;
        int64_t* dP = nullptr;
        int* dS = nullptr;
        if (cudaMalloc(&sub.d_desc, sizeof(int64_t) * 5 * take) != cudaSuccess ||
            cudaMalloc(&sub.d_order, sizeof(int) * take) != cudaSuccess ||
            cudaMalloc(&sub.d_args, sizeof(BatchDev)) != cudaSuccess ||
            cudaMallocHost(&sub.h_args, sizeof(BatchDev)) != cudaSuccess ||
            cudaMalloc(&sub.d_queue, sizeof(unsigned)) != cudaSuccess ||
            cudaMalloc(&dA, sizeof(double) * std::max<int64_t>(A_el, 1)) != cudaSuccess ||
            cudaMalloc(&dB, sizeof(double) * std::max<int64_t>(B_el, 1)) != cudaSuccess ||
            cudaMalloc(&dP, sizeof(int64_t) * std::max<int64_t>(P_el, 1)) != cudaSuccess ||
            cudaMalloc(&dS, sizeof(int) * take) != cudaSuccess) {
            cudaGetLastError();
            st = set_error(c, TMVG_OOM, "batched tuning: scratch");
        }
        if (!st) {
            std::vector<int64_t> desc;
            desc.insert(desc.end(), n.begin(), n.end());
            desc.insert(desc.end(), r.begin(), r.end());
            desc.insert(desc.end(), ao.begin(), ao.end());
            desc.insert(desc.end(), bo.begin(), bo.end());
            desc.insert(desc.end(), po.begin(), po.end());
            std::vector<int> ord(take);
            std::iota(ord.begin(), ord.end(), 0);
            cudaMemcpy(sub.d_desc, desc.data(), sizeof(int64_t) * desc.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(sub.d_order, ord.data(), sizeof(int) * take, cudaMemcpyHostToDevice);
            // diagonally dominant test systems (values only affect pivoting)
            std::vector<double> hA(A_el), hB(B_el, 1.0);
            uint64_t x = 88172645463325252ull;
            for (int64_t i = 0; i < A_el; ++i) {
                x ^= x << 13; x ^= x >> 7; x ^= x << 17;
                hA[i] = (double)(x >> 11) * (1.0 / 9007199254740992.0) - 0.5;
            }
            for (size_t i = 0; i < take; ++i)
                for (int64_t d = 0; d < n[i]; ++d) hA[ao[i] + d * (n[i] + 1)] += 2.0 * n[i];
            float best_ms = 1e30f;
            int best = 16;
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            for (int ci = 0; ci < 2 && !st; ++ci) {
                for (int q = 0; q < kNumClasses; ++q) sub.pw[q] = cand[ci];
                st = build_graph(&sub);
                if (st) break;
                float ms_sum = 0;
                for (int rep = 0; rep < 2 && !st; ++rep) {
                    cudaMemcpy(dA, hA.data(), sizeof(double) * A_el, cudaMemcpyHostToDevice);
                    cudaMemcpy(dB, hB.data(), sizeof(double) * B_el, cudaMemcpyHostToDevice);
                    cudaEventRecord(e0, c->stream);
                    st = run_plan(&sub, dA, dB, dP, dS);
                    cudaEventRecord(e1, c->stream);
                    cudaEventSynchronize(e1);
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep == 1) ms_sum += ms;
                }
                if (!st && ms_sum < best_ms) { best_ms = ms_sum; best = cand[ci]; }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            p->pw[k] = best;
            if (!st) {
                table.push_back({c->num_sms, k, best, best_ms, dev_name});
                table_changed = true;
            }
        }
        if (sub.exec) cudaGraphExecDestroy(sub.exec);
        if (sub.graph) cudaGraphDestroy(sub.graph);
        cudaFree(sub.d_desc); cudaFree(sub.d_order); cudaFree(sub.d_args);
        if (sub.h_args) cudaFreeHost(sub.h_args);
        cudaFree(sub.d_queue); cudaFree(dA); cudaFree(dB); cudaFree(dP); cudaFree(dS);
        if (st) return st;
    }
    if (table_changed) write_tune_cache(cache, table);
    return TMVG_OK;
}

}  // namespace tmvg

using namespace tmvg;

extern "C" {

tmvg_status tmvg_batch_plan_create(tmvg_handle h, int64_t count, const int64_t* n,
                                   const int64_t* nrhs, const int64_t* a_off, const int64_t* b_off,
                                   int tune_tiles, tmvg_batch_plan* plan)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c || !plan || count < 0 || (count > 0 && (!n || !nrhs))) return TMVG_BAD_ARG;
    *plan = nullptr;
    c->last_error.clear();
    cudaSetDevice(c->device);
    if (count > INT_MAX) return set_error(c, TMVG_UNSUPPORTED, "batch: too many systems");
    BatchPlan* p = new BatchPlan();
    p->c = c;
    p->count = count;
    p->hn.assign(n, n + count);
    p->hr.assign(nrhs, nrhs + count);
    std::vector<int64_t> desc(5 * count);
    int64_t A_el = 0, B_el = 0, P_el = 0;
    for (int64_t s = 0; s < count; ++s) {
        if (n[s] < 1 || n[s] > kBatchMaxN || nrhs[s] < 0 || nrhs[s] > kBatchMaxRhs) {
            delete p;
            return set_error(c, TMVG_UNSUPPORTED,
                             "batch: each system needs 1 <= n <= 256 and 0 <= nrhs <= 16");
        }
        desc[s] = n[s];
        desc[count + s] = nrhs[s];
        desc[2 * count + s] = a_off ? a_off[s] : A_el;
        desc[3 * count + s] = b_off ? b_off[s] : B_el;
        desc[4 * count + s] = P_el;
        A_el = std::max(A_el, desc[2 * count + s] + n[s] * n[s]);
        B_el = std::max(B_el, desc[3 * count + s] + n[s] * nrhs[s]);
        P_el += n[s];
        p->flops += 2.0 * n[s] * n[s] * n[s] / 3.0 + 2.0 * n[s] * n[s] * nrhs[s];
    }
    p->a_elems = A_el;
    p->b_elems = B_el;
    p->p_elems = P_el;
    // largest systems first
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
    tmvg_status st = TMVG_OK;
    if (cudaMalloc(&p->d_desc, sizeof(int64_t) * std::max<int64_t>(5 * count, 1)) != cudaSuccess ||
        cudaMalloc(&p->d_order, sizeof(int) * std::max<int64_t>(count, 1)) != cudaSuccess ||
        cudaMalloc(&p->d_args, sizeof(BatchDev)) != cudaSuccess ||
        cudaMallocHost(&p->h_args, sizeof(BatchDev)) != cudaSuccess ||
        cudaMalloc(&p->d_queue, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        st = set_error(c, TMVG_OOM, "batch plan allocation");
    }
    if (!st && count > 0) {
        st = check_cuda(c, cudaMemcpy(p->d_desc, desc.data(), sizeof(int64_t) * 5 * count,
                                      cudaMemcpyHostToDevice), "batch desc upload");
        if (!st)
            st = check_cuda(c, cudaMemcpy(p->d_order, order.data(), sizeof(int) * count,
                                          cudaMemcpyHostToDevice), "batch order upload");
    }
    if (!st && tune_tiles && count > 0) st = tune(p);
    if (!st) st = build_graph(p);
    if (st) {
        tmvg_batch_plan_destroy(reinterpret_cast<tmvg_batch_plan>(p));
        return st;
    }
    *plan = reinterpret_cast<tmvg_batch_plan>(p);
    return TMVG_OK;
}

tmvg_status tmvg_batch_plan_info(tmvg_batch_plan plan, int64_t* a_elems, int64_t* b_elems,
                                 int64_t* p_elems, double* flops, int* panel_widths)
{
    BatchPlan* p = reinterpret_cast<BatchPlan*>(plan);
    if (!p) return TMVG_BAD_ARG;
    if (a_elems) *a_elems = p->a_elems;
    if (b_elems) *b_elems = p->b_elems;
    if (p_elems) *p_elems = p->p_elems;
    if (flops) *flops = p->flops;
    if (panel_widths)
        for (int k = 0; k < kNumClasses; ++k) panel_widths[k] = p->pw[k];
    return TMVG_OK;
}

tmvg_status tmvg_batch_plan_set_tiles(tmvg_batch_plan plan, const int* panel_widths)
{
    BatchPlan* p = reinterpret_cast<BatchPlan*>(plan);
    if (!p || !panel_widths) return TMVG_BAD_ARG;
    for (int k = 0; k < kNumClasses; ++k) {
        const int w = panel_widths[k];
        if (w != 8 && w != 16) return set_error(p->c, TMVG_BAD_ARG, "panel width must be 8 or 16");
    }
    for (int k = 0; k < kNumClasses; ++k) p->pw[k] = panel_widths[k];
    cudaSetDevice(p->c->device);
    return build_graph(p);
}

tmvg_status tmvg_batched_lu_solve_f64(tmvg_batch_plan plan, double* A, double* B, int64_t* P,
                                      int32_t* status)
{
    BatchPlan* p = reinterpret_cast<BatchPlan*>(plan);
    if (!p) return TMVG_BAD_ARG;
    Context* c = p->c;
    c->last_error.clear();
    cudaSetDevice(c->device);
    if (p->count == 0) return TMVG_OK;
    if (!A || !B || !P || !status) return set_error(c, TMVG_BAD_ARG, "batched: null buffer");
    return run_plan(p, A, B, P, status);
}

tmvg_status tmvg_batched_lu_solve_mixed_f64(tmvg_batch_plan plan, const double* A, double* B, int64_t* P,
                                            int32_t* status, int max_iter, double tol, int32_t* iters,
                                            double* berr)
{
    BatchPlan* p = reinterpret_cast<BatchPlan*>(plan);
    if (!p) return TMVG_BAD_ARG;
    Context* c = p->c;
    c->last_error.clear();
    cudaSetDevice(c->device);
    if (max_iter < 0 || !(tol >= 0.0)) return set_error(c, TMVG_BAD_ARG, "batched mixed: max_iter/tol");
    if (p->count == 0) return TMVG_OK;
    if (!A || !B || !P || !status) return set_error(c, TMVG_BAD_ARG, "batched mixed: null buffer");
    return run_plan_mixed(p, A, B, P, status, max_iter, tol, iters, berr);
}

tmvg_status tmvg_batch_plan_destroy(tmvg_batch_plan plan)
{
    BatchPlan* p = reinterpret_cast<BatchPlan*>(plan);
    if (!p) return TMVG_OK;
    cudaSetDevice(p->c->device);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->exec_mixed) cudaGraphExecDestroy(p->exec_mixed);
    if (p->graph_mixed) cudaGraphDestroy(p->graph_mixed);
    cudaFree(p->d_As);
    cudaFree(p->d_desc);
    cudaFree(p->d_order);
    cudaFree(p->d_args);
    if (p->h_args) cudaFreeHost(p->h_args);
    cudaFree(p->d_queue);
    delete p;
    return TMVG_OK;
}

}  // extern "C"
