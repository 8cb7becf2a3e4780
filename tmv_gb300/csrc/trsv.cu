// trsv.cu -- single-launch triangular solves for few right-hand sides, and
// the interchange-to-permutation conversion used by the solves.
//
// Sync-free blocked substitution: the n rows are cut into 64-row blocks and
// each CTA takes the next block from a ticket counter, so a CTA only ever
// waits on blocks whose tickets were handed out earlier (they are running or
// done: no deadlock whatever the residency).  For its block b the CTA
//   1. for every earlier block j, loads the 64x64 tile T[b, j] into registers
//      (independent of x), waits (bounded) until block j publishes its
//      solution, and accumulates T[b, j] x_j;
//   2. substitutes through the diagonal block with one warp per right-hand
//      side;
//   3. writes x_b and publishes it (release store of the launch's epoch).
// An upper-triangular solve is the same lower solve on index-reversed views
// (negative strides), so the sums are taken in the order of TMV's
// column-oriented vector solve (src/TMV_TriDiv_V.cpp:148-236, 322-398):
// x_i = b_i - sum_j T_ij x_j over j in dependency order.
#include "trsv.cuh"
#include "async.cuh"
#include "pivots.cuh"

#include <type_traits>

#include <algorithm>
#include <vector>

namespace tmvg {

constexpr int kTrsvBlock = 64;
constexpr int kTrsvThreads = 256;
// right-hand sides per launch of the multi-column variant (keeps the static
// shared memory of the FP64 instance under 48 KB)
template <typename T>
constexpr int kTrsvMaxRhs = sizeof(T) == 8 ? 4 : 8;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Inverse of each 64 x 64 lower diagonal block (an upper triangle arrives
// index-reversed), for the many-column solve: one CTA per block, thread j
// builds column j by forward substitution with the diagonal's reciprocals
// (taken once per block).  dinv[b] is row-major 64 x 64; sing[b] = 1 when
// the block has a zero diagonal (that block keeps the substitution, with
// TMV's zero-skipping and singular semantics).
template <typename T>
__global__ void __launch_bounds__(kTrsvBlock)
tri_inv64_kernel(int64_t n, const T* __restrict__ tri, int64_t tsi, int64_t tsj, bool unit,
                 T* __restrict__ dinv, int* __restrict__ sing)
{
    // dynamic shared memory: D and X, each kTrsvBlock x (kTrsvBlock + 1)
    extern __shared__ __align__(16) unsigned char inv_smem[];
    T(*D)[kTrsvBlock + 1] = reinterpret_cast<T(*)[kTrsvBlock + 1]>(inv_smem);
    T(*X)[kTrsvBlock + 1] = D + kTrsvBlock;
    __shared__ T rd[kTrsvBlock];
    __shared__ int s_sing;
    const int tid = threadIdx.x;
    const int64_t b = blockIdx.x, r0 = b * kTrsvBlock;
    const int rows = (int)min((int64_t)kTrsvBlock, n - r0);
    if (tid == 0) s_sing = 0;
    for (int t = tid; t < kTrsvBlock * kTrsvBlock; t += kTrsvBlock) {
        const int rr = t % kTrsvBlock, cc = t / kTrsvBlock;
        D[rr][cc] = (rr < rows && cc <= rr) ? tri[(r0 + rr) * tsi + (r0 + cc) * tsj] : T(0);
    }
    __syncthreads();
    if (!unit && tid < rows) {
        if (D[tid][tid] == T(0)) s_sing = 1;
        else rd[tid] = T(1) / D[tid][tid];
    }
    __syncthreads();
    if (tid == 0) sing[b] = s_sing;
    if (s_sing) return;
    const int j = tid;
    for (int i = 0; i < kTrsvBlock; ++i) {
        T v = T(0);
        if (i < rows && j < rows && i >= j) {
            T acc = i == j ? T(1) : T(0);
            for (int k = j; k < i; ++k) acc -= D[i][k] * X[k][j];
            v = unit ? acc : acc * rd[i];
        }
        X[i][j] = v;
    }
    __syncthreads();
    T* out = dinv + b * kTrsvBlock * kTrsvBlock;
    for (int t = tid; t < kTrsvBlock * kTrsvBlock; t += kTrsvBlock) out[t] = X[t / kTrsvBlock][t % kTrsvBlock];
}

// One CTA per (row block, group of NR right-hand sides); tickets hand the
// pairs out block by block (all groups of block b before block b+1), and a
// CTA waits only on earlier blocks of its own group, so every wait is on a
// ticket already handed out.  flags[g * nblk + b] publishes (b, g).
template <typename T, int NR>
__global__ void __launch_bounds__(kTrsvThreads)
trsm_sync_free_kernel(int64_t n, const T* __restrict__ tri, int64_t tsi, int64_t tsj, bool unit,
                      int64_t nrhs, int groups, T* B, int64_t bsi, int64_t bsj, bool skip_zero,
                      unsigned* flags, unsigned epoch, unsigned long long* ticket,
                      unsigned long long tbase, unsigned spin_limit, int* err,
                      const T* __restrict__ dinv, const int* __restrict__ dinv_sing)
{
    __shared__ long long s_tk;
    __shared__ T xs[kTrsvBlock][NR];
    __shared__ T xj[kTrsvBlock][NR];
    __shared__ T Td[kTrsvBlock][kTrsvBlock + 1];
    __shared__ T part[4][kTrsvBlock][NR];
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    const int i = tid & 63, g = tid >> 6;
    if (tid == 0) {
        s_tk = (long long)(atomicAdd(ticket, 1ull) - tbase);
        s_abort = 0;
    }
    __syncthreads();
    const int64_t nblk = (n + kTrsvBlock - 1) / kTrsvBlock;
    if (s_tk < 0 || s_tk >= nblk * groups) return;
    const int64_t b = s_tk / groups;
    const int grp = (int)(s_tk % groups);
    const int nr = (int)min((int64_t)NR, nrhs - (int64_t)grp * NR);
    B += (int64_t)grp * NR * bsj;
    flags += (int64_t)grp * nblk;
    const int64_t r0 = b * kTrsvBlock;
    const int rows = (int)min((int64_t)kTrsvBlock, n - r0);

    // diagonal block (or its inverse) and right-hand side
    const bool use_inv = dinv != nullptr && dinv_sing[b] == 0;
    if (use_inv) {
        const T* di = dinv + b * kTrsvBlock * kTrsvBlock;
        for (int t = tid; t < kTrsvBlock * kTrsvBlock; t += kTrsvThreads)
            Td[t / kTrsvBlock][t % kTrsvBlock] = di[t];
    } else {
        for (int t = tid; t < kTrsvBlock * kTrsvBlock; t += kTrsvThreads) {
            const int rr = t % kTrsvBlock, cc = t / kTrsvBlock;
            Td[rr][cc] = (rr < rows && cc <= rr) ? tri[(r0 + rr) * tsi + (r0 + cc) * tsj] : T(0);
        }
    }
    for (int t = tid; t < kTrsvBlock * NR; t += kTrsvThreads) {
        const int rr = t % kTrsvBlock, q = t / kTrsvBlock;
        xs[rr][q] = (rr < rows && q < nr) ? B[(r0 + rr) * bsi + q * bsj] : T(0);
    }

    T acc[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = T(0);

    for (int64_t j = 0; j < b; ++j) {
        const int64_t c0 = j * kTrsvBlock;
        T a[16];
#pragma unroll
        for (int c = 0; c < 16; ++c)
            a[c] = (i < rows) ? tri[(r0 + i) * tsi + (c0 + g * 16 + c) * tsj] : T(0);
        if (tid == 0) {
            unsigned spins = 0;
            while (ld_acquire(flags + j) != epoch) {
                if (++spins > spin_limit || *((volatile int*)err) == kDevTimeout) {
                    atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                    s_abort = 1;
                    break;
                }
                if (spins > 32) __nanosleep(32);
            }
        }
        __syncthreads();
        if (s_abort) return;
        for (int t = tid; t < kTrsvBlock * NR; t += kTrsvThreads) {
            const int rr = t % kTrsvBlock, q = t / kTrsvBlock;
            xj[rr][q] = (q < nr) ? __ldcg(&B[(c0 + rr) * bsi + q * bsj]) : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 16; ++c)
#pragma unroll
            for (int q = 0; q < NR; ++q) acc[q] -= a[c] * xj[g * 16 + c][q];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) part[g][i][q] = acc[q];
    __syncthreads();
    for (int t = tid; t < kTrsvBlock * NR; t += kTrsvThreads) {
        const int rr = t % kTrsvBlock, q = t / kTrsvBlock;
        xs[rr][q] += ((part[0][rr][q] + part[1][rr][q]) + part[2][rr][q]) + part[3][rr][q];
    }
    __syncthreads();

    // diagonal block: x_b = D_b^-1 x_b as a product (thread (i, q) one entry),
    // or warp q substitutes right-hand side q (2 rows per lane)
    const int warp = tid >> 5, lane = tid & 31;
    bool sing = false;
    if (use_inv) {
        constexpr int PER = (NR * kTrsvBlock + kTrsvThreads - 1) / kTrsvThreads;
        T v[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int t = tid + u * kTrsvThreads, ii = t % kTrsvBlock, q = t / kTrsvBlock;
            v[u] = T(0);
            if (q < nr && ii < rows)
                for (int kk = 0; kk <= ii; ++kk) v[u] += Td[ii][kk] * xs[kk][q];
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int t = tid + u * kTrsvThreads, ii = t % kTrsvBlock, q = t / kTrsvBlock;
            if (q < nr && ii < rows) xs[ii][q] = v[u];
        }
    }
    for (int q = warp; q < nr && !use_inv; q += kTrsvThreads / 32) {
        for (int jj = 0; jj < rows; ++jj) {
            __syncwarp();
            T v = xs[jj][q];
            if (!unit) {
                const T d = Td[jj][jj];
                if (skip_zero) {
                    if (v != T(0)) {
                        if (d == T(0)) sing = true;
                        else v = v / d;
                    }
                } else {
                    if (d == T(0)) sing = true;
                    else v = v * (T(1) / d);
                }
            }
            __syncwarp();
            if (lane == 0) xs[jj][q] = v;
            if (v != T(0) || !skip_zero) {
                const int k1 = lane, k2 = lane + 32;
                if (k1 > jj && k1 < rows) xs[k1][q] -= Td[k1][jj] * v;
                if (k2 > jj && k2 < rows) xs[k2][q] -= Td[k2][jj] * v;
            }
        }
    }
    if (sing) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
    __syncthreads();
    for (int t = tid; t < kTrsvBlock * NR; t += kTrsvThreads) {
        const int rr = t % kTrsvBlock, q = t / kTrsvBlock;
        if (rr < rows && q < nr) B[(r0 + rr) * bsi + q * bsj] = xs[rr][q];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(flags + b, epoch);
}

template <typename T>
tmvg_status trsm_sync_free(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                           bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi, int64_t bsj,
                           bool skip_zero)
{
    if (n <= 0 || nrhs <= 0) return TMVG_OK;
    if (upper) {
        // reverse both index orders: U(n-1-i, n-1-j) is lower in (i, j)
        tri = tri + (n - 1) * (tsi + tsj);
        tsi = -tsi;
        tsj = -tsj;
        B = B + (n - 1) * bsi;
        bsi = -bsi;
    }
    const int64_t nblk = ceil_div(n, kTrsvBlock);
    constexpr int NRM = kTrsvMaxRhs<T>;
    const int64_t groups = nrhs == 1 ? 1 : ceil_div(nrhs, NRM);
    if (nblk * groups > (int64_t)kTrsvFlagCap)
        return set_error(c, TMVG_UNSUPPORTED, "trsv: n x nrhs too large for the flag array");
    const unsigned epoch = ++c->trsv_epoch;
    // tickets restart at 0 for every launch
    tmvg_status st = check_cuda(
        c, cudaMemsetAsync(c->trsv_ticket, 0, sizeof(unsigned long long), c->stream),
        "trsv ticket reset");
    if (st) return st;
    // tickets map to (block, group) pairs (ticket - tbase); the failure-path
    // test hook starts them at block test_skip_blocks, so the blocks before
    // it are never solved and the first waiting block's bounded wait gives up
    unsigned long long tbase = 0ull;
    if (c->test_skip_blocks > 0) {
        tbase = 0ull - (unsigned long long)c->test_skip_blocks * (unsigned long long)groups;
        c->test_skip_blocks = 0;
    }
    const unsigned limit = c->poll_limit ? c->poll_limit : kSpinLimit;
    const unsigned grid = (unsigned)(nblk * groups);
    // Beyond two groups (more than 2 NR columns) the diagonal blocks are
    // inverted first, so that a block's step on the chain is a short product
    // instead of a 64-step substitution with a division per step.
    const T* dinv = nullptr;
    const int* dsing = nullptr;
    if (groups > 2) {
        const size_t ib = sizeof(T) * (size_t)nblk * kTrsvBlock * kTrsvBlock;
        unsigned char* w = (unsigned char*)trsv_dinv_buffer(c, ib + sizeof(int) * (size_t)nblk);
        if (!w) return set_error(c, TMVG_OOM, "trsv: inverse blocks");
        T* dv = (T*)w;
        int* ds = (int*)(w + ib);
        const size_t smem = sizeof(T) * 2 * kTrsvBlock * (kTrsvBlock + 1);
        st = check_cuda(c, cudaFuncSetAttribute(tri_inv64_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem),
                        "trsv inverse blocks: smem attribute");
        if (st) return st;
        tri_inv64_kernel<T><<<(unsigned)nblk, kTrsvBlock, smem, c->stream>>>(n, tri, tsi, tsj, unit, dv, ds);
        ++c->launches;
        st = check_cuda(c, cudaGetLastError(), "trsv inverse blocks");
        if (st) return st;
        dinv = dv;
        dsing = ds;
    }
    if (nrhs == 1)
        trsm_sync_free_kernel<T, 1><<<grid, kTrsvThreads, 0, c->stream>>>(
            n, tri, tsi, tsj, unit, nrhs, 1, B, bsi, bsj, skip_zero, c->trsv_flags, epoch,
            c->trsv_ticket, tbase, limit, c->dflags, nullptr, nullptr);
    else
        trsm_sync_free_kernel<T, NRM><<<grid, kTrsvThreads, 0, c->stream>>>(
            n, tri, tsi, tsj, unit, nrhs, (int)groups, B, bsi, bsj, skip_zero, c->trsv_flags, epoch,
            c->trsv_ticket, tbase, limit, c->dflags, dinv, dsing);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "trsv launch");
}

// ---------------------------------------------------------------------
// Repeated single right-hand-side solves with one factor (the refinement
// loop of the mixed solve): the same sync-free block chain, with 128-row
// blocks whose diagonal blocks are inverted once per factor, so the step on
// the chain's critical path is two short mat-vecs instead of a 128-step
// substitution.  Blocks with a zero diagonal keep the substitution (and
// TMV's zero-skipping semantics); the others use D^-1.
// ---------------------------------------------------------------------
constexpr int kIB = 128;  // block rows of the inverse-diagonal solve

// One triangle's diagonal blocks to invert: D = the lower triangle at tri
// with strides (tsi, tsj) (an upper triangle is passed reversed), the
// inverses to dinv, the zero-diagonal flags to singular.
template <typename T>
struct InvBlocksJob {
    const T* tri;
    int64_t tsi, tsj;
    bool unit;
    T* dinv;
    int* singular;
};

// One CTA per diagonal block: Dinv_b = D_b^-1 (lower, column-major kIB x kIB
// at dinv + b*kIB*kIB).  singular[b] = 1 if D_b has a zero diagonal.  Blocks
// [0, nblk) are job 0's, [nblk, 2 nblk) job 1's (the two triangles of one
// factor in one launch).  Column j of the inverse by forward substitution in
// thread j; the diagonal's reciprocals are taken once per block.
template <typename T>
__global__ void __launch_bounds__(kIB)
invert_diag_blocks_kernel(int64_t n, int64_t nblk, InvBlocksJob<T> job0, InvBlocksJob<T> job1)
{
    extern __shared__ __align__(16) unsigned char inv_smem[];
    T* D = reinterpret_cast<T*>(inv_smem);  // [kIB][kIB+1]
    T* X = D + kIB * (kIB + 1);              // [kIB][kIB+1], X[i][j] = (D^-1)_ij
    __shared__ T rdiag[kIB];
    __shared__ int s_sing;
    const bool second = blockIdx.x >= nblk;
    const InvBlocksJob<T> job = second ? job1 : job0;
    const int64_t b = second ? blockIdx.x - nblk : blockIdx.x;
    const int64_t r0 = b * kIB;
    const int rows = (int)min((int64_t)kIB, n - r0);
    const int tid = threadIdx.x;
    if (tid == 0) s_sing = 0;
    // staged sixteen loads at a time per thread (column j = t / kIB of the
    // block, row i = t % kIB = this thread)
    constexpr int QS = 16;
    for (int t0 = tid; t0 < kIB * kIB; t0 += kIB * QS) {
        T v[QS];
#pragma unroll
        for (int u = 0; u < QS; ++u) {
            const int t = t0 + u * kIB;
            const int i = t % kIB, j = t / kIB;
            v[u] = (i < rows && j <= i) ? job.tri[(r0 + i) * job.tsi + (r0 + j) * job.tsj] : T(0);
        }
#pragma unroll
        for (int u = 0; u < QS; ++u) {
            const int t = t0 + u * kIB;
            D[(t % kIB) * (kIB + 1) + t / kIB] = v[u];
        }
    }
    __syncthreads();
    if (!job.unit && tid < rows && D[tid * (kIB + 1) + tid] == T(0)) s_sing = 1;
    rdiag[tid] = (job.unit || tid >= rows) ? T(1) : T(1) / D[tid * (kIB + 1) + tid];
    __syncthreads();
    if (s_sing) {
        if (tid == 0) job.singular[b] = 1;
        return;
    }
    const int j = tid;
    if (j < rows) {
        for (int i = 0; i < j; ++i) X[i * (kIB + 1) + j] = T(0);
        X[j * (kIB + 1) + j] = rdiag[j];
        for (int i = j + 1; i < rows; ++i) {
            const T* Di = D + i * (kIB + 1);
            T s0 = T(0), s1 = T(0);
            int l = j;
            for (; l + 2 <= i; l += 2) {
                s0 -= Di[l] * X[l * (kIB + 1) + j];
                s1 -= Di[l + 1] * X[(l + 1) * (kIB + 1) + j];
            }
            if (l < i) s0 -= Di[l] * X[l * (kIB + 1) + j];
            X[i * (kIB + 1) + j] = (s0 + s1) * rdiag[i];
        }
    }
    __syncthreads();
    T* out = job.dinv + b * (int64_t)kIB * kIB;
    for (int t = tid; t < kIB * kIB; t += kIB) {
        const int i = t % kIB, jj = t / kIB;
        out[t] = (i < rows && jj < rows) ? X[i * (kIB + 1) + jj] : T(0);
    }
    if (tid == 0) job.singular[b] = 0;
}

template <typename T>
__global__ void __launch_bounds__(256)
trsv_invdiag_kernel(int64_t n, const T* __restrict__ tri, int64_t tsi, int64_t tsj,
                    const T* __restrict__ dinv, const int* __restrict__ singular, bool unit,
                    T* x, int64_t incx, bool skip_zero, unsigned* flags, unsigned epoch,
                    unsigned long long* ticket, int* err, const int* stop)
{
    if (stop && *stop) return;  // a device-side loop has finished: no work, no waits
    __shared__ int s_blk, s_abort;
    __shared__ T xj[kIB];
    __shared__ T rhs[kIB];
    __shared__ T part[2][kIB];
    const int tid = threadIdx.x;
    const int i = tid & (kIB - 1), h = tid >> 7;  // row of the block, half of the columns
    if (tid == 0) {
        s_blk = (int)atomicAdd(ticket, 1ull);
        s_abort = 0;
    }
    __syncthreads();
    const int64_t b = s_blk;
    const int64_t nblk = (n + kIB - 1) / kIB;
    if (b >= nblk) return;
    const int64_t r0 = b * kIB;
    const int rows = (int)min((int64_t)kIB, n - r0);

    T acc = T(0);
    for (int64_t j = 0; j < b; ++j) {
        const int64_t c0 = j * kIB + h * 64;
        T a[64];
#pragma unroll
        for (int c = 0; c < 64; ++c) a[c] = (i < rows) ? tri[(r0 + i) * tsi + (c0 + c) * tsj] : T(0);
        if (tid == 0) {
            unsigned spins = 0;
            while (ld_acquire(flags + j) != epoch) {
                if (++spins > kSpinLimit || *((volatile int*)err) == kDevTimeout) {
                    atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                    s_abort = 1;
                    break;
                }
                if (spins > 32) __nanosleep(32);
            }
        }
        __syncthreads();
        if (s_abort) return;
        if (tid < kIB) xj[tid] = __ldcg(&x[(j * kIB + tid) * incx]);
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 64; ++c) acc -= a[c] * xj[h * 64 + c];
        __syncthreads();
    }
    part[h][i] = acc;
    if (tid < kIB) rhs[tid] = tid < rows ? x[(r0 + tid) * incx] : T(0);
    __syncthreads();
    if (tid < kIB) rhs[tid] += part[0][tid] + part[1][tid];
    __syncthreads();
    if (!singular[b]) {
        // x_b = Dinv_b rhs (lower): row i sums columns l <= i, split in halves
        const T* Di = dinv + b * (int64_t)kIB * kIB;
        T s = T(0);
        const int l0 = h * 64;
        for (int l = l0; l < l0 + 64; ++l) s += Di[i + l * kIB] * rhs[l];
        part[h][i] = s;
        __syncthreads();
        if (tid < rows) x[(r0 + tid) * incx] = part[0][tid] + part[1][tid];
    } else if (tid < 32) {
        // zero diagonal somewhere: substitution with TMV's zero skipping
        bool sing = false;
        for (int jj = 0; jj < rows; ++jj) {
            __syncwarp();
            T v = rhs[jj];
            if (!unit) {
                const T d = tri[(r0 + jj) * tsi + (r0 + jj) * tsj];
                if (skip_zero) {
                    if (v != T(0)) {
                        if (d == T(0)) sing = true;
                        else v = v / d;
                    }
                } else {
                    if (d == T(0)) sing = true;
                    else v = v * (T(1) / d);
                }
            }
            __syncwarp();
            if (tid == 0) rhs[jj] = v;
            if (v != T(0) || !skip_zero)
                for (int k2 = jj + 1 + tid; k2 < rows; k2 += 32)
                    rhs[k2] -= tri[(r0 + k2) * tsi + (r0 + jj) * tsj] * v;
        }
        if (sing) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
        __syncwarp();
        for (int k2 = tid; k2 < rows; k2 += 32) x[(r0 + k2) * incx] = rhs[k2];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release(flags + b, epoch);
}

// ---------------------------------------------------------------------
// FP32 inverse-block solve with published values.
//
// Same blocking and arithmetic as trsv_invdiag_kernel, but a finished block
// publishes each entry as one 64-bit word (epoch << 32 | float bits) with a
// relaxed gpu-scope store, so the word is both the value and its ready flag:
// a consumer thread polls exactly the word it needs (bounded), and the
// separate flag, fence and reload of x drop out of the dependency chain.
// Each CTA also loads its inverse diagonal block and right-hand side before
// it waits for anything.
// ---------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

constexpr int kPubThreads = 512;          // four threads per row of a block
constexpr int kPubCols = kIB / 4;          // columns of a tile per thread

__global__ void __launch_bounds__(kPubThreads)
trsv_pub_kernel(int64_t n, const float* __restrict__ tri, int64_t tsi, int64_t tsj,
                const float* __restrict__ dinv, const int* __restrict__ singular, bool unit,
                float* x, int64_t incx, bool skip_zero, unsigned long long* pub, unsigned epoch,
                unsigned long long* ticket, int* err, const int* stop)
{
    if (stop && *stop) return;  // a device-side loop has finished: no work, no waits
    __shared__ int s_blk, s_abort[2];  // one per parity of the wait: a single barrier separates two waits
    __shared__ float xj[2][kIB];
    __shared__ float rhs[kIB];
    __shared__ float part[4][kIB];
    const int tid = threadIdx.x;
    const int i = tid & (kIB - 1), q = tid >> 7;  // row of the block, quarter of the columns
    if (tid == 0) {
        s_blk = (int)atomicAdd(ticket, 1ull);
        s_abort[0] = s_abort[1] = 0;
    }
    __syncthreads();
    const int64_t b = s_blk;
    const int64_t nblk = (n + kIB - 1) / kIB;
    if (b >= nblk) return;
    const int64_t r0 = b * kIB;
    const int rows = (int)min((int64_t)kIB, n - r0);
    const unsigned long long tag = (unsigned long long)epoch << 32;

    // independent of the other blocks: right-hand side and inverse block
    const float b_i = (tid < kIB && tid < rows) ? x[(r0 + tid) * incx] : 0.0f;
    const bool sing = singular[b] != 0;
    float di[kPubCols];
    {
        const float* Di = dinv + b * (int64_t)kIB * kIB;
#pragma unroll
        for (int l = 0; l < kPubCols; ++l) di[l] = sing ? 0.0f : Di[i + (q * kPubCols + l) * kIB];
    }

    // tile j of this block's rows: the next tile's entries are loaded while
    // the current one waits for x_j and is applied (two register buffers)
    auto load_tile = [&](float (&a)[kPubCols], int64_t j) {
        const int64_t c0 = j * kIB + q * kPubCols;
#pragma unroll
        for (int c = 0; c < kPubCols; ++c) a[c] = (i < rows) ? tri[(r0 + i) * tsi + (c0 + c) * tsj] : 0.0f;
    };
    float acc0 = 0.0f, acc1 = 0.0f;
    // the word of x_j a thread polls was loaded one tile ahead (vpre), so its
    // latency hides behind the previous tile's barrier and FMAs
    unsigned long long vpre = 0;
    if (b > 0 && tid < kIB) vpre = ld_relaxed_u64(pub + tid);
    auto apply_tile = [&](const float (&a)[kPubCols], int64_t j) -> bool {
        float* xb = xj[j & 1];
        if (tid < kIB) {
            const unsigned long long* w = pub + j * kIB + tid;
            unsigned long long v = vpre;
            unsigned spins = 0;
            while ((v & 0xffffffff00000000ull) != tag) {
                if (++spins > kSpinLimit || *((volatile int*)err) == kDevTimeout) {
                    atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                    s_abort[j & 1] = 1;
                    break;
                }
                if (spins > 32) __nanosleep(32);
                v = ld_relaxed_u64(w);
            }
            xb[tid] = __uint_as_float((unsigned)v);
            if (j + 1 < b) vpre = ld_relaxed_u64(w + kIB);
        }
        __syncthreads();  // xb complete; the other buffer is free again
        if (s_abort[j & 1]) return false;
#pragma unroll
        for (int c = 0; c < kPubCols; c += 2) {
            acc0 -= a[c] * xb[q * kPubCols + c];
            acc1 -= a[c + 1] * xb[q * kPubCols + c + 1];
        }
        return true;
    };
    {
        float ta[kPubCols], tb[kPubCols];
        if (b > 0) load_tile(ta, 0);
        for (int64_t j = 0; j < b; j += 2) {
            if (j + 1 < b) load_tile(tb, j + 1);
            if (!apply_tile(ta, j)) return;
            if (j + 1 >= b) break;
            if (j + 2 < b) load_tile(ta, j + 2);
            if (!apply_tile(tb, j + 1)) return;
        }
    }
    part[q][i] = acc0 + acc1;
    __syncthreads();
    if (tid < kIB) rhs[tid] = b_i + ((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]));
    __syncthreads();
    if (!sing) {
        // x_b = Dinv_b rhs: row i sums its quarter of the columns
        float sum = 0.0f;
#pragma unroll
        for (int l = 0; l < kPubCols; ++l) sum += di[l] * rhs[q * kPubCols + l];
        part[q][i] = sum;
        __syncthreads();
        if (tid < rows) {
            const float v = (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
            x[(r0 + tid) * incx] = v;
            st_relaxed_u64(pub + r0 + tid, tag | __float_as_uint(v));
        }
    } else if (tid < 32) {
        // zero diagonal somewhere: substitution with TMV's zero skipping
        bool sg = false;
        for (int jj = 0; jj < rows; ++jj) {
            __syncwarp();
            float v = rhs[jj];
            if (!unit) {
                const float d = tri[(r0 + jj) * tsi + (r0 + jj) * tsj];
                if (skip_zero) {
                    if (v != 0.0f) {
                        if (d == 0.0f) sg = true;
                        else v = v / d;
                    }
                } else {
                    if (d == 0.0f) sg = true;
                    else v = v * (1.0f / d);
                }
            }
            __syncwarp();
            if (tid == 0) rhs[jj] = v;
            if (v != 0.0f || !skip_zero)
                for (int k2 = jj + 1 + tid; k2 < rows; k2 += 32)
                    rhs[k2] -= tri[(r0 + k2) * tsi + (r0 + jj) * tsj] * v;
        }
        if (sg) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
        __syncwarp();
        for (int k2 = tid; k2 < rows; k2 += 32) {
            x[(r0 + k2) * incx] = rhs[k2];
            st_relaxed_u64(pub + r0 + k2, tag | __float_as_uint(rhs[k2]));
        }
    }
}

template <typename T>
static InvBlocksJob<T> inv_blocks_job(int64_t n, const T* tri, int64_t tsi, int64_t tsj, bool upper,
                                      bool unit, T* dinv, int* singular)
{
    if (upper) {
        tri = tri + (n - 1) * (tsi + tsj);
        tsi = -tsi;
        tsj = -tsj;
    }
    return InvBlocksJob<T>{tri, tsi, tsj, unit, dinv, singular};
}

template <typename T>
static tmvg_status launch_inv_blocks(Context* c, int64_t n, const InvBlocksJob<T>& j0,
                                     const InvBlocksJob<T>& j1, int jobs)
{
    const int64_t nblk = ceil_div(n, kIB);
    const size_t smem = sizeof(T) * 2 * kIB * (kIB + 1);
    cudaFuncSetAttribute(invert_diag_blocks_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    invert_diag_blocks_kernel<T><<<(unsigned)(jobs * nblk), kIB, smem, c->stream>>>(n, nblk, j0, j1);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "invert diag launch");
}

template <typename T>
tmvg_status trsv_factor_inverse_blocks(Context* c, int64_t n, const T* tri, int64_t tsi,
                                       int64_t tsj, bool upper, bool unit, T* dinv, int* singular)
{
    if (n <= 0) return TMVG_OK;
    const InvBlocksJob<T> j = inv_blocks_job<T>(n, tri, tsi, tsj, upper, unit, dinv, singular);
    return launch_inv_blocks<T>(c, n, j, j, 1);
}

template <typename T>
tmvg_status trsv_lu_inverse_blocks(Context* c, int64_t n, const T* LU, int64_t ld, T* dinvL,
                                   int* singL, T* dinvU, int* singU)
{
    if (n <= 0) return TMVG_OK;
    const InvBlocksJob<T> jl = inv_blocks_job<T>(n, LU, 1, ld, false, true, dinvL, singL);
    const InvBlocksJob<T> ju = inv_blocks_job<T>(n, LU, 1, ld, true, false, dinvU, singU);
    return launch_inv_blocks<T>(c, n, jl, ju, 2);
}

// ---------------------------------------------------------------------
// The refinement's FP32 solve with its tiles streamed through shared memory
// (n a multiple of 128).  Timestamps per block showed the register form
// bound by streaming: a block's CTA spends about 2.2 us per 64 KB tile with
// one tile in flight.  Here each CTA keeps two tiles in flight in a ring of
// three shared-memory slots filled by cp.async (no register cost), and the
// last tile enters through a link block M_b = Dinv_b T[b, b-1] precomputed
// once per factor: y_b = Dinv_b (r_b - sum_{j<b-1} T[b,j] x_j) is formed
// before x_{b-1} arrives and the step on the chain is x_b = y_b - M_b x_{b-1}
// (Dinv_b and M_b rows in registers).  Blocks with a zero diagonal keep the
// substitution.
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(256)
link_blocks_kernel(int64_t n, int64_t nblk, InvBlocksJob<float> j0, InvBlocksJob<float> j1, float* ml0,
                   float* ml1)
{
    extern __shared__ __align__(16) float lk_smem[];
    float* Ds = lk_smem;                    // Dinv_b, [kIB][kIB+1] by row
    float* Ts = lk_smem + kIB * (kIB + 1);  // T[b, b-1], [kIB][kIB+1] by row
    const int job = (int)(blockIdx.x / (nblk - 1));
    const int64_t b = 1 + blockIdx.x % (nblk - 1);
    const InvBlocksJob<float>& J = job ? j1 : j0;
    float* ml = job ? ml1 : ml0;
    if (J.singular[b]) return;
    const int64_t r0 = b * kIB, c0 = (b - 1) * kIB;
    const int rows = (int)min((int64_t)kIB, n - r0);
    const float* Di = J.dinv + b * (int64_t)kIB * kIB;
    for (int t = threadIdx.x; t < kIB * kIB; t += 256) {
        const int i = t % kIB, k = t / kIB;  // coalesced along i
        Ds[i * (kIB + 1) + k] = Di[i + k * kIB];
        Ts[i * (kIB + 1) + k] = i < rows ? J.tri[(r0 + i) * J.tsi + (c0 + k) * J.tsj] : 0.0f;
    }
    __syncthreads();
    const int i0 = (threadIdx.x & 31) * 4, cc0 = (threadIdx.x >> 5) * 16;
    float acc[4][16];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[a][c] = 0.0f;
    for (int k = 0; k < kIB; ++k) {
        float d[4], tt[16];
#pragma unroll
        for (int a = 0; a < 4; ++a) d[a] = Ds[(i0 + a) * (kIB + 1) + k];
#pragma unroll
        for (int c = 0; c < 16; ++c) tt[c] = Ts[k * (kIB + 1) + cc0 + c];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 16; ++c) acc[a][c] = fmaf(d[a], tt[c], acc[a][c]);
    }
    float* out = ml + b * (int64_t)kIB * kIB;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 16; ++c) out[(i0 + a) + (cc0 + c) * kIB] = acc[a][c];
}

tmvg_status trsv_lu_link_blocks(Context* c, int64_t n, const float* LU, int64_t ld, const float* dinvL,
                                const int* singL, float* mlinkL, const float* dinvU, const int* singU,
                                float* mlinkU)
{
    const int64_t nblk = ceil_div(n, kIB);
    if (nblk < 2) return TMVG_OK;
    const InvBlocksJob<float> jl =
        inv_blocks_job<float>(n, LU, 1, ld, false, true, const_cast<float*>(dinvL), const_cast<int*>(singL));
    const InvBlocksJob<float> ju =
        inv_blocks_job<float>(n, LU, 1, ld, true, false, const_cast<float*>(dinvU), const_cast<int*>(singU));
    const size_t smem = sizeof(float) * 2 * kIB * (kIB + 1);
    tmvg_status st = check_cuda(
        c, cudaFuncSetAttribute(link_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
        "link blocks: smem attribute");
    if (st) return st;
    link_blocks_kernel<<<(unsigned)(2 * (nblk - 1)), 256, smem, c->stream>>>(n, nblk, jl, ju, mlinkL, mlinkU);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "link blocks launch");
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

constexpr int kRing = 3;  // shared-memory tile slots: two tiles in flight beside the one in use

// Rows of blocks b >= b0 are split between two CTAs: a helper takes the
// tiles j < b/2 (their x_j are published first) and publishes its partial
// row sums as tagged words in hpub; the block's own CTA takes the tiles from
// b/2 on and adds the helper's sums before its diagonal block.  Tickets run
// 0 .. b0-1 for the unsplit blocks, then helper(b), block(b) for b = b0, ...,
// so that every CTA waits only on CTAs with lower tickets.
__global__ void __launch_bounds__(kPubThreads)
trsv_pub_async_kernel(int64_t n, const float* __restrict__ tri, int64_t tsi, int64_t tsj, bool upper,
                      const float* __restrict__ dinv, const int* __restrict__ singular,
                      const float* __restrict__ mlink, bool unit, float* x, int64_t incx, bool skip_zero,
                      unsigned long long* pub, unsigned long long* hpub, int64_t b0, unsigned epoch,
                      unsigned long long* ticket, int64_t tk0, unsigned limit, int* err, const int* stop)
{
    if (stop && *stop) return;  // a device-side loop has finished: no work, no waits
    extern __shared__ __align__(16) float ring[];  // [kRing][kIB columns][kIB]
    __shared__ int64_t s_tk;
    __shared__ int s_abort[2];  // one per parity of the wait: a single barrier separates two waits
    __shared__ float xj[2][kIB];
    __shared__ float rhs[kIB];
    __shared__ float hp[kIB];
    __shared__ float part[4][kIB];
    const int tid = threadIdx.x;
    const int i = tid & (kIB - 1), q = tid >> 7;  // row of the block, quarter of the columns
    if (tid == 0) {
        // tickets from tk0 on (tk0 > 0 only for the failure-path test hook)
        s_tk = (int64_t)atomicAdd(ticket, 1ull) + tk0;
        s_abort[0] = s_abort[1] = 0;
    }
    __syncthreads();
    const int64_t tk = s_tk;
    const int64_t nblk = n / kIB;
    const int64_t b = tk < b0 ? tk : b0 + (tk - b0) / 2;
    const bool helper = tk >= b0 && ((tk - b0) & 1) == 0;
    const bool split = b >= b0;
    if (b >= nblk) return;
    const int64_t r0 = b * kIB;
    const unsigned long long tag = (unsigned long long)epoch << 32;
    // a tile column's 128 entries are contiguous in memory, from view row
    // r0 (lower) or r0 + 127 (upper: the view is index-reversed)
    const int64_t rbase = upper ? (r0 + kIB - 1) * tsi : r0 * tsi;
    const int pos = upper ? kIB - 1 - i : i;  // this row's place in a slot column

    // independent of the other blocks: right-hand side, inverse and link rows
    const bool sing = singular[b] != 0;
    const bool use_link = !helper && b >= 1 && !sing;
    const int64_t jbeg = split && !helper ? b / 2 : 0;
    const int64_t jend = helper ? b / 2 : (use_link ? b - 1 : b);
    const float b_i = !helper && tid < kIB ? x[(r0 + tid) * incx] : 0.0f;
    float di[kPubCols], mi[kPubCols];
    {
        const float* Di = dinv + b * (int64_t)kIB * kIB;
        const float* Mb = use_link ? mlink + b * (int64_t)kIB * kIB : nullptr;
#pragma unroll
        for (int l = 0; l < kPubCols; ++l) {
            di[l] = sing || helper ? 0.0f : Di[i + (q * kPubCols + l) * kIB];
            mi[l] = use_link ? Mb[i + (q * kPubCols + l) * kIB] : 0.0f;
        }
    }
    // tile j into slot s: 4096 pieces of 16 bytes, 8 per thread
    auto fetch = [&](int64_t j, int s) {
        if (j < jend) {
            float* slot = ring + (size_t)s * kIB * kIB;
#pragma unroll
            for (int u = 0; u < (kIB * kIB / 4) / kPubThreads; ++u) {
                const int t = tid + u * kPubThreads;
                const int c = t / (kIB / 4), k = t % (kIB / 4);
                cp_async16(slot + c * kIB + 4 * k, tri + rbase + (j * kIB + c) * tsj + 4 * k);
            }
        }
        cp_async_commit();  // one group per tile, empty past the last
    };
    int waits = 0;  // waits so far: the parity of the next one's buffers
    // poll 128 tagged words from w into dst (the first value already loaded)
    auto wait_words = [&](const unsigned long long* w, unsigned long long v, float* dst) -> bool {
        const int par = waits++ & 1;
        if (tid < kIB) {
            unsigned spins = 0;
            while ((v & 0xffffffff00000000ull) != tag) {
                if (++spins > limit || *((volatile int*)err) == kDevTimeout) {
                    atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
                    s_abort[par] = 1;
                    break;
                }
                if (spins > 32) __nanosleep(32);
                v = ld_relaxed_u64(w + tid);
            }
            dst[tid] = __uint_as_float((unsigned)v);
        }
        __syncthreads();  // dst complete (and every thread's landed tile copies visible)
        return !s_abort[par];
    };
    // the word of x_j a thread polls is loaded one wait ahead
    unsigned long long vpre = 0;
    if (b > 0 && tid < kIB) vpre = ld_relaxed_u64(pub + jbeg * kIB + tid);
    auto wait_x = [&](int64_t j) -> const float* {
        float* xb = xj[waits & 1];
        const unsigned long long v = vpre;
        if (tid < kIB && j + 1 < b) vpre = ld_relaxed_u64(pub + (j + 1) * kIB + tid);
        return wait_words(pub + j * kIB, v, xb) ? xb : nullptr;
    };
    float acc0 = 0.0f, acc1 = 0.0f;
    fetch(jbeg, 0);
    fetch(jbeg + 1, 1);
    for (int64_t j = jbeg; j < jend; ++j) {
        const int64_t k = j - jbeg;
        cp_async_wait1();  // this thread's pieces of tile j have landed
        const float* xb = wait_x(j);
        if (!xb) {
            asm volatile("cp.async.wait_all;" ::: "memory");
            return;
        }
        // slot (k + 2) % 3 held tile j - 1, which every thread finished
        // before the barrier above
        fetch(j + 2, (int)((k + 2) % kRing));
        const float* slot = ring + (size_t)(k % kRing) * kIB * kIB;
#pragma unroll
        for (int l = 0; l < kPubCols; l += 2) {
            acc0 -= slot[(q * kPubCols + l) * kIB + pos] * xb[q * kPubCols + l];
            acc1 -= slot[(q * kPubCols + l + 1) * kIB + pos] * xb[q * kPubCols + l + 1];
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");  // the empty groups past the last tile
    part[q][i] = acc0 + acc1;
    if (helper) {
        __syncthreads();
        if (tid < kIB) {
            const float p = (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
            st_relaxed_u64(hpub + r0 + tid, tag | __float_as_uint(p));
        }
        return;
    }
    if (split) {
        const unsigned long long v = tid < kIB ? ld_relaxed_u64(hpub + r0 + tid) : 0ull;
        if (!wait_words(hpub + r0, v, hp)) return;  // its barrier also completes part
    } else {
        __syncthreads();
    }
    if (tid < kIB) {
        const float h = split ? hp[tid] : 0.0f;
        rhs[tid] = b_i + (((part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid])) + h);
    }
    __syncthreads();
    if (!sing) {
        float sum = 0.0f;
#pragma unroll
        for (int l = 0; l < kPubCols; ++l) sum += di[l] * rhs[q * kPubCols + l];
        part[q][i] = sum;
        __syncthreads();
        float v = tid < kIB ? (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]) : 0.0f;
        if (use_link) {
            const float* xb = wait_x(b - 1);  // its barrier also orders the reads of part above
            if (!xb) return;
            float m0 = 0.0f, m1 = 0.0f;
#pragma unroll
            for (int l = 0; l < kPubCols; l += 2) {
                m0 = fmaf(mi[l], xb[q * kPubCols + l], m0);
                m1 = fmaf(mi[l + 1], xb[q * kPubCols + l + 1], m1);
            }
            part[q][i] = m0 + m1;
            __syncthreads();
            if (tid < kIB) v -= (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
        }
        if (tid < kIB) {
            x[(r0 + tid) * incx] = v;
            st_relaxed_u64(pub + r0 + tid, tag | __float_as_uint(v));
        }
    } else if (tid < 32) {
        // zero diagonal somewhere: substitution with TMV's zero skipping
        bool sg = false;
        for (int jj = 0; jj < kIB; ++jj) {
            __syncwarp();
            float v = rhs[jj];
            if (!unit) {
                const float d = tri[(r0 + jj) * tsi + (r0 + jj) * tsj];
                if (skip_zero) {
                    if (v != 0.0f) {
                        if (d == 0.0f) sg = true;
                        else v = v / d;
                    }
                } else {
                    if (d == 0.0f) sg = true;
                    else v = v * (1.0f / d);
                }
            }
            __syncwarp();
            if (tid == 0) rhs[jj] = v;
            if (v != 0.0f || !skip_zero)
                for (int k2 = jj + 1 + tid; k2 < kIB; k2 += 32)
                    rhs[k2] -= tri[(r0 + k2) * tsi + (r0 + jj) * tsj] * v;
        }
        if (sg) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
        __syncwarp();
        for (int k2 = tid; k2 < kIB; k2 += 32) {
            x[(r0 + k2) * incx] = rhs[k2];
            st_relaxed_u64(pub + r0 + k2, tag | __float_as_uint(rhs[k2]));
        }
    }
}

template <typename T>
tmvg_status trsv_with_inverse_blocks(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                                     bool upper, bool unit, const T* dinv, const int* singular,
                                     T* x, int64_t incx, bool skip_zero, const int* stop,
                                     const T* mlink)
{
    const bool is_upper = upper;
    const T* tri_in = tri;  // the triangle's storage, before an upper view is reversed
    const int64_t tsi_in = tsi;
    if (n <= 0) return TMVG_OK;
    if (upper) {
        tri = tri + (n - 1) * (tsi + tsj);
        tsi = -tsi;
        tsj = -tsj;
        x = x + (n - 1) * incx;
        incx = -incx;
    }
    const int64_t nblk = ceil_div(n, kIB);
    if (nblk > kTrsvFlagCap) return set_error(c, TMVG_UNSUPPORTED, "trsv: n too large");
    const unsigned epoch = ++c->trsv_epoch;
    tmvg_status st = check_cuda(
        c, cudaMemsetAsync(c->trsv_ticket, 0, sizeof(unsigned long long), c->stream), "ticket");
    if (st) return st;
    if constexpr (std::is_same<T, float>::value) {
        if ((size_t)n > c->trsv_pub_len) {
            // grow-only; the old words are discarded with the buffer
            st = check_cuda(c, cudaStreamSynchronize(c->stream), "trsv pub sync");
            if (st) return st;
            if (c->trsv_pub) cudaFree(c->trsv_pub);
            c->trsv_pub = nullptr;
            c->trsv_pub_len = 0;
            // x's words, then the split rows' partial sums
            if (cudaMalloc(&c->trsv_pub, 2 * sizeof(unsigned long long) * (size_t)n) != cudaSuccess) {
                cudaGetLastError();
                return set_error(c, TMVG_OOM, "trsv: publication buffer");
            }
            // epoch 0 is never used by a solve
            st = check_cuda(c, cudaMemset(c->trsv_pub, 0, 2 * sizeof(unsigned long long) * (size_t)n),
                            "trsv pub clear");
            if (st) return st;
            c->trsv_pub_len = (size_t)n;
        }
        if (epoch == 0) ++c->trsv_epoch;  // skip the clear value on wrap-around
        // the streamed form: whole 128-row blocks, 16-byte aligned tile columns
        if (mlink && n % kIB == 0 && tsi_in == 1 && (tsj % 4) == 0 && ((uintptr_t)tri_in % 16) == 0) {
            const size_t smem = sizeof(float) * kRing * kIB * kIB;
            st = check_cuda(c, cudaFuncSetAttribute(trsv_pub_async_kernel,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                            "trsv async: smem attribute");
            if (st) return st;
            // split rows from b0 on while every CTA has an SM of its own
            // (one 197 KB CTA per SM)
            const int64_t b0 = std::min<int64_t>(nblk, std::max<int64_t>(4, 2 * nblk - c->num_sms));
            // the failure-path test hook: tickets start at test_skip_blocks,
            // so the blocks before it are never solved and the waits on them
            // give up after poll_limit polls
            const int64_t tk0 = c->test_skip_blocks > 0 ? c->test_skip_blocks : 0;
            c->test_skip_blocks = 0;
            const unsigned limit = c->poll_limit ? c->poll_limit : kSpinLimit;
            trsv_pub_async_kernel<<<(unsigned)(2 * nblk - b0), kPubThreads, smem, c->stream>>>(
                n, tri, tsi, tsj, is_upper, dinv, singular, mlink, unit, x, incx, skip_zero, c->trsv_pub,
                c->trsv_pub + c->trsv_pub_len, b0, c->trsv_epoch, c->trsv_ticket, tk0, limit, c->dflags,
                stop);
            ++c->launches;
            return check_cuda(c, cudaGetLastError(), "trsv async launch");
        }
        trsv_pub_kernel<<<(unsigned)nblk, kPubThreads, 0, c->stream>>>(
            n, tri, tsi, tsj, dinv, singular, unit, x, incx, skip_zero, c->trsv_pub,
            c->trsv_epoch, c->trsv_ticket, c->dflags, stop);
        ++c->launches;
        return check_cuda(c, cudaGetLastError(), "trsv pub launch");
    }
    trsv_invdiag_kernel<T><<<(unsigned)nblk, 256, 0, c->stream>>>(
        n, tri, tsi, tsj, dinv, singular, unit, x, incx, skip_zero, c->trsv_flags, epoch,
        c->trsv_ticket, c->dflags, stop);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "trsv invdiag launch");
}

template tmvg_status trsv_lu_inverse_blocks<float>(Context*, int64_t, const float*, int64_t, float*,
                                                   int*, float*, int*);
template tmvg_status trsv_factor_inverse_blocks<float>(Context*, int64_t, const float*, int64_t,
                                                       int64_t, bool, bool, float*, int*);
template tmvg_status trsv_factor_inverse_blocks<double>(Context*, int64_t, const double*, int64_t,
                                                        int64_t, bool, bool, double*, int*);
template tmvg_status trsv_with_inverse_blocks<float>(Context*, int64_t, const float*, int64_t,
                                                     int64_t, bool, bool, const float*, const int*,
                                                     float*, int64_t, bool, const int*, const float*);
template tmvg_status trsv_with_inverse_blocks<double>(Context*, int64_t, const double*, int64_t,
                                                      int64_t, bool, bool, const double*,
                                                      const int*, double*, int64_t, bool, const int*,
                                                      const double*);

// ---------------------------------------------------------------------
// Interchanges -> gather permutation: perm = identity, then for i in order
// swap(perm[i], perm[P[i]]) (a P[i] outside [0, n) is skipped); row i of
// P*B is row perm[i] of B.  The swaps are cut into chunks of kPermChunk: a
// chunk [k, k+64) moves only rows k..k+63 and its pivot rows, so one 32-thread
// CTA per chunk turns its swaps into a row gather of at most 128 pairs
// (panel_row_pairs), all chunks at once; then one CTA applies the gathers in
// chunk order to the permutation, in shared memory (n <= kPermSmemMax) or in
// global memory.  The sequential form costs a dependent shared-memory round
// trip per swap (about 330 us at n = 8192); this one about a chunk's.
// ---------------------------------------------------------------------
constexpr int kPermChunk = 64;
constexpr int kPermListInts = 1 + 2 * kMaxPairs;  // one chunk's list: count, dst[], src[]
constexpr int kPermChunkPairs = 2 * kPermChunk;    // most pairs a chunk can have
constexpr int kPermStage = 16;                     // chunk lists staged in shared memory at once
constexpr int kPermThreads = 128;
constexpr int kPermSmemMax = 49152;
static_assert(kPermChunkPairs <= kPermThreads, "a thread per pair");

__global__ void __launch_bounds__(32) perm_chunk_pairs_kernel(int64_t n, const int64_t* __restrict__ P,
                                                              int* __restrict__ lists)
{
    __shared__ int piv[kPermChunk];
    const int64_t k = (int64_t)blockIdx.x * kPermChunk;
    const int nb = (int)min((int64_t)kPermChunk, n - k);
    for (int t = threadIdx.x; t < nb; t += 32) {
        const int64_t p = P[k + t];
        piv[t] = (p >= 0 && p < n) ? (int)p : (int)(k + t);
    }
    __syncwarp();
    panel_row_pairs(k, nb, piv, lists + (int64_t)blockIdx.x * kPermListInts);
}

__global__ void __launch_bounds__(kPermThreads) perm_apply_kernel(int64_t n, int nchunks,
                                                                  const int* __restrict__ lists,
                                                                  int* __restrict__ perm, bool in_smem)
{
    extern __shared__ int sy[];  // the permutation, when it fits
    __shared__ int st_cnt[kPermStage];
    __shared__ int st_dst[kPermStage][kPermChunkPairs];
    __shared__ int st_src[kPermStage][kPermChunkPairs];
    int* y = in_smem ? sy : perm;
    const int tid = threadIdx.x;
    for (int64_t t = tid; t < n; t += kPermThreads) y[t] = (int)t;
    for (int b0 = 0; b0 < nchunks; b0 += kPermStage) {
        const int nst = min(kPermStage, nchunks - b0);
        __syncthreads();  // the previous stage is applied (and y initialised)
        // a stage's lists, every load of a thread issued before its stores
        // (kPermChunkPairs == kPermThreads: a thread takes one pair slot of
        // every chunk)
        static_assert(kPermChunkPairs == kPermThreads, "one slot per thread and chunk");
        int vd[kPermStage], vs[kPermStage];
#pragma unroll
        for (int b = 0; b < kPermStage; ++b) {
            const int* L = lists + (int64_t)(b0 + (b < nst ? b : 0)) * kPermListInts;
            vd[b] = L[1 + tid];
            vs[b] = L[1 + kMaxPairs + tid];
        }
#pragma unroll
        for (int b = 0; b < kPermStage; ++b) {
            st_dst[b][tid] = vd[b];
            st_src[b][tid] = vs[b];
        }
        if (tid < nst) st_cnt[tid] = lists[(int64_t)(b0 + tid) * kPermListInts];
        __syncthreads();
        for (int b = 0; b < nst; ++b) {
            const int np = st_cnt[b];
            const int v = tid < np ? y[st_src[b][tid]] : 0;
            __syncthreads();
            if (tid < np) y[st_dst[b][tid]] = v;
            __syncthreads();
        }
    }
    if (in_smem) {
        __syncthreads();
        for (int64_t t = tid; t < n; t += kPermThreads) perm[t] = sy[t];
    }
}

tmvg_status pivots_to_perm(Context* c, int64_t n, const int64_t* P, int* perm)
{
    if (n <= 0) return TMVG_OK;
    if (n > (int64_t)INT32_MAX) return set_error(c, TMVG_UNSUPPORTED, "perm: n too large");
    const int64_t nchunks = ceil_div(n, kPermChunk);
    int* lists = (int*)perm_lists_buffer(c, sizeof(int) * (size_t)nchunks * kPermListInts);
    if (!lists) return TMVG_OOM;
    perm_chunk_pairs_kernel<<<(unsigned)nchunks, 32, 0, c->stream>>>(n, P, lists);
    ++c->launches;
    tmvg_status st = check_cuda(c, cudaGetLastError(), "perm: chunk launch");
    if (st) return st;
    const bool in_smem = n <= kPermSmemMax;
    const size_t smem = in_smem ? sizeof(int) * (size_t)n : 0;
    // the staged lists take 16 KB of static shared memory beside the
    // permutation: above 48 KB in all, the kernel must opt in
    if (smem + sizeof(int) * (kPermStage * (2 * kPermChunkPairs + 1)) > 48 * 1024)
        cudaFuncSetAttribute(perm_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(int) * kPermSmemMax));
    perm_apply_kernel<<<1, kPermThreads, smem, c->stream>>>(n, (int)nchunks, lists, perm, in_smem);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "perm: apply launch");
}

// out[i, q] = in[perm[i], q] (forward) or out[perm[i], q] = in[i, q] (inverse).
template <typename T>
__global__ void permute_rows_kernel(int64_t n, int64_t ncols, const int* __restrict__ perm,
                                    const T* __restrict__ in, int64_t isi, int64_t isj,
                                    T* __restrict__ out, int64_t osi, int64_t osj, bool inverse)
{
    const int64_t total = n * ncols;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % n, q = t / n;
        const int64_t p = perm[i];
        if (!inverse) out[i * osi + q * osj] = in[p * isi + q * isj];
        else out[p * osi + q * osj] = in[i * isi + q * isj];
    }
}

template <typename T>
tmvg_status permute_rows(Context* c, int64_t n, int64_t ncols, const int* perm, const T* in,
                         int64_t isi, int64_t isj, T* out, int64_t osi, int64_t osj, bool inverse)
{
    if (n <= 0 || ncols <= 0) return TMVG_OK;
    const int64_t total = n * ncols;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(total, 256), 8 * c->num_sms);
    permute_rows_kernel<T><<<blocks, 256, 0, c->stream>>>(n, ncols, perm, in, isi, isj, out, osi,
                                                          osj, inverse);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "permute launch");
}

template tmvg_status trsm_sync_free<double>(Context*, int64_t, const double*, int64_t, int64_t,
                                            bool, bool, int64_t, double*, int64_t, int64_t, bool);
template tmvg_status trsm_sync_free<float>(Context*, int64_t, const float*, int64_t, int64_t,
                                           bool, bool, int64_t, float*, int64_t, int64_t, bool);
template tmvg_status permute_rows<double>(Context*, int64_t, int64_t, const int*, const double*,
                                          int64_t, int64_t, double*, int64_t, int64_t, bool);
template tmvg_status permute_rows<float>(Context*, int64_t, int64_t, const int*, const float*,
                                         int64_t, int64_t, float*, int64_t, int64_t, bool);

}  // namespace tmvg
