// gemm_tc.cu -- FP32-accurate trailing update C -= A B on the fifth-generation
// tensor cores (tcgen05.mma kind::tf32, accumulators in tensor memory).
//
// 3xTF32 split: x = hi + lo with hi = tf32(x), lo = tf32(x - hi); the product
// is accumulated as lo_A hi_B + hi_A lo_B + hi_A hi_B in FP32, dropping only
// lo_A lo_B (about 2^-22 relative), so the update keeps FP32 accuracy, which
// the iterative refinement of the mixed solve needs (plain TF32 factors do
// not converge at cond 1e6).
//
// Data flow per CTA (one 128 x BN tile of C, K = 32 * KCH <= 128):
//   split kernels write hi/lo copies of A (row-major, K contiguous) and of B
//   (column-major, K contiguous) -> TMA loads every K chunk of the four
//   operands into 128-byte-swizzled shared memory (one mbarrier) -> one
//   thread issues 3 * K/8 MMAs into a 128 x BN FP32 accumulator in TMEM and
//   commits to a second mbarrier -> four warps read the accumulator with
//   tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows of the tile) and
//   write C -= acc with coalesced column stores.
// All waits are bounded; on a timeout the kernel records kDevTimeout.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "async.cuh"
#include "gemm.cuh"
#include "gemm_tc.cuh"

#include <algorithm>
#include <climits>

namespace tmvg {

constexpr int kTcM = 128;        // tile rows (UMMA M)
constexpr int kTcThreads = 128;  // four warps: one per 32 TMEM lanes
constexpr int kKChunk = 32;      // floats in one 128-byte swizzle row

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                            int c1)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
        : "memory");
}

// Bulk tensor store of a shared-memory tile (clipped at the tensor's bounds).
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int c0, int c1)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(smem_u32(src)), "r"(c0), "r"(c1)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void tma_store_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes in 8-row (1024-byte) groups.
__device__ __forceinline__ uint64_t sw128_desc(const void* p)
{
    const uint64_t addr = smem_u32(p);
    uint64_t d = (addr >> 4) & 0x3FFFull;  // start address
    d |= 1ull << 16;                        // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset: 8 rows x 128 B
    d |= 1ull << 46;                        // descriptor version
    d |= 2ull << 61;                        // 128-byte swizzle
    return d;
}

// Instruction descriptor: D FP32, A and B TF32, both K-major, M = 128, N = BN.
template <int BN>
__host__ __device__ constexpr uint32_t tf32_idesc()
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
           ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
          "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// TMAC: the C tile travels by TMA (loaded into shared memory beside the
// operands on its own mbarrier, updated there, stored back in bulk), which
// needs C 16-byte aligned with ldc a multiple of 4; otherwise the epilogue
// reads and writes C directly.
template <int BN, int KCH, bool TMAC>
__global__ void __launch_bounds__(kTcThreads, 1)
tf32x3_update_kernel(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                     const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
                     const __grid_constant__ CUtensorMap mC, float* __restrict__ C, int64_t ldc, int M,
                     int N, int* err)
{
    constexpr int A_BYTES = kTcM * 128;
    constexpr int B_BYTES = BN * 128;
    constexpr int CHUNK = 2 * A_BYTES + 2 * B_BYTES;
    constexpr int C_BYTES = BN * kTcM * 4;
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) &
                                               ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t bar_tma;
    __shared__ __align__(8) uint64_t bar_mma;
    __shared__ __align__(8) uint64_t bar_c;
    float* Cs = reinterpret_cast<float*>(base + KCH * CHUNK);  // [BN][128] when TMAC
    __shared__ uint32_t s_tmem;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.x * kTcM, col0 = blockIdx.y * BN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s_tmem)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bar_tma, 1);
        mbar_init(&bar_mma, 1);
        mbar_init(&bar_c, 1);
        s_fail = 0;
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    if (tid == 0) {
        if constexpr (TMAC) {
            mbar_expect_tx(&bar_c, (uint32_t)C_BYTES);
            tma_load_2d(Cs, &mC, &bar_c, row0, col0);
        }
        mbar_expect_tx(&bar_tma, (uint32_t)(KCH * CHUNK));
#pragma unroll
        for (int kc = 0; kc < KCH; ++kc) {
            uint8_t* ch = base + kc * CHUNK;
            tma_load_2d(ch, &mAhi, &bar_tma, kc * kKChunk, row0);
            tma_load_2d(ch + A_BYTES, &mAlo, &bar_tma, kc * kKChunk, row0);
            tma_load_2d(ch + 2 * A_BYTES, &mBhi, &bar_tma, kc * kKChunk, col0);
            tma_load_2d(ch + 2 * A_BYTES + B_BYTES, &mBlo, &bar_tma, kc * kKChunk, col0);
        }
        if (!mbar_wait(&bar_tma, 0)) {
            s_fail = 1;
            atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
        } else {
            tc_fence_after();
            constexpr uint32_t idesc = tf32_idesc<BN>();
            uint32_t acc = 0;
#pragma unroll
            for (int kc = 0; kc < KCH; ++kc) {
                uint8_t* ch = base + kc * CHUNK;
                const uint64_t ahi = sw128_desc(ch), alo = sw128_desc(ch + A_BYTES);
                const uint64_t bhi = sw128_desc(ch + 2 * A_BYTES);
                const uint64_t blo = sw128_desc(ch + 2 * A_BYTES + B_BYTES);
#pragma unroll
                for (int kk = 0; kk < kKChunk / 8; ++kk) {
                    const uint64_t off = (uint64_t)(kk * 32) >> 4;  // 8 TF32 = 32 bytes
                    umma_tf32(tmem, alo + off, bhi + off, idesc, acc);
                    acc = 1;
                    umma_tf32(tmem, ahi + off, blo + off, idesc, 1);
                    umma_tf32(tmem, ahi + off, bhi + off, idesc, 1);
                }
            }
            umma_commit(&bar_mma);
        }
    }
    __syncthreads();
    if (!s_fail) {
        bool done = mbar_wait(&bar_mma, 0);
        if (TMAC && done) done = mbar_wait(&bar_c, 0);
        if (!done) {
            atomicCAS(err, (int)kDevOk, (int)kDevTimeout);
            s_fail = 1;
        }
        tc_fence_after();
        if (done) {
            const int rl = warp * 32 + lane;  // row within the tile = TMEM lane
            const int r = row0 + rl;
            const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
            for (int cb = 0; cb < BN; cb += 16) {
                uint32_t v[16];
                tmem_ld16(lane_addr + (uint32_t)cb, v);
                if constexpr (TMAC) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) Cs[(cb + q) * kTcM + rl] -= __uint_as_float(v[q]);
                } else if (r < M) {
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int col = col0 + cb + q;
                        if (col < N) C[r + (int64_t)col * ldc] -= __uint_as_float(v[q]);
                    }
                }
            }
            if constexpr (TMAC) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
    } else if (tid == 0) {
        // copies may still be in flight: give them a bounded chance to land
        mbar_wait(&bar_tma, 0);
        if (TMAC) mbar_wait(&bar_c, 0);
    }
    tc_fence_before();
    __syncthreads();
    if constexpr (TMAC) {
        if (tid == 0 && !s_fail) {
            tma_store_2d(&mC, Cs, row0, col0);
            tma_store_wait_read();  // the tile must be read out before the CTA exits
        }
    }
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"((uint32_t)BN)
                     : "memory");
    }
}


// A (m x K, column-major, lda) -> hi/lo row-major m x K (K contiguous), via
// 32 x 32 shared-memory tiles so both sides stay coalesced.
__global__ void split_transpose_kernel(int64_t m, int K, const float* __restrict__ A, int64_t lda,
                                       float* __restrict__ hi, float* __restrict__ lo)
{
    __shared__ float tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int k0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + threadIdx.x;
        const int k = k0 + r;
        tile[r][threadIdx.x] = (i < m && k < K) ? A[i + (int64_t)k * lda] : 0.0f;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + r;
        const int k = k0 + threadIdx.x;
        if (i < m && k < K) {
            const float x = tile[threadIdx.x][r];
            const float h = tf32_round(x);
            hi[i * K + k] = h;
            lo[i * K + k] = tf32_round(x - h);
        }
    }
}

// B (K x n, column-major, ldb) -> hi/lo column-major with leading dimension K.
__global__ void split_cols_kernel(int64_t n, int K, const float* __restrict__ B, int64_t ldb,
                                  float* __restrict__ hi, float* __restrict__ lo)
{
    const int64_t total = n * K;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / K;
        const int k = (int)(t % K);
        const float x = B[k + j * ldb];
        const float h = tf32_round(x);
        hi[t] = h;
        lo[t] = tf32_round(x - h);
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// rows x K operand with K contiguous (row stride K floats); box 32 x box_rows.
static bool make_map(CUtensorMap* map, const float* base, int64_t rows, int K, int box_rows)
{
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)K * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kKChunk, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool tf32x3_supported(int64_t K) { return K > 0 && K % kKChunk == 0 && K <= 128 && encode_fn(); }

template <int BN, int KCH>
static tmvg_status launch_update(Context* c, const CUtensorMap* maps, bool tmac, float* C, int64_t ldc,
                                 int64_t m, int64_t n)
{
    constexpr size_t ops = (size_t)KCH * (2 * kTcM * 128 + 2 * BN * 128);
    dim3 grid((unsigned)ceil_div(m, kTcM), (unsigned)ceil_div(n, BN));
    if (tmac) {
        constexpr size_t smem = ops + (size_t)BN * kTcM * 4 + 1024;
        static_assert(smem <= 232448, "shared memory of one CTA");
        cudaFuncSetAttribute(tf32x3_update_kernel<BN, KCH, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        tf32x3_update_kernel<BN, KCH, true><<<grid, kTcThreads, smem, c->stream>>>(
            maps[0], maps[1], maps[2], maps[3], maps[4], C, ldc, (int)m, (int)n, c->dflags);
    } else {
        constexpr size_t smem = ops + 1024;
        cudaFuncSetAttribute(tf32x3_update_kernel<BN, KCH, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        tf32x3_update_kernel<BN, KCH, false><<<grid, kTcThreads, smem, c->stream>>>(
            maps[0], maps[1], maps[2], maps[3], maps[0], C, ldc, (int)m, (int)n, c->dflags);
    }
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "tf32x3 update launch");
}

// C (m x n, column-major, ldc) as a tensor of 128 x BN tiles, rows innermost.
static bool make_c_map(CUtensorMap* map, float* C, int64_t m, int64_t n, int64_t ldc, int bn)
{
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)n};
    cuuint64_t strides[1] = {(cuuint64_t)ldc * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kTcM, (cuuint32_t)bn};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

tmvg_status tf32x3_buffers(Context* c, int64_t m, int64_t n, int64_t K, Tf32x3Buffers* b)
{
    // B hi/lo first so that their place depends on n and K only
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t sa = al(sizeof(float) * (size_t)m * K), sb = al(sizeof(float) * (size_t)n * K);
    unsigned char* ws = (unsigned char*)workspace3(c, 2 * sa + 2 * sb);
    if (!ws) return TMVG_OOM;
    b->Bhi = (float*)ws;
    b->Blo = (float*)(ws + sb);
    b->Ahi = (float*)(ws + 2 * sb);
    b->Alo = (float*)(ws + 2 * sb + sa);
    return TMVG_OK;
}

tmvg_status tf32x3_split_a(Context* c, int64_t m, int64_t K, const float* A, int64_t lda,
                           const Tf32x3Buffers& b)
{
    if (m <= 0) return TMVG_OK;
    split_transpose_kernel<<<dim3((unsigned)ceil_div(m, 32), (unsigned)ceil_div(K, 32)), dim3(32, 8), 0,
                             c->stream>>>(m, (int)K, A, lda, b.Ahi, b.Alo);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "tf32x3 split A");
}

tmvg_status tf32x3_split_b(Context* c, int64_t n, int64_t K, const float* B, int64_t ldb,
                           const Tf32x3Buffers& b)
{
    if (n <= 0) return TMVG_OK;
    split_cols_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n * K, 256), 16 * c->num_sms), 256, 0,
                        c->stream>>>(n, (int)K, B, ldb, b.Bhi, b.Blo);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "tf32x3 split B");
}

tmvg_status gemm_f32_tf32x3_update(Context* c, int64_t m, int64_t n, int64_t K, const float* A,
                                   int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc)
{
    if (m <= 0 || n <= 0 || K <= 0) return TMVG_OK;
    if (!tf32x3_supported(K)) return set_error(c, TMVG_UNSUPPORTED, "tf32x3: K must be 32, 64, 96 or 128");
    if (m > INT_MAX || n > INT_MAX) return set_error(c, TMVG_UNSUPPORTED, "tf32x3: size");
    Tf32x3Buffers b;
    tmvg_status st = tf32x3_buffers(c, m, n, K, &b);
    if (!st) st = tf32x3_split_a(c, m, K, A, lda, b);
    if (!st) st = tf32x3_split_b(c, n, K, B, ldb, b);
    if (!st) st = tf32x3_apply(c, m, n, K, b, C, ldc);
    return st;
}

tmvg_status tf32x3_apply(Context* c, int64_t m, int64_t n, int64_t K, const Tf32x3Buffers& b, float* C,
                         int64_t ldc)
{
    if (m <= 0 || n <= 0 || K <= 0) return TMVG_OK;
    if (!tf32x3_supported(K)) return set_error(c, TMVG_UNSUPPORTED, "tf32x3: K must be 32, 64, 96 or 128");
    if (m > INT_MAX || n > INT_MAX) return set_error(c, TMVG_UNSUPPORTED, "tf32x3: size");
    const float *Ahi = b.Ahi, *Alo = b.Alo, *Bhi = b.Bhi, *Blo = b.Blo;
    const bool wide = n >= 128 && K <= 64;
    const int BN = wide ? 128 : 64;
    CUtensorMap maps[5];
    if (!make_map(&maps[0], Ahi, m, (int)K, kTcM) || !make_map(&maps[1], Alo, m, (int)K, kTcM) ||
        !make_map(&maps[2], Bhi, n, (int)K, BN) || !make_map(&maps[3], Blo, n, (int)K, BN))
        return set_error(c, TMVG_CUDA_ERROR, "tf32x3: tensor map encoding failed");
    // the C tile by TMA when C's base and column stride are 16-byte aligned
    const bool tmac = (reinterpret_cast<uintptr_t>(C) & 15) == 0 && ldc % 4 == 0 &&
                      make_c_map(&maps[4], C, m, n, ldc, BN);
    const int kch = (int)(K / kKChunk);
    if (wide) {
        if (kch == 1) return launch_update<128, 1>(c, maps, tmac, C, ldc, m, n);
        return launch_update<128, 2>(c, maps, tmac, C, ldc, m, n);
    }
    switch (kch) {
        case 1: return launch_update<64, 1>(c, maps, tmac, C, ldc, m, n);
        case 2: return launch_update<64, 2>(c, maps, tmac, C, ldc, m, n);
        case 3: return launch_update<64, 3>(c, maps, tmac, C, ldc, m, n);
        default: return launch_update<64, 4>(c, maps, tmac, C, ldc, m, n);
    }
}

}  // namespace tmvg
