// gemm_simt.cu -- FP64 (DFMA) and FP32 (FFMA) tiled products.
//
// GB300 executes FP64 at about 2 DFMA per SM per clock (the library's DFMA
// rate probe, tmvg_probe_fp64_rate, reads about 1.25 TFLOP/s at 2070 MHz),
// so a register-tiled DFMA kernel is the native FP64 engine: it keeps the
// FP64 pipe issuing every cycle without needing the tensor path.  The FP32 variant (about 70 TFLOP/s
// FFMA) serves the mixed-precision trailing updates.
//
// Layouts: op(A)(i,k) is A[i + k*lda] (column-major) or A[i*lda + k]
// (row-major); likewise B.  C is column-major (a row-major C is handled by
// the dispatcher through C^T = B^T A^T, as TMV's MultMM does,
// src/TMV_MultMM.cpp:447-448).  Each thread owns a TM x TN block of C whose
// rows are consecutive, so a warp stores 16*TM consecutive rows per column.
#include "gemm.cuh"

#include <algorithm>

namespace tmvg {

template <typename T, int TM, int TN, int BK, bool ARM, bool BRM>
__global__ void __launch_bounds__(256)
gemm_simt_kernel(int64_t M, int64_t N, int64_t K, T alpha,
                 const T* __restrict__ A, int64_t lda,
                 const T* __restrict__ B, int64_t ldb, T beta,
                 T* __restrict__ C, int64_t ldc)
{
    constexpr int BM = 16 * TM, BN = 16 * TN;
    constexpr int NA = BM * BK / 256, NB = BN * BK / 256;
    static_assert(NA * 256 == BM * BK && NB * 256 == BN * BK, "tile");
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t i0 = (int64_t)blockIdx.x * BM;
    const int64_t j0 = (int64_t)blockIdx.y * BN;

    T acc[TM][TN];
#pragma unroll
    for (int r = 0; r < TM; ++r)
#pragma unroll
        for (int s = 0; s < TN; ++s) acc[r][s] = T(0);

    T ra[NA], rb[NB];
    auto load = [&](int64_t k0) {
#pragma unroll
        for (int t = 0; t < NA; ++t) {
            const int idx = tid + t * 256;
            int ii, kk;
            if (ARM) { ii = idx / BK; kk = idx % BK; }
            else { ii = idx % BM; kk = idx / BM; }
            const int64_t gi = i0 + ii, gk = k0 + kk;
            T v = T(0);
            if (gi < M && gk < K) v = ARM ? A[gi * lda + gk] : A[gi + gk * lda];
            ra[t] = v;
        }
#pragma unroll
        for (int t = 0; t < NB; ++t) {
            const int idx = tid + t * 256;
            int jj, kk;
            if (BRM) { jj = idx % BN; kk = idx / BN; }
            else { jj = idx / BK; kk = idx % BK; }
            const int64_t gj = j0 + jj, gk = k0 + kk;
            T v = T(0);
            if (gj < N && gk < K) v = BRM ? B[gk * ldb + gj] : B[gk + gj * ldb];
            rb[t] = v;
        }
    };
    auto store = [&]() {
#pragma unroll
        for (int t = 0; t < NA; ++t) {
            const int idx = tid + t * 256;
            int ii, kk;
            if (ARM) { ii = idx / BK; kk = idx % BK; }
            else { ii = idx % BM; kk = idx / BM; }
            As[kk][ii] = ra[t];
        }
#pragma unroll
        for (int t = 0; t < NB; ++t) {
            const int idx = tid + t * 256;
            int jj, kk;
            if (BRM) { jj = idx % BN; kk = idx / BN; }
            else { jj = idx / BK; kk = idx % BK; }
            Bs[kk][jj] = rb[t];
        }
    };

    load(0);
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
        __syncthreads();
        store();
        __syncthreads();
        if (k0 + BK < K) load(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T a[TM], b[TN];
#pragma unroll
            for (int r = 0; r < TM; ++r) a[r] = As[kk][tx * TM + r];
#pragma unroll
            for (int s = 0; s < TN; ++s) b[s] = Bs[kk][ty * TN + s];
#pragma unroll
            for (int r = 0; r < TM; ++r)
#pragma unroll
                for (int s = 0; s < TN; ++s) acc[r][s] = fma(a[r], b[s], acc[r][s]);
        }
    }

#pragma unroll
    for (int s = 0; s < TN; ++s) {
        const int64_t gj = j0 + ty * TN + s;
        if (gj >= N) continue;
#pragma unroll
        for (int r = 0; r < TM; ++r) {
            const int64_t gi = i0 + tx * TM + r;
            if (gi >= M) continue;
            T* cp = C + gi + gj * ldc;
            const T v = alpha * acc[r][s];
            *cp = beta == T(0) ? v : v + beta * (*cp);
        }
    }
}

template <typename T>
struct SimtTile;
template <>
struct SimtTile<double> { static constexpr int TM = 4, TN = 4, BK = 16; };
template <>
struct SimtTile<float> { static constexpr int TM = 8, TN = 8, BK = 8; };

// Half-size tiles for products whose full-size grid would not cover the SMs
// (the narrow updates of blocked triangular solves: m x 64 x 64).  Each C
// element is still one thread's k-ordered FMA chain, so the result does not
// depend on the tile size.
template <typename T>
struct SimtSmallTile;
template <>
struct SimtSmallTile<double> { static constexpr int TM = 2, TN = 2, BK = 16; };
template <>
struct SimtSmallTile<float> { static constexpr int TM = 4, TN = 4, BK = 8; };

template <typename T, bool ARM, bool BRM>
static tmvg_status launch_gemm(Context* c, int64_t m, int64_t n, int64_t k, T alpha,
                               const T* A, int64_t lda, const T* B, int64_t ldb,
                               T beta, T* C, int64_t ldc)
{
    constexpr int TM = SimtTile<T>::TM, TN = SimtTile<T>::TN, BK = SimtTile<T>::BK;
    dim3 grid((unsigned)ceil_div(m, 16 * TM), (unsigned)ceil_div(n, 16 * TN));
    if ((int64_t)grid.x * grid.y < c->num_sms) {
        constexpr int STM = SimtSmallTile<T>::TM, STN = SimtSmallTile<T>::TN, SBK = SimtSmallTile<T>::BK;
        dim3 g2((unsigned)ceil_div(m, 16 * STM), (unsigned)ceil_div(n, 16 * STN));
        if (g2.y > 65535) return set_error(c, TMVG_UNSUPPORTED, "gemm: n too large");
        gemm_simt_kernel<T, STM, STN, SBK, ARM, BRM><<<g2, 256, 0, c->stream>>>(
            m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        ++c->launches;
        return check_cuda(c, cudaGetLastError(), "gemm launch");
    }
    if (grid.y > 65535) return set_error(c, TMVG_UNSUPPORTED, "gemm: n too large");
    gemm_simt_kernel<T, TM, TN, BK, ARM, BRM><<<grid, 256, 0, c->stream>>>(
        m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "gemm launch");
}

// Scale C by beta (0 or 1) when there is nothing to multiply.
template <typename T>
__global__ void scale_kernel(int64_t m, int64_t n, T* C, int64_t si, int64_t sj, T beta)
{
    const int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % m, j = t / m;
        T* p = C + i * si + j * sj;
        *p = beta == T(0) ? T(0) : beta * (*p);
    }
}

template <typename T>
tmvg_status gemm(Context* c, int64_t m, int64_t n, int64_t k, T alpha,
                 Mat<const T> A, Mat<const T> B, T beta, Mat<T> C)
{
    if (m < 0 || n < 0 || k < 0) return set_error(c, TMVG_BAD_ARG, "gemm: negative size");
    if (m == 0 || n == 0) return TMVG_OK;
    if (k == 0 || alpha == T(0)) {
        if (beta == T(1)) return TMVG_OK;
        scale_kernel<T><<<(unsigned)std::min<int64_t>(ceil_div(m * n, 256), 4096), 256, 0, c->stream>>>(
            m, n, C.p, C.si, C.sj, beta);
        ++c->launches;
        return check_cuda(c, cudaGetLastError(), "scale launch");
    }
    // C must be usable column-major (stepi == 1, or a single row); otherwise
    // a row-major C is computed as C^T = B^T A^T (src/TMV_MultMM.cpp:447-448).
    if (!(C.si == 1 || m == 1)) {
        if (!(C.sj == 1 || n == 1))
            return set_error(c, TMVG_BAD_ARG, "gemm: C must be column- or row-major");
        return gemm<T>(c, n, m, k, alpha, Mat<const T>{B.p, B.sj, B.si},
                       Mat<const T>{A.p, A.sj, A.si}, beta, Mat<T>{C.p, C.sj, C.si});
    }
    const int64_t ldc = (n == 1) ? std::max<int64_t>(m, 1) : C.sj;
    // Operand classification: column-major usable when stepi == 1 (or one
    // row), row-major usable when stepj == 1 (or one column).
    auto classify = [](int64_t rows, int64_t cols, int64_t si, int64_t sj, bool& rm,
                       int64_t& ld) -> bool {
        if (si == 1 || rows == 1) {
            rm = false;
            ld = cols == 1 ? std::max<int64_t>(rows, 1) : sj;
            return true;
        }
        if (sj == 1 || cols == 1) {
            rm = true;
            ld = rows == 1 ? std::max<int64_t>(cols, 1) : si;
            return true;
        }
        return false;
    };
    bool arm = false, brm = false;
    int64_t lda = 0, ldb = 0;
    if (!classify(m, k, A.si, A.sj, arm, lda) || !classify(k, n, B.si, B.sj, brm, ldb))
        return set_error(c, TMVG_BAD_ARG, "gemm: A and B must be column- or row-major");
    if (arm) {
        if (brm) return launch_gemm<T, true, true>(c, m, n, k, alpha, A.p, lda, B.p, ldb, beta, C.p, ldc);
        return launch_gemm<T, true, false>(c, m, n, k, alpha, A.p, lda, B.p, ldb, beta, C.p, ldc);
    }
    if (brm) return launch_gemm<T, false, true>(c, m, n, k, alpha, A.p, lda, B.p, ldb, beta, C.p, ldc);
    return launch_gemm<T, false, false>(c, m, n, k, alpha, A.p, lda, B.p, ldb, beta, C.p, ldc);
}

template tmvg_status gemm<double>(Context*, int64_t, int64_t, int64_t, double, Mat<const double>,
                                  Mat<const double>, double, Mat<double>);
template tmvg_status gemm<float>(Context*, int64_t, int64_t, int64_t, float, Mat<const float>,
                                 Mat<const float>, float, Mat<float>);

}  // namespace tmvg
