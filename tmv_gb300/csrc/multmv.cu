// multmv.cu -- y (+)= alpha A x on sm_103a (tmv::MultMV<add>, src/TMV_MultMV.cpp:1134-1175).
//
// FP64, HBM-bound (8mn bytes of A per product, 2mn flops).  The two forms
// of TMV's UnitAMultMV1 (src/TMV_MultMV.cpp:186-215), chosen the same way
// (row form for a row-major A, column form for a column-major one, else the
// row form when N >= M):
//   * column form (ColMultMV, :124-184): a column sweep, one thread per two
//     adjacent rows, the columns split into chunks of kMvChunk over blockIdx.y; a column
//     whose x_j is zero is skipped, as TMV skips it (a NaN there does not
//     reach y); each chunk writes its partial sums and one pass adds the
//     chunks in order and applies alpha and add;
//   * row form (RowMultMV, :80-122): one warp per row, lanes striding the
//     row, shuffle reduction, every product taken.
// x is first copied into scratch, so x and y may share storage (TMV copies x
// then, src/TMV_MultMV.cpp:1097-1110).
// alpha == 0 or an empty x leaves A unread: y = 0 (add = false) or unchanged,
// as TMV's MultMV does.
#include "multmv.cuh"

#include <algorithm>

namespace tmvg {

constexpr int kMvChunk = 256;  // columns per partial sum of the column sweep (1024 CTAs at 8192^2)
constexpr int kMvThreads = 256;

__global__ void mv_copy_kernel(int64_t n, const double* __restrict__ x, int64_t incx, double* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = x[i * incx];
}

// part[chunk * m + i] = sum_{j in chunk} A[i, j] x[j]; with a unit row step
// each thread takes two adjacent rows (one 16-byte load per column)
__global__ void __launch_bounds__(kMvThreads)
mv_cols_partial_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t sAi, int64_t sAj,
                       const double* __restrict__ x, double* __restrict__ part)
{
    __shared__ double xs[kMvChunk];
    const int64_t j0 = (int64_t)blockIdx.y * kMvChunk;
    const int cn = (int)min((int64_t)kMvChunk, n - j0);
    for (int t = threadIdx.x; t < cn; t += blockDim.x) xs[t] = x[j0 + t];
    __syncthreads();
    const int64_t i = 2 * (blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
    if (i >= m) return;
    const double* a = A + i * sAi + j0 * sAj;
    // a column with x_j == 0 keeps the sums as they are (TMV skips it)
    const bool pair = sAi == 1 && i + 1 < m && ((reinterpret_cast<uintptr_t>(a) | (uintptr_t)(sAj * 8)) & 15) == 0;
    double s0 = 0.0, s1 = 0.0, t0 = 0.0, t1 = 0.0;
    if (pair) {
        int j = 0;
        for (; j + 2 <= cn; j += 2) {
            const double2 v0 = *reinterpret_cast<const double2*>(a + (int64_t)j * sAj);
            const double2 v1 = *reinterpret_cast<const double2*>(a + (int64_t)(j + 1) * sAj);
            const double x0 = xs[j], x1 = xs[j + 1];
            if (x0 != 0.0) { s0 = fma(v0.x, x0, s0); t0 = fma(v0.y, x0, t0); }
            if (x1 != 0.0) { s1 = fma(v1.x, x1, s1); t1 = fma(v1.y, x1, t1); }
        }
        if (j < cn) {
            const double2 v0 = *reinterpret_cast<const double2*>(a + (int64_t)j * sAj);
            if (xs[j] != 0.0) { s0 = fma(v0.x, xs[j], s0); t0 = fma(v0.y, xs[j], t0); }
        }
        part[(int64_t)blockIdx.y * m + i] = s0 + s1;
        part[(int64_t)blockIdx.y * m + i + 1] = t0 + t1;
        return;
    }
    for (int r = 0; r < 2 && i + r < m; ++r) {
        const double* ar = a + r * sAi;
        double u0 = 0.0, u1 = 0.0;
        int j = 0;
        for (; j + 2 <= cn; j += 2) {
            if (xs[j] != 0.0) u0 = fma(ar[(int64_t)j * sAj], xs[j], u0);
            if (xs[j + 1] != 0.0) u1 = fma(ar[(int64_t)(j + 1) * sAj], xs[j + 1], u1);
        }
        if (j < cn && xs[j] != 0.0) u0 = fma(ar[(int64_t)j * sAj], xs[j], u0);
        part[(int64_t)blockIdx.y * m + i + r] = u0 + u1;
    }
}

__global__ void mv_cols_final_kernel(int64_t m, int nchunks, const double* __restrict__ part, double alpha,
                                     bool add, double* __restrict__ y, int64_t incy)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < nchunks; ++k) s += part[(int64_t)k * m + i];
        const double v = alpha * s;
        y[i * incy] = add ? y[i * incy] + v : v;
    }
}

// one warp per row (row form)
__global__ void __launch_bounds__(kMvThreads)
mv_rows_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t sAi, int64_t sAj,
               const double* __restrict__ x, double alpha, bool add, double* __restrict__ y, int64_t incy)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); i < m; i += warps) {
        const double* a = A + i * sAi;
        double s0 = 0.0, s1 = 0.0;
        int64_t j = lane;
        for (; j + 32 < n; j += 64) {
            s0 = fma(a[j * sAj], x[j], s0);
            s1 = fma(a[(j + 32) * sAj], x[j + 32], s1);
        }
        if (j < n) s0 = fma(a[j * sAj], x[j], s0);
        double s = s0 + s1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            const double v = alpha * s;
            y[i * incy] = add ? y[i * incy] + v : v;
        }
    }
}

__global__ void mv_scale_kernel(int64_t m, double* __restrict__ y, int64_t incy)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        y[i * incy] = 0.0;
}

tmvg_status multmv(Context* c, bool add, double alpha, int64_t m, int64_t n, const double* A, int64_t sAi,
                   int64_t sAj, const double* x, int64_t incx, double* y, int64_t incy)
{
    if (m <= 0) return TMVG_OK;
    const unsigned grid_m = (unsigned)std::min<int64_t>(ceil_div(m, kMvThreads), 8 * c->num_sms);
    if (n <= 0 || alpha == 0.0) {
        if (add) return TMVG_OK;
        mv_scale_kernel<<<grid_m, kMvThreads, 0, c->stream>>>(m, y, incy);
        ++c->launches;
        return check_cuda(c, cudaGetLastError(), "multmv: zero launch");
    }
    // TMV's UnitAMultMV1 choice, in its order: A.isrm() (unit column step)
    // takes the row form, A.iscm() the column form, otherwise N >= M the row form
    const bool rows = sAj == 1 || (sAi != 1 && n >= m);
    const int nchunks = rows ? 0 : (int)ceil_div(n, kMvChunk);
    const size_t xbytes = (sizeof(double) * (size_t)n + 255) & ~size_t(255);
    unsigned char* ws = (unsigned char*)workspace(c, xbytes + sizeof(double) * (size_t)m * nchunks);
    if (!ws) return TMVG_OOM;
    double* xc = (double*)ws;
    double* part = (double*)(ws + xbytes);
    ScopedTimer timer(c, kClsResidual, 8.0 * (double)m * n, 2.0 * (double)m * n);
    mv_copy_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n, kMvThreads), 8 * c->num_sms), kMvThreads, 0,
                     c->stream>>>(n, x, incx, xc);
    ++c->launches;
    tmvg_status st = check_cuda(c, cudaGetLastError(), "multmv: copy launch");
    if (st) return st;
    if (rows) {
        const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(m, kMvThreads / 32), 32 * c->num_sms);
        mv_rows_kernel<<<blocks, kMvThreads, 0, c->stream>>>(m, n, A, sAi, sAj, xc, alpha, add, y, incy);
        ++c->launches;
        return check_cuda(c, cudaGetLastError(), "multmv: rows launch");
    }
    dim3 g((unsigned)ceil_div(m, 2 * kMvThreads), (unsigned)nchunks);
    if (g.x > 65535u * 1024u || g.y > 65535u) return set_error(c, TMVG_UNSUPPORTED, "multmv: matrix too large");
    mv_cols_partial_kernel<<<g, kMvThreads, 0, c->stream>>>(m, n, A, sAi, sAj, xc, part);
    ++c->launches;
    st = check_cuda(c, cudaGetLastError(), "multmv: partial launch");
    if (st) return st;
    mv_cols_final_kernel<<<grid_m, kMvThreads, 0, c->stream>>>(m, nchunks, part, alpha, add, y, incy);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "multmv: final launch");
}

}  // namespace tmvg
