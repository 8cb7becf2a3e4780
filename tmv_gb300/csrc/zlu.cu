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
// Complex products are (ac - bd, ad + bc) with separately rounded products
// (no fused multiply-add), as the host computes them.
//
// A first GPU form: right-looking, one column per step (pivot search in one
// CTA, row interchange, scaling, rank-1 update over the grid), the left
// solve one CTA per right-hand side, the right solve (LU_RDivEq) one row per
// CTA substituted in TMV's order.  Values agree with TMV's recursive factorisation
// to rounding; pivots are TMV's wherever rounding does not decide a tie.
#include "zlu.cuh"

#include <algorithm>

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

tmvg_status zlu_factor(Context* c, int64_t n, double2* A, int64_t lda, int64_t* P)
{
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "lu_z: bad n/lda");
    if (n == 0) return TMVG_OK;
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

tmvg_status zlu_ldiveq(Context* c, int64_t n, const double2* LU, int64_t lda, const int64_t* P, int64_t nrhs,
                       double2* B, int64_t ldb)
{
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "lu_ldiveq_z: bad sizes");
    if (n == 0 || nrhs == 0) return TMVG_OK;
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
