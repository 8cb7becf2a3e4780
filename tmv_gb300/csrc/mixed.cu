// mixed.cu -- mixed-precision LU solve with FP64 iterative refinement.
//
//   As = fl32(A)              (one pass over A, also giving ||A||_inf)
//   P As = L U                (FP32 LU, the blocked factorisation of lu.cu)
//   x = U^-1 L^-1 P b         (FP32 solves, FP64 result)
//   repeat: r = b - A x       (FP64 residual, A read in FP64)
//           stop if ||r||_inf <= tol (||A||_inf ||x||_inf + ||b||_inf)
//           x += U^-1 L^-1 P r (FP32 solves of the residual, FP64 update)
//
// FP64 appears only where the refinement needs it: the residual, the
// correction update and (through pivot_key) the pivot comparisons.  The
// stopping test is the normwise backward error, the accuracy an FP64 LU solve
// itself delivers; with FP32-accurate factors one step contracts the error by
// about cond(A) * 2^-24, so cond <= 1e6 converges in a few steps.
#include "lu.cuh"
#include "mixed.cuh"
#include "trsv.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace tmvg {

constexpr int kChunk = 256;  // columns per residual/conversion partial sum

// Non-negative doubles order like their bit patterns, so max |v| can be
// reduced with integer atomics (deterministic: max is order independent).
__device__ __forceinline__ void atomic_max_abs(unsigned long long* dst, double v)
{
    atomicMax(dst, (unsigned long long)__double_as_longlong(fabs(v)));
}

// As = (float) A, and per-row partial sums of |A| over column chunks.  The
// sums are taken in FP32 over the converted values (two accumulators of 128
// terms): FP64 additions run at 1/64 of the FP32 rate on this part, and an
// FP64 sum per element made this pass FP64-bound (261 us at n = 8192 against
// 131 us, 91 % of the HBM copy rate, with FP32 sums).  Their relative error
// is below 2e-5; each partial is scaled down by (1 - 2^-12) so that ||A||_inf
// never comes out larger than it is and the backward error the refinement
// tests against (|r| / (||A|| ||x|| + ||b||)) never smaller.  A chunk whose
// FP32 sum overflows is summed again in FP64.
__global__ void prep_kernel(int64_t n, const double* __restrict__ A, int64_t lda,
                            float* __restrict__ As, int64_t ldas, double* __restrict__ rowpart)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t c0 = (int64_t)blockIdx.y * kChunk;
    if (i >= n) return;
    const int64_t c1 = min(n, c0 + kChunk);
    float s0 = 0.f, s1 = 0.f;
    int64_t c = c0;
    for (; c + 2 <= c1; c += 2) {
        const float v0 = (float)A[i + c * lda], v1 = (float)A[i + (c + 1) * lda];
        As[i + c * ldas] = v0;
        As[i + (c + 1) * ldas] = v1;
        s0 += fabsf(v0);
        s1 += fabsf(v1);
    }
    if (c < c1) {
        const float v = (float)A[i + c * lda];
        As[i + c * ldas] = v;
        s0 += fabsf(v);
    }
    double sum = ((double)s0 + (double)s1) * (1.0 - 0x1p-12);
    if (!isfinite(s0 + s1)) {
        // an FP32 sum that overflowed (entries near the FP32 limit), or a
        // NaN: the chunk again in FP64
        sum = 0.0;
        for (c = c0; c < c1; ++c) sum += fabs(A[i + c * lda]);
    }
    rowpart[blockIdx.y * n + i] = sum;
}

// ||A||_inf = max_i sum_chunks rowpart[chunk][i]
__global__ void rownorm_kernel(int64_t n, int nchunks, const double* __restrict__ rowpart,
                               unsigned long long* anorm)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = 0; k < nchunks; ++k) s += rowpart[k * n + i];
    atomic_max_abs(anorm, s);
}

__global__ void absmax_kernel(int64_t n, const double* __restrict__ v, int64_t inc,
                              unsigned long long* out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        atomic_max_abs(out, v[i * inc]);
}

__global__ void invert_perm_kernel(int64_t n, const int* __restrict__ perm, int* __restrict__ inv)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) inv[perm[i]] = (int)i;
}

// v32[i] = (float) b[perm[i]]
__global__ void gather_to_f32_kernel(int64_t n, const int* __restrict__ perm,
                                     const double* __restrict__ b, int64_t inc, float* __restrict__ v)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = (float)b[(int64_t)perm[i] * inc];
}

// x (+)= (double) v32 (nothing once *stop is set)
__global__ void update_kernel(int64_t n, const float* __restrict__ v, double* __restrict__ x,
                              int64_t inc, bool add, const int* stop)
{
    if (stop && *stop) return;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) x[i * inc] = add ? x[i * inc] + (double)v[i] : (double)v[i];
}

// Residual partial sums: part[chunk][i] = sum_{c in chunk} A[i,c] x[c] (FP64).
__global__ void __launch_bounds__(256)
residual_partial_kernel(int64_t n, const double* __restrict__ A, int64_t lda,
                        const double* __restrict__ x, int64_t incx, double* __restrict__ part,
                        const int* stop)
{
    if (*stop) return;
    __shared__ double xs[kChunk];
    const int64_t c0 = (int64_t)blockIdx.y * kChunk;
    const int cn = (int)min((int64_t)kChunk, n - c0);
    for (int t = threadIdx.x; t < cn; t += blockDim.x) xs[t] = x[(c0 + t) * incx];
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = A + i + c0 * lda;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int c = 0;
    for (; c + 4 <= cn; c += 4) {
        s0 = fma(a[(c + 0) * lda], xs[c + 0], s0);
        s1 = fma(a[(c + 1) * lda], xs[c + 1], s1);
        s2 = fma(a[(c + 2) * lda], xs[c + 2], s2);
        s3 = fma(a[(c + 3) * lda], xs[c + 3], s3);
    }
    for (; c < cn; ++c) s0 = fma(a[c * lda], xs[c], s0);
    part[blockIdx.y * n + i] = (s0 + s1) + (s2 + s3);
}

// r_i = b_i - sum part[.][i]; rp[inv[i]] = (float) r_i (pivoted FP32
// right-hand side of the correction solve); max |r| and max |x|.
__global__ void residual_final_kernel(int64_t n, int nchunks, const double* __restrict__ part,
                                      const double* __restrict__ b, int64_t incb,
                                      const double* __restrict__ x, int64_t incx,
                                      const int* __restrict__ inv, float* __restrict__ rp,
                                      unsigned long long* rmax, unsigned long long* xmax,
                                      const int* stop)
{
    if (*stop) return;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = 0; k < nchunks; ++k) s += part[k * n + i];
    const double r = b[i * incb] - s;
    rp[inv[i]] = (float)r;
    atomic_max_abs(rmax, r);
    atomic_max_abs(xmax, x[i * incx]);
}

// The refinement loop's state on the device, so that the loop runs without
// a host round trip per step: the host enqueues max_iter steps, each step's
// kernels return at once when `done` is set, and one copy at the end reads
// the summary.
struct IrState {
    int done;       // this right-hand side has stopped
    int conv;       // ... with the backward error at or below tol
    int iters;      // corrections applied to this right-hand side
    int pad;
    double berr;    // its last backward error
    // over all right-hand sides
    int worst_iters;
    int all_conv;
    double worst_berr;
    double anorm;
};

// After step it's residual: the normwise backward error
// ||r|| / (||A|| ||x|| + ||b||) from the reduced norms sc = (||A||, ||b||,
// ||r||, ||x||) (bit patterns of non-negative doubles); stop on tol, on
// max_iter corrections or on NaN (recording in *iters_q the corrections this
// right-hand side received); fold a stopped right-hand side into the
// summary; clear ||r|| and ||x|| for the next residual.
__global__ void ir_check_kernel(unsigned long long* sc, double tol, int it, int max_iter, IrState* st,
                                int* iters_q)
{
    if (st->done) return;
    const double an = __longlong_as_double((long long)sc[0]);
    const double bn = __longlong_as_double((long long)sc[1]);
    const double rn = __longlong_as_double((long long)sc[2]);
    const double xn = __longlong_as_double((long long)sc[3]);
    const double denom = an * xn + bn;
    const double berr = denom > 0 ? rn / denom : (rn == 0 ? 0.0 : INFINITY);
    st->berr = berr;
    st->iters = it;
    st->anorm = an;
    const bool conv = berr <= tol;
    if (conv || it >= max_iter || !(berr == berr)) {
        st->done = 1;
        *iters_q = it;
        st->conv = conv ? 1 : 0;
        st->worst_iters = max(st->worst_iters, it);
        st->worst_berr = fmax(st->worst_berr, berr);  // NaN-free unless berr is NaN
        if (!(berr == berr)) st->worst_berr = berr;
        st->all_conv = st->all_conv && conv;
    }
    sc[2] = 0ull;
    sc[3] = 0ull;
}

// A new right-hand side: clear its stop flag (the summary carries over).
__global__ void ir_begin_kernel(IrState* st, int first)
{
    st->done = 0;
    st->conv = 0;
    st->iters = 0;
    st->berr = 0.0;
    if (first) {
        st->worst_iters = 0;
        st->all_conv = 1;
        st->worst_berr = 0.0;
        st->anorm = 0.0;
    }
}

static inline unsigned blocks_for(int64_t n, int t) { return (unsigned)ceil_div(n, t); }

tmvg_status lu_solve_mixed(Context* c, int64_t n, const double* A, int64_t lda, int64_t nrhs,
                           const double* B, int64_t ldb, double* X, int64_t ldx, int max_iter,
                           double tol, tmvg_ir_info* info)
{
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(n, 1) ||
        ldx < std::max<int64_t>(n, 1) || max_iter < 0)
        return set_error(c, TMVG_BAD_ARG, "lu_solve_mixed: bad sizes");
    if (info) *info = tmvg_ir_info{0, 1, 0.0, 0.0};
    if (n == 0 || nrhs == 0) return TMVG_OK;

    const int nchunks = (int)ceil_div(n, kChunk);
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_As = 0;
    const size_t o_P = o_As + al(sizeof(float) * (size_t)n * n);
    const size_t o_perm = o_P + al(sizeof(int64_t) * n);
    const size_t o_inv = o_perm + al(sizeof(int) * n);
    const size_t o_v = o_inv + al(sizeof(int) * n);
    const size_t o_part = o_v + al(sizeof(float) * n);
    const size_t o_sc = o_part + al(sizeof(double) * (size_t)nchunks * n);
    const int64_t nib = ceil_div(n, kInvBlock);
    const size_t o_dl = o_sc + 256;
    const size_t o_du = o_dl + al(sizeof(float) * (size_t)nib * kInvBlock * kInvBlock);
    const size_t o_sg = o_du + al(sizeof(float) * (size_t)nib * kInvBlock * kInvBlock);
    const size_t o_ml = o_sg + al(sizeof(int) * 2 * nib);
    const size_t o_mu = o_ml + al(sizeof(float) * (size_t)nib * kInvBlock * kInvBlock);
    const size_t o_ir = o_mu + al(sizeof(float) * (size_t)nib * kInvBlock * kInvBlock);
    const size_t o_iq = o_ir + al(sizeof(IrState));
    const size_t bytes = o_iq + al(sizeof(int) * (size_t)nrhs);
    unsigned char* ws = (unsigned char*)workspace2(c, bytes);
    if (!ws) return TMVG_OOM;
    float* As = (float*)(ws + o_As);
    int64_t* P = (int64_t*)(ws + o_P);
    int* perm = (int*)(ws + o_perm);
    int* inv = (int*)(ws + o_inv);
    float* v = (float*)(ws + o_v);
    double* part = (double*)(ws + o_part);
    unsigned long long* sc = (unsigned long long*)(ws + o_sc);  // anorm, bmax, rmax, xmax
    IrState* irs = (IrState*)(ws + o_ir);
    int* iters_q = (int*)(ws + o_iq);  // corrections applied, per right-hand side
    const int* stop = &irs->done;
    // With kernel timing on, the spans of each enqueued step, so that the
    // steps the device skipped can be dropped once the loop is known.
    struct StepSpans {
        int64_t q;
        int it;
        size_t res0, res1, cor0, cor1;
    };
    std::vector<StepSpans> step_spans;
    float* dinvL = (float*)(ws + o_dl);
    float* dinvU = (float*)(ws + o_du);
    int* singL = (int*)(ws + o_sg);
    int* singU = singL + nib;
    float* mlinkL = (float*)(ws + o_ml);
    float* mlinkU = (float*)(ws + o_mu);

    tmvg_status st;
    auto launched = [&](const char* what) {
        ++c->launches;
        return check_cuda(c, cudaGetLastError(), what);
    };

    // 1. FP32 copy and ||A||_inf
    st = check_cuda(c, cudaMemsetAsync(sc, 0, 4 * sizeof(unsigned long long), c->stream), "memset");
    if (st) return st;
    prep_kernel<<<dim3(blocks_for(n, 256), nchunks), 256, 0, c->stream>>>(n, A, lda, As, n, part);
    if ((st = launched("prep"))) return st;
    rownorm_kernel<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, nchunks, part, sc + 0);
    if ((st = launched("rownorm"))) return st;

    // 2. FP32 factorisation
    st = lu_factor<float>(c, n, As, n, P);
    if (st) return st;
    st = pivots_to_perm(c, n, P, perm);
    if (st) return st;
    invert_perm_kernel<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, perm, inv);
    if ((st = launched("invperm"))) return st;
    // inverses of the 128 x 128 diagonal blocks of L and U, reused by every
    // solve of the refinement loop
    st = trsv_lu_inverse_blocks<float>(c, n, As, n, dinvL, singL, dinvU, singU);
    if (st) return st;
    // and the link blocks M_b = Dinv_b T[b, b-1] of both triangles
    st = trsv_lu_link_blocks(c, n, As, n, dinvL, singL, mlinkL, dinvU, singU, mlinkU);
    if (st) return st;
    // one triangular solve reads its triangle, the inverted diagonal blocks
    // and the vector (in and out)
    const double fn = (double)n;
    const double tri_bytes = 4.0 * (fn * (fn + 1) / 2 + fn * kInvBlock + 2 * fn);
    auto solve32 = [&](float* vec, const int* stp) -> tmvg_status {
        tmvg_status s2;
        {
            ScopedTimer timer(c, kClsTriSolve, tri_bytes, fn * fn);
            s2 = trsv_with_inverse_blocks<float>(c, n, As, 1, n, false, true, dinvL, singL, vec, 1,
                                                 true, stp, mlinkL);
        }
        if (s2) return s2;
        ScopedTimer timer(c, kClsTriSolve, tri_bytes, fn * fn);
        return trsv_with_inverse_blocks<float>(c, n, As, 1, n, true, false, dinvU, singU, vec, 1,
                                               true, stp, mlinkU);
    };

    // All steps of all right-hand sides are enqueued without a host round
    // trip: ir_check_kernel decides on the device after each residual, and
    // the kernels of the steps after it return at once.
    for (int64_t q = 0; q < nrhs; ++q) {
        const double* b = B + q * ldb;
        double* x = X + q * ldx;
        ir_begin_kernel<<<1, 1, 0, c->stream>>>(irs, q == 0 ? 1 : 0);
        if ((st = launched("ir begin"))) return st;
        st = check_cuda(c, cudaMemsetAsync(sc + 1, 0, 3 * sizeof(unsigned long long), c->stream),
                        "memset");
        if (st) return st;
        absmax_kernel<<<std::min<unsigned>(blocks_for(n, 256), 64), 256, 0, c->stream>>>(n, b, 1,
                                                                                         sc + 1);
        if ((st = launched("bmax"))) return st;
        // 3. initial solve
        gather_to_f32_kernel<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, perm, b, 1, v);
        if ((st = launched("gather"))) return st;
        st = solve32(v, nullptr);
        if (st) return st;
        update_kernel<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, v, x, 1, false, nullptr);
        if ((st = launched("update"))) return st;
        for (int it = 0; it <= max_iter; ++it) {
            StepSpans ss{q, it, c->spans.size(), 0, 0, 0};
            // 4. FP64 residual, pivoted FP32 copy, norms, stopping test
            {
                // reads A (FP64) once, x per column chunk, b; writes the FP32 residual
                ScopedTimer timer(c, kClsResidual, 8.0 * fn * fn + 8.0 * fn * (nchunks + 1) + 4.0 * fn,
                                  2.0 * fn * fn);
                residual_partial_kernel<<<dim3(blocks_for(n, 256), nchunks), 256, 0, c->stream>>>(
                    n, A, lda, x, 1, part, stop);
                if ((st = launched("residual"))) return st;
                residual_final_kernel<<<blocks_for(n, 256), 256, 0, c->stream>>>(
                    n, nchunks, part, b, 1, x, 1, inv, v, sc + 2, sc + 3, stop);
                if ((st = launched("residual_final"))) return st;
            }
            ss.res1 = c->spans.size();
            ir_check_kernel<<<1, 1, 0, c->stream>>>(sc, tol, it, max_iter, irs, iters_q + q);
            if ((st = launched("ir check"))) return st;
            ss.cor0 = c->spans.size();
            if (it < max_iter) {
                // 5. correction
                st = solve32(v, stop);
                if (st) return st;
                update_kernel<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, v, x, 1, true, stop);
                if ((st = launched("update"))) return st;
            }
            ss.cor1 = c->spans.size();
            if (c->timing) step_spans.push_back(ss);
        }
    }
    IrState hs;
    st = check_cuda(c, cudaMemcpyAsync(&hs, irs, sizeof(hs), cudaMemcpyDeviceToHost, c->stream),
                    "ir state d2h");
    if (st) return st;
    st = collect_device_error(c, "lu_solve_mixed");  // synchronises the stream
    if (st) return st;
    if (!step_spans.empty()) {
        // drop the timed spans of the steps the device skipped: the residual
        // of step it ran iff it <= iters, its correction iff it < iters
        std::vector<int> iq((size_t)nrhs);
        st = check_cuda(c, cudaMemcpy(iq.data(), iters_q, sizeof(int) * (size_t)nrhs, cudaMemcpyDeviceToHost),
                        "ir iterations d2h");
        if (st) return st;
        std::vector<char> drop(c->spans.size(), 0);
        for (const StepSpans& ss : step_spans) {
            const int done_at = iq[(size_t)ss.q];
            if (ss.it > done_at)
                for (size_t k = ss.res0; k < ss.res1; ++k) drop[k] = 1;
            if (ss.it >= done_at)
                for (size_t k = ss.cor0; k < ss.cor1; ++k) drop[k] = 1;
        }
        std::vector<TimedSpan> kept;
        kept.reserve(c->spans.size());
        for (size_t k = 0; k < c->spans.size(); ++k) {
            if (drop[k]) {
                c->event_pool.push_back(c->spans[k].a);
                c->event_pool.push_back(c->spans[k].b);
            } else {
                kept.push_back(c->spans[k]);
            }
        }
        c->spans.swap(kept);
    }
    const int worst_iters = hs.worst_iters;
    const bool all_conv = hs.all_conv != 0;
    const double worst_berr = hs.worst_berr, anorm = hs.anorm;
    if (info) *info = tmvg_ir_info{worst_iters, all_conv ? 1 : 0, worst_berr, anorm};
    if (!all_conv)
        return set_error(c, TMVG_NOT_CONVERGED,
                         "lu_solve_mixed: backward error above tolerance after max_iter steps");
    return TMVG_OK;
}

}  // namespace tmvg
