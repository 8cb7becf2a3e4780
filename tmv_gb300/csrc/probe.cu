// probe.cu -- the FP64 FMA rate of the device, measured in the caller's
// process: the denominator of every FP64-bound roofline fraction, taken
// under the same clocks as the work it is compared with.
#include <string>

#include "common.cuh"

namespace tmvg {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 8;  // independent FMA chains per thread

// Each thread runs kProbeChains independent chains x <- x * a + b (a just
// below 1, b small, so values stay bounded and no chain can be folded),
// iters times each, and stores the sum so that nothing is dead code.
__global__ void __launch_bounds__(kProbeThreads)
dfma_rate_kernel(double* __restrict__ out, int iters, double a, double b)
{
    double x[kProbeChains];
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) x[j] = 1.0 + 1e-3 * (threadIdx.x + j);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
#pragma unroll
            for (int j = 0; j < kProbeChains; ++j) x[j] = fma(x[j], a, b);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) s += x[j];
    out[blockIdx.x * kProbeThreads + threadIdx.x] = s;
}

}  // namespace

tmvg_status probe_fp64_rate(Context* c, double* tflops)
{
    const int blocks = c->num_sms * 4;
    const int iters = 2048;
    double* out = static_cast<double*>(workspace(c, sizeof(double) * blocks * kProbeThreads));
    if (!out) return TMVG_OOM;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        return set_error(c, TMVG_CUDA_ERROR, "probe: event creation failed");
    }
    const double fmas = (double)blocks * kProbeThreads * kProbeChains * 4.0 * iters;
    float best = 0.0f;
    tmvg_status st = TMVG_OK;
    for (int rep = 0; rep < 4 && st == TMVG_OK; ++rep) {  // the first launch warms up
        cudaEventRecord(e0, c->stream);
        dfma_rate_kernel<<<blocks, kProbeThreads, 0, c->stream>>>(out, iters, 0.9999999, 1e-7);
        ++c->launches;
        cudaEventRecord(e1, c->stream);
        st = check_cuda(c, cudaEventSynchronize(e1), "probe: dfma_rate_kernel");
        float ms = 0.0f;
        if (st == TMVG_OK && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.0f &&
            (best == 0.0f || ms < best))
            best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    *tflops = best > 0.0f ? 2.0 * fmas / (best * 1e-3) / 1e12 : 0.0;
    return TMVG_OK;
}

}  // namespace tmvg
