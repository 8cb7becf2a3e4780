// capi.cu -- extern "C" entry points (include/tmvg.h) and context plumbing.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <complex>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "gemm_tc.cuh"
#include "lu.cuh"
#include "mixed.cuh"
#include "multmv.cuh"
#include "zlu.cuh"
#include "trsv.cuh"

namespace tmvg {

tmvg_status set_error(Context* c, tmvg_status s, const std::string& msg)
{
    if (c) c->last_error = msg;
    return s;
}

tmvg_status check_cuda(Context* c, cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return TMVG_OK;
    if (e == cudaErrorMemoryAllocation)
        return set_error(c, TMVG_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    return set_error(c, TMVG_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

static void* grow(Context* c, void*& buf, size_t& have, size_t bytes)
{
    if (bytes <= have) return buf;
    if (buf) {
        cudaStreamSynchronize(c->stream);
        cudaFree(buf);
        buf = nullptr;
        have = 0;
    }
    size_t want = bytes + bytes / 4 + 4096;
    if (cudaMalloc(&buf, want) != cudaSuccess) {
        cudaGetLastError();
        buf = nullptr;
        set_error(c, TMVG_OOM, "workspace allocation failed");
        return nullptr;
    }
    have = want;
    return buf;
}

void* workspace(Context* c, size_t bytes) { return grow(c, c->work, c->work_bytes, bytes); }
void* workspace2(Context* c, size_t bytes) { return grow(c, c->work2, c->work2_bytes, bytes); }
void* workspace3(Context* c, size_t bytes) { return grow(c, c->work3, c->work3_bytes, bytes); }
void* perm_lists_buffer(Context* c, size_t bytes) { return grow(c, c->perm_lists, c->perm_lists_bytes, bytes); }
void* trsv_dinv_buffer(Context* c, size_t bytes) { return grow(c, c->trsv_dinv, c->trsv_dinv_bytes, bytes); }

static cudaEvent_t pooled_event(Context* c)
{
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

ScopedTimer::ScopedTimer(Context* c, int cls, double bytes, double flops, cudaStream_t stream)
    : c_(c), cls_(cls), bytes_(bytes), flops_(flops), stream_(stream)
{
    if (!c_->timing) return;
    a_ = pooled_event(c_);
    if (a_ && cudaEventRecord(a_, stream_) != cudaSuccess) {
        cudaGetLastError();
        c_->event_pool.push_back(a_);
        a_ = nullptr;
    }
}

ScopedTimer::~ScopedTimer()
{
    if (!a_) return;
    cudaEvent_t b = pooled_event(c_);
    if (!b || cudaEventRecord(b, stream_) != cudaSuccess) {
        cudaGetLastError();
        c_->event_pool.push_back(a_);
        if (b) c_->event_pool.push_back(b);
        return;
    }
    c_->spans.push_back({a_, b, cls_, bytes_, flops_});
}

tmvg_status ensure_side_stream(Context* c)
{
    if (c->side) return TMVG_OK;
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, greatest) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_wide, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_panel, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, TMVG_CUDA_ERROR, "side stream creation failed");
    }
    return TMVG_OK;
}

// Folds every recorded span into the per-class sums (synchronises).
static tmvg_status drain_spans(Context* c)
{
    tmvg_status st = check_cuda(c, cudaStreamSynchronize(c->stream), "timing: sync");
    if (st) return st;
    if (c->side) {
        st = check_cuda(c, cudaStreamSynchronize(c->side), "timing: sync");
        if (st) return st;
    }
    for (const TimedSpan& s : c->spans) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, s.a, s.b) != cudaSuccess) {
            cudaGetLastError();
        } else {
            c->t_launches[s.cls] += 1;
            c->t_ms[s.cls] += ms;
            c->t_bytes[s.cls] += s.bytes;
            c->t_flops[s.cls] += s.flops;
        }
        c->event_pool.push_back(s.a);
        c->event_pool.push_back(s.b);
    }
    c->spans.clear();
    return TMVG_OK;
}

tmvg_status collect_device_error(Context* c, const char* what)
{
    tmvg_status st = check_cuda(
        c, cudaMemcpyAsync(c->hflags, c->dflags, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream),
        what);
    if (st) return st;
    st = check_cuda(c, cudaStreamSynchronize(c->stream), what);
    if (st) return st;
    const int code = c->hflags[0];
    if (code == kDevOk) return TMVG_OK;
    cudaMemsetAsync(c->dflags, 0, 2 * sizeof(int), c->stream);
    cudaStreamSynchronize(c->stream);
    if (code == kDevSingular)
        return set_error(c, TMVG_SINGULAR, std::string(what) + ": singular triangular factor");
    if (code == kDevTimeout)
        return set_error(c, TMVG_TIMEOUT, std::string(what) + ": a device-side wait timed out");
    return set_error(c, TMVG_CUDA_ERROR, std::string(what) + ": device error word set");
}

// RAII stream-ordered device buffer for the host-pointer entry points.
// Device buffers of the host (_host) entry points: views into one grow-only
// context arena, so repeated calls of the same size allocate nothing.  The
// arena is only used inside one synchronous host call at a time.
struct DevBuf {
    void* p = nullptr;
    template <typename T>
    T* as() { return static_cast<T*>(p); }
};

struct IoBufs {
    DevBuf b[4];
    bool ok = false;
    IoBufs(Context* c, std::initializer_list<size_t> sizes)
    {
        size_t off[4] = {0, 0, 0, 0}, total = 0;
        int q = 0;
        for (size_t sz : sizes) {
            off[q++] = total;
            total += ((sz ? sz : 16) + 255) & ~size_t(255);
        }
        unsigned char* base = static_cast<unsigned char*>(grow(c, c->io, c->io_bytes, total));
        if (!base) return;
        for (int i = 0; i < q; ++i) b[i].p = base + off[i];
        ok = true;
    }
    DevBuf& operator[](int i) { return b[i]; }
};

// 32x32 tiled transpose: out (cols x rows, column-major) = in^T where in is
// rows x cols column-major.
template <typename T>
__global__ void transpose_kernel(int64_t rows, int64_t cols, const T* __restrict__ in,
                                 int64_t ldi, T* __restrict__ out, int64_t ldo)
{
    __shared__ T tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, j = j0 + r;
        if (i < rows && j < cols) tile[r][threadIdx.x] = in[i + j * ldi];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t j = j0 + threadIdx.x, i = i0 + r;
        if (i < rows && j < cols) out[j + i * ldo] = tile[threadIdx.x][r];
    }
}

template <typename T>
static tmvg_status transpose(Context* c, int64_t rows, int64_t cols, const T* in, int64_t ldi,
                             T* out, int64_t ldo)
{
    if (rows <= 0 || cols <= 0) return TMVG_OK;
    dim3 grid((unsigned)ceil_div(rows, 32), (unsigned)ceil_div(cols, 32));
    transpose_kernel<T><<<grid, dim3(32, 8), 0, c->stream>>>(rows, cols, in, ldi, out, ldo);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "transpose launch");
}

// Copy a strided host matrix (rows x cols, element (i,j) at p[i*si + j*sj])
// into a dense column-major device buffer, and back.  Column- and row-major
// host layouts move with one 2-D copy; anything else is packed on the host.
template <typename T>
static tmvg_status h2d_matrix(Context* c, T* dst, const T* src, int64_t rows, int64_t cols,
                              int64_t si, int64_t sj, T* tmp_dev)
{
    if (rows <= 0 || cols <= 0) return TMVG_OK;
    if (si == 1 || cols == 1) {
        const int64_t ld = cols == 1 ? rows : sj;
        return check_cuda(c,
                          cudaMemcpy2DAsync(dst, rows * sizeof(T), src, ld * sizeof(T),
                                            rows * sizeof(T), cols, cudaMemcpyHostToDevice,
                                            c->stream),
                          "h2d");
    }
    if (sj == 1 || rows == 1) {
        const int64_t ld = rows == 1 ? cols : si;
        tmvg_status st = check_cuda(
            c,
            cudaMemcpy2DAsync(tmp_dev, cols * sizeof(T), src, ld * sizeof(T),
                              cols * sizeof(T), rows, cudaMemcpyHostToDevice, c->stream),
            "h2d");
        if (st) return st;
        return transpose<T>(c, cols, rows, tmp_dev, cols, dst, rows);
    }
    return set_error(c, TMVG_BAD_ARG, "host matrix must be column- or row-major");
}

template <typename T>
static tmvg_status d2h_matrix(Context* c, T* dst, const T* src, int64_t rows, int64_t cols,
                              int64_t si, int64_t sj, T* tmp_dev)
{
    if (rows <= 0 || cols <= 0) return TMVG_OK;
    if (si == 1 || cols == 1) {
        const int64_t ld = cols == 1 ? rows : sj;
        return check_cuda(c,
                          cudaMemcpy2DAsync(dst, ld * sizeof(T), src, rows * sizeof(T),
                                            rows * sizeof(T), cols, cudaMemcpyDeviceToHost,
                                            c->stream),
                          "d2h");
    }
    if (sj == 1 || rows == 1) {
        const int64_t ld = rows == 1 ? cols : si;
        tmvg_status st = transpose<T>(c, rows, cols, src, rows, tmp_dev, cols);
        if (st) return st;
        return check_cuda(c,
                          cudaMemcpy2DAsync(dst, ld * sizeof(T), tmp_dev, cols * sizeof(T),
                                            cols * sizeof(T), rows, cudaMemcpyDeviceToHost,
                                            c->stream),
                          "d2h");
    }
    return set_error(c, TMVG_BAD_ARG, "host matrix must be column- or row-major");
}


// ---- host-view entry points for float and complex<double> ---------------
// The same transfers as the double ones: dense column-major device copies in
// the context's arena, the device routine, the results back, synchronous.
template <typename T, typename Factor>
static tmvg_status lu_decompose_host(Context* c, int64_t n, T* A, int64_t sAi, int64_t sAj,
                                     int64_t* P, Factor factor)
{
    if (n < 0) return set_error(c, TMVG_BAD_ARG, "lu: negative n");
    if (n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(T) * n * n, sizeof(T) * n * n, sizeof(int64_t) * n});
    if (!io.ok) return set_error(c, TMVG_OOM, "lu: device buffers");
    DevBuf &dA = io[0], &tmp = io[1], &dP = io[2];
    tmvg_status st = h2d_matrix<T>(c, dA.as<T>(), A, n, n, sAi, sAj, tmp.as<T>());
    if (!st) st = factor(dA.as<T>(), dP.as<int64_t>());
    if (!st) st = d2h_matrix<T>(c, A, dA.as<T>(), n, n, sAi, sAj, tmp.as<T>());
    if (!st)
        st = check_cuda(c, cudaMemcpyAsync(P, dP.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, c->stream),
                        "lu: pivots d2h");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "lu sync");
    return st;
}

// B := B / (P L U) (left) or B (P L U)^-1 (right) on host views; Div(dLU,
// dP, other, dB, ldb) runs the device solve.
template <typename T, typename Div>
static tmvg_status lu_div_host(Context* c, bool right, int64_t n, const T* LU, int64_t lda,
                               const int64_t* P, int64_t other, T* B, int64_t sBi, int64_t sBj, Div div)
{
    if (n < 0 || other < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "div: bad sizes");
    if (n == 0 || other == 0) return TMVG_OK;
    const int64_t rows = right ? other : n, cols = right ? n : other;
    IoBufs io(c, {sizeof(T) * n * n, sizeof(int64_t) * n, sizeof(T) * rows * cols, sizeof(T) * rows * cols});
    if (!io.ok) return set_error(c, TMVG_OOM, "div: device buffers");
    DevBuf &dLU = io[0], &dP = io[1], &dB = io[2], &tmp = io[3];
    tmvg_status st = check_cuda(c,
                                cudaMemcpy2DAsync(dLU.p, n * sizeof(T), LU, lda * sizeof(T), n * sizeof(T), n,
                                                  cudaMemcpyHostToDevice, c->stream),
                                "div: LU h2d");
    if (!st)
        st = check_cuda(c, cudaMemcpyAsync(dP.p, P, sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->stream),
                        "div: P h2d");
    if (!st) st = h2d_matrix<T>(c, dB.as<T>(), B, rows, cols, sBi, sBj, tmp.as<T>());
    if (!st) st = div(dLU.as<T>(), dP.as<int64_t>(), other, dB.as<T>(), rows);
    if (st == TMVG_OK || st == TMVG_SINGULAR) {
        tmvg_status st2 = d2h_matrix<T>(c, B, dB.as<T>(), rows, cols, sBi, sBj, tmp.as<T>());
        if (!st2) st2 = check_cuda(c, cudaStreamSynchronize(c->stream), "div sync");
        if (st2) return st2;
    }
    return st;
}

template <typename T, typename Inv>
static tmvg_status lu_inverse_host(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                                   T* Minv, int64_t msi, int64_t msj, Inv inv)
{
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "inverse: bad sizes");
    if (n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(T) * n * n, sizeof(int64_t) * n, sizeof(T) * n * n, sizeof(T) * n * n});
    if (!io.ok) return set_error(c, TMVG_OOM, "inverse: device buffers");
    DevBuf &dLU = io[0], &dP = io[1], &dM = io[2], &tmp = io[3];
    tmvg_status st = check_cuda(c,
                                cudaMemcpy2DAsync(dLU.p, n * sizeof(T), LU, lda * sizeof(T), n * sizeof(T), n,
                                                  cudaMemcpyHostToDevice, c->stream),
                                "inverse: LU h2d");
    if (!st)
        st = check_cuda(c, cudaMemcpyAsync(dP.p, P, sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->stream),
                        "inverse: P h2d");
    if (!st) st = inv(dLU.as<T>(), dP.as<int64_t>(), dM.as<T>());
    if (!st) st = d2h_matrix<T>(c, Minv, dM.as<T>(), n, n, msi, msj, tmp.as<T>());
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "inverse sync");
    return st;
}

}  // namespace tmvg

using namespace tmvg;

#define CTX_OR_BAIL(h)                                     \
    Context* c = reinterpret_cast<Context*>(h);            \
    if (!c) return TMVG_BAD_ARG;                           \
    c->last_error.clear();                                 \
    if (cudaSetDevice(c->device) != cudaSuccess)           \
        return set_error(c, TMVG_CUDA_ERROR, "cudaSetDevice failed");

extern "C" {

int tmvg_version(void) { return 1; }

const char* tmvg_status_string(tmvg_status s)
{
    switch (s) {
        case TMVG_OK: return "ok";
        case TMVG_SINGULAR: return "singular";
        case TMVG_NOT_CONVERGED: return "not converged";
        case TMVG_BAD_ARG: return "bad argument";
        case TMVG_OOM: return "out of memory";
        case TMVG_TIMEOUT: return "device wait timed out";
        case TMVG_CUDA_ERROR: return "cuda error";
        case TMVG_NO_DEVICE: return "no cuda device";
        case TMVG_UNSUPPORTED: return "unsupported";
    }
    return "unknown";
}

tmvg_status tmvg_create(tmvg_handle* h, int device)
{
    if (!h) return TMVG_BAD_ARG;
    *h = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return TMVG_NO_DEVICE;
    }
    if (device < 0 || device >= count) return TMVG_BAD_ARG;
    Context* c = new (std::nothrow) Context();
    if (!c) return TMVG_OOM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&c->dflags, 64 * sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&c->hflags, 64 * sizeof(int)) != cudaSuccess ||
        cudaMemset(c->dflags, 0, 64 * sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        if (c->dflags) cudaFree(c->dflags);
        if (c->hflags) cudaFreeHost(c->hflags);
        delete c;
        return TMVG_CUDA_ERROR;
    }
    c->dbar = reinterpret_cast<unsigned*>(c->dflags + 16);
    c->trsv_ticket = reinterpret_cast<unsigned long long*>(c->dflags + 32);
    if (cudaMalloc(&c->trsv_flags, sizeof(unsigned) * kTrsvFlagCap) != cudaSuccess ||
        cudaMemset(c->trsv_flags, 0, sizeof(unsigned) * kTrsvFlagCap) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->dflags);
        cudaFreeHost(c->hflags);
        if (c->trsv_flags) cudaFree(c->trsv_flags);
        delete c;
        return TMVG_CUDA_ERROR;
    }
    const char* ser = std::getenv("TMVG_SERIALIZE_LOOKAHEAD");
    c->serialize_lookahead = ser && ser[0] == '1';
    const char* reg2 = std::getenv("TMVG_PANEL_REG2");
    c->panel_reg2 = reg2 && reg2[0] == '1';
    *h = reinterpret_cast<tmvg_handle>(c);
    return TMVG_OK;
}

tmvg_status tmvg_destroy(tmvg_handle h)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->work) cudaFree(c->work);
    if (c->work2) cudaFree(c->work2);
    if (c->work3) cudaFree(c->work3);
    if (c->io) cudaFree(c->io);
    if (c->perm_lists) cudaFree(c->perm_lists);
    if (c->trsv_flags) cudaFree(c->trsv_flags);
    if (c->trsv_pub) cudaFree(c->trsv_pub);
    if (c->trsv_dinv) cudaFree(c->trsv_dinv);
    if (c->dflags) cudaFree(c->dflags);
    if (c->hflags) cudaFreeHost(c->hflags);
    for (const TimedSpan& sp : c->spans) {
        cudaEventDestroy(sp.a);
        cudaEventDestroy(sp.b);
    }
    for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_wide) cudaEventDestroy(c->ev_wide);
    if (c->ev_panel) cudaEventDestroy(c->ev_panel);
    if (c->side) cudaStreamDestroy(c->side);
    delete c;
    return TMVG_OK;
}

tmvg_status tmvg_timing_enable(tmvg_handle h, int on)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c) return TMVG_BAD_ARG;
    cudaSetDevice(c->device);
    tmvg_status st = drain_spans(c);
    if (st) return st;
    c->timing = on != 0;
    for (int k = 0; k < kClsCount; ++k) {
        c->t_launches[k] = 0;
        c->t_ms[k] = c->t_bytes[k] = c->t_flops[k] = 0.0;
    }
    return TMVG_OK;
}

tmvg_status tmvg_timing_read(tmvg_handle h, int kclass, tmvg_kernel_timing* out)
{
    Context* c = reinterpret_cast<Context*>(h);
    if (!c || !out) return TMVG_BAD_ARG;
    if (kclass < 0 || kclass >= kClsCount) return set_error(c, TMVG_BAD_ARG, "timing: unknown kernel class");
    cudaSetDevice(c->device);
    tmvg_status st = drain_spans(c);
    if (st) return st;
    out->spans = c->t_launches[kclass];
    out->total_ms = c->t_ms[kclass];
    out->bytes = c->t_bytes[kclass];
    out->flops = c->t_flops[kclass];
    return TMVG_OK;
}

tmvg_status tmvg_set_stream(tmvg_handle h, void* stream)
{
    CTX_OR_BAIL(h);
    c->stream = reinterpret_cast<cudaStream_t>(stream);
    return TMVG_OK;
}

tmvg_status tmvg_synchronize(tmvg_handle h)
{
    CTX_OR_BAIL(h);
    return check_cuda(c, cudaStreamSynchronize(c->stream), "synchronize");
}

const char* tmvg_last_error(tmvg_handle h)
{
    Context* c = reinterpret_cast<Context*>(h);
    return c ? c->last_error.c_str() : "";
}

int64_t tmvg_launch_count(tmvg_handle h)
{
    Context* c = reinterpret_cast<Context*>(h);
    return c ? c->launches : 0;
}

tmvg_status tmvg_test_set_wait(tmvg_handle h, uint32_t poll_limit, int32_t skip_blocks)
{
    CTX_OR_BAIL(h);
    if (skip_blocks < 0) return set_error(c, TMVG_BAD_ARG, "test_set_wait: negative skip");
    c->poll_limit = poll_limit;
    c->test_skip_blocks = skip_blocks;
    return TMVG_OK;
}

tmvg_status tmvg_probe_fp64_rate(tmvg_handle h, double* tflops)
{
    CTX_OR_BAIL(h);
    if (!tflops) return set_error(c, TMVG_BAD_ARG, "probe: null output");
    return probe_fp64_rate(c, tflops);
}

tmvg_status tmvg_multmm_f64(tmvg_handle h, int add, double alpha, int64_t m, int64_t n, int64_t k,
                            const double* A, int64_t sAi, int64_t sAj, const double* B,
                            int64_t sBi, int64_t sBj, double* C, int64_t sCi, int64_t sCj)
{
    CTX_OR_BAIL(h);
    return gemm<double>(c, m, n, k, alpha, Mat<const double>{A, sAi, sAj},
                        Mat<const double>{B, sBi, sBj}, add ? 1.0 : 0.0, Mat<double>{C, sCi, sCj});
}

tmvg_status tmvg_multmm_f64_host(tmvg_handle h, int add, double alpha, int64_t m, int64_t n,
                                 int64_t k, const double* A, int64_t sAi, int64_t sAj,
                                 const double* B, int64_t sBi, int64_t sBj, double* C,
                                 int64_t sCi, int64_t sCj)
{
    CTX_OR_BAIL(h);
    if (m < 0 || n < 0 || k < 0) return set_error(c, TMVG_BAD_ARG, "multmm: negative size");
    if (m == 0 || n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(double) * m * k, sizeof(double) * k * n, sizeof(double) * m * n,
                  sizeof(double) * std::max(std::max(m * k, k * n), m * n)});
    if (!io.ok) return set_error(c, TMVG_OOM, "multmm: device buffers");
    DevBuf &dA = io[0], &dB = io[1], &dC = io[2], &tmp = io[3];
    tmvg_status st = h2d_matrix(c, dA.as<double>(), A, m, k, sAi, sAj, tmp.as<double>());
    if (!st) st = h2d_matrix(c, dB.as<double>(), B, k, n, sBi, sBj, tmp.as<double>());
    if (!st && add) st = h2d_matrix(c, dC.as<double>(), C, m, n, sCi, sCj, tmp.as<double>());
    if (!st)
        st = gemm<double>(c, m, n, k, alpha, Mat<const double>{dA.as<double>(), 1, m},
                          Mat<const double>{dB.as<double>(), 1, k}, add ? 1.0 : 0.0,
                          Mat<double>{dC.as<double>(), 1, m});
    if (!st) st = d2h_matrix(c, C, dC.as<double>(), m, n, sCi, sCj, tmp.as<double>());
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "multmm sync");
    return st;
}

tmvg_status tmvg_lu_decompose_f64(tmvg_handle h, int64_t n, double* A, int64_t lda, int64_t* P)
{
    CTX_OR_BAIL(h);
    return lu_factor<double>(c, n, A, lda, P);
}

tmvg_status tmvg_lu_decompose_f64_host(tmvg_handle h, int64_t n, double* A, int64_t sAi,
                                       int64_t sAj, int64_t* P)
{
    CTX_OR_BAIL(h);
    if (n < 0) return set_error(c, TMVG_BAD_ARG, "lu: negative n");
    if (n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(double) * n * n, sizeof(double) * n * n, sizeof(int64_t) * n});
    if (!io.ok) return set_error(c, TMVG_OOM, "lu: device buffers");
    DevBuf &dA = io[0], &tmp = io[1], &dP = io[2];
    tmvg_status st = h2d_matrix(c, dA.as<double>(), A, n, n, sAi, sAj, tmp.as<double>());
    if (!st) st = lu_factor<double>(c, n, dA.as<double>(), n, dP.as<int64_t>());
    if (!st) st = d2h_matrix(c, A, dA.as<double>(), n, n, sAi, sAj, tmp.as<double>());
    if (!st)
        st = check_cuda(c,
                        cudaMemcpyAsync(P, dP.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost,
                                        c->stream),
                        "lu: pivots d2h");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "lu sync");
    return st;
}

tmvg_status tmvg_lu_ldiveq_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                               const int64_t* P, int64_t nrhs, double* B, int64_t ldb)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "ldiveq: bad sizes");
    return lu_ldiveq<double>(c, n, LU, lda, P, nrhs, B, 1, ldb);
}

tmvg_status tmvg_lu_rdiveq_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                               const int64_t* P, int64_t nrows, double* B, int64_t ldb)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrows < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(nrows, 1))
        return set_error(c, TMVG_BAD_ARG, "rdiveq: bad sizes");
    return lu_rdiveq<double>(c, n, LU, lda, P, nrows, B, 1, ldb);
}

static tmvg_status div_host(Context* c, bool right, int64_t n, const double* LU, int64_t lda,
                            const int64_t* P, int64_t other, double* B, int64_t sBi, int64_t sBj)
{
    if (n < 0 || other < 0 || lda < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "div: bad sizes");
    if (n == 0 || other == 0) return TMVG_OK;
    const int64_t rows = right ? other : n, cols = right ? n : other;
    IoBufs io(c, {sizeof(double) * n * n, sizeof(int64_t) * n, sizeof(double) * rows * cols,
                  sizeof(double) * rows * cols});
    if (!io.ok) return set_error(c, TMVG_OOM, "div: device buffers");
    DevBuf &dLU = io[0], &dP = io[1], &dB = io[2], &tmp = io[3];
    tmvg_status st = check_cuda(
        c,
        cudaMemcpy2DAsync(dLU.p, n * sizeof(double), LU, lda * sizeof(double), n * sizeof(double),
                          n, cudaMemcpyHostToDevice, c->stream),
        "div: LU h2d");
    if (!st)
        st = check_cuda(c,
                        cudaMemcpyAsync(dP.p, P, sizeof(int64_t) * n, cudaMemcpyHostToDevice,
                                        c->stream),
                        "div: P h2d");
    if (!st) st = h2d_matrix(c, dB.as<double>(), B, rows, cols, sBi, sBj, tmp.as<double>());
    if (!st)
        st = right ? lu_rdiveq<double>(c, n, dLU.as<double>(), n, dP.as<int64_t>(), other,
                                       dB.as<double>(), 1, rows)
                   : lu_ldiveq<double>(c, n, dLU.as<double>(), n, dP.as<int64_t>(), other,
                                       dB.as<double>(), 1, rows);
    if (st == TMVG_OK || st == TMVG_SINGULAR) {
        tmvg_status st2 = d2h_matrix(c, B, dB.as<double>(), rows, cols, sBi, sBj, tmp.as<double>());
        if (!st2) st2 = check_cuda(c, cudaStreamSynchronize(c->stream), "div sync");
        if (st2) return st2;
    }
    return st;
}

tmvg_status tmvg_lu_ldiveq_f64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                    const int64_t* P, int64_t nrhs, double* B, int64_t sBi,
                                    int64_t sBj)
{
    CTX_OR_BAIL(h);
    return div_host(c, false, n, LU, lda, P, nrhs, B, sBi, sBj);
}

tmvg_status tmvg_lu_rdiveq_f64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                    const int64_t* P, int64_t nrows, double* B, int64_t sBi,
                                    int64_t sBj)
{
    CTX_OR_BAIL(h);
    return div_host(c, true, n, LU, lda, P, nrows, B, sBi, sBj);
}

tmvg_status tmvg_divide_f64(tmvg_handle h, int64_t n, const double* A, int64_t lda, int64_t nrhs,
                            const double* B, int64_t ldb, double* X, int64_t ldx, double* LU,
                            int64_t* P)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || ldb < std::max<int64_t>(n, 1) ||
        ldx < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "divide: bad sizes");
    if (n == 0) return TMVG_OK;
    tmvg_status st = check_cuda(
        c,
        cudaMemcpy2DAsync(LU, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                          cudaMemcpyDeviceToDevice, c->stream),
        "divide: copy A");
    if (st) return st;
    st = lu_factor<double>(c, n, LU, n, P);
    if (st) return st;
    if (nrhs == 0) return TMVG_OK;
    st = check_cuda(c,
                    cudaMemcpy2DAsync(X, ldx * sizeof(double), B, ldb * sizeof(double),
                                      n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, c->stream),
                    "divide: copy B");
    if (st) return st;
    return lu_ldiveq<double>(c, n, LU, n, P, nrhs, X, 1, ldx);
}

tmvg_status tmvg_divide_f64_host(tmvg_handle h, int64_t n, const double* A, int64_t nrhs,
                                 const double* B, double* X, double* LU, int64_t* P)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrhs < 0) return set_error(c, TMVG_BAD_ARG, "divide: bad sizes");
    if (n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(double) * n * n, sizeof(int64_t) * n,
                  sizeof(double) * n * std::max<int64_t>(nrhs, 1)});
    if (!io.ok) return set_error(c, TMVG_OOM, "divide: device buffers");
    DevBuf &dA = io[0], &dP = io[1], &dX = io[2];
    tmvg_status st = check_cuda(
        c, cudaMemcpyAsync(dA.p, A, sizeof(double) * n * n, cudaMemcpyHostToDevice, c->stream),
        "divide: A h2d");
    if (!st && nrhs > 0)
        st = check_cuda(c,
                        cudaMemcpyAsync(dX.p, B, sizeof(double) * n * nrhs, cudaMemcpyHostToDevice,
                                        c->stream),
                        "divide: B h2d");
    if (!st) st = lu_factor<double>(c, n, dA.as<double>(), n, dP.as<int64_t>());
    if (!st && nrhs > 0)
        st = lu_ldiveq<double>(c, n, dA.as<double>(), n, dP.as<int64_t>(), nrhs, dX.as<double>(),
                               1, n);
    if (st == TMVG_OK || st == TMVG_SINGULAR) {
        tmvg_status st2 = TMVG_OK;
        if (X && nrhs > 0)
            st2 = check_cuda(c,
                             cudaMemcpyAsync(X, dX.p, sizeof(double) * n * nrhs,
                                             cudaMemcpyDeviceToHost, c->stream),
                             "divide: X d2h");
        if (!st2 && LU)
            st2 = check_cuda(c,
                             cudaMemcpyAsync(LU, dA.p, sizeof(double) * n * n,
                                             cudaMemcpyDeviceToHost, c->stream),
                             "divide: LU d2h");
        if (!st2 && P)
            st2 = check_cuda(c,
                             cudaMemcpyAsync(P, dP.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost,
                                             c->stream),
                             "divide: P d2h");
        if (!st2) st2 = check_cuda(c, cudaStreamSynchronize(c->stream), "divide sync");
        if (st2) return st2;
    }
    return st;
}

tmvg_status tmvg_lu_det_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                            const int64_t* P, double* det, double* logdet, double* sign)
{
    // LUDiv::det / logDet (src/TMV_LUD.cpp:132-156) over GenDiagMatrix::logDet
    // (src/TMV_DiagMatrix.cpp:59-85): log|U_jj| summed, a zero U_jj gives
    // sign 0; det = sign * exp(logdet).  O(n) work: the diagonal and P are
    // read back and reduced on the host in TMV's order.
    CTX_OR_BAIL(h);
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "det: bad sizes");
    double* diag = nullptr;
    int64_t* hp = nullptr;
    if (cudaMallocHost(&diag, sizeof(double) * std::max<int64_t>(n, 1)) != cudaSuccess ||
        cudaMallocHost(&hp, sizeof(int64_t) * std::max<int64_t>(n, 1)) != cudaSuccess) {
        cudaGetLastError();
        if (diag) cudaFreeHost(diag);
        return set_error(c, TMVG_OOM, "det: host buffers");
    }
    tmvg_status st = TMVG_OK;
    if (n > 0) {
        st = check_cuda(c,
                        cudaMemcpy2DAsync(diag, sizeof(double), LU, (lda + 1) * sizeof(double),
                                          sizeof(double), n, cudaMemcpyDeviceToHost, c->stream),
                        "det: diag d2h");
        if (!st)
            st = check_cuda(c,
                            cudaMemcpyAsync(hp, P, sizeof(int64_t) * n, cudaMemcpyDeviceToHost,
                                            c->stream),
                            "det: P d2h");
        if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "det sync");
    }
    if (!st) {
        double ld = 0.0, s = 1.0;
        int pd = 1;
        for (int64_t j = 0; j < n; ++j) {
            const double u = diag[j];
            if (u == 0.0) {
                ld = std::log(0.0);
                s = 0.0;
            } else {
                ld += std::log(std::fabs(u));
                s *= u > 0 ? 1.0 : -1.0;
            }
            if (hp[j] != j) pd = -pd;
        }
        s *= (double)pd;
        if (logdet) *logdet = ld;
        if (sign) *sign = s;
        if (det) *det = s == 0.0 ? 0.0 : s * std::exp(ld);
    }
    cudaFreeHost(diag);
    cudaFreeHost(hp);
    return st;
}

tmvg_status tmvg_lu_inverse_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                const int64_t* P, double* Minv, int64_t ldm)
{
    CTX_OR_BAIL(h);
    if (n < 0 || lda < std::max<int64_t>(n, 1) || ldm < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "inverse: bad sizes");
    return lu_inverse<double>(c, n, LU, lda, P, Minv, ldm);
}

tmvg_status tmvg_lu_inverse_f64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                     const int64_t* P, double* Minv, int64_t msi, int64_t msj)
{
    // LUDiv::doMakeInverse -> LU_Inverse on host views (src/TMV_LUD.cpp:158-170)
    CTX_OR_BAIL(h);
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "inverse: bad sizes");
    if (n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(double) * n * n, sizeof(int64_t) * n, sizeof(double) * n * n,
                  sizeof(double) * n * n});
    if (!io.ok) return set_error(c, TMVG_OOM, "inverse: device buffers");
    DevBuf &dLU = io[0], &dP = io[1], &dM = io[2], &tmp = io[3];
    tmvg_status st = check_cuda(
        c,
        cudaMemcpy2DAsync(dLU.p, n * sizeof(double), LU, lda * sizeof(double), n * sizeof(double), n,
                          cudaMemcpyHostToDevice, c->stream),
        "inverse: LU h2d");
    if (!st)
        st = check_cuda(c, cudaMemcpyAsync(dP.p, P, sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->stream),
                        "inverse: P h2d");
    if (!st) st = lu_inverse<double>(c, n, dLU.as<double>(), n, dP.as<int64_t>(), dM.as<double>(), n);
    if (!st) st = d2h_matrix(c, Minv, dM.as<double>(), n, n, msi, msj, tmp.as<double>());
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "inverse sync");
    return st;
}

tmvg_status tmvg_lu_inverse_ata_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                    double* ATA, int64_t ldata)
{
    CTX_OR_BAIL(h);
    if (n < 0 || lda < std::max<int64_t>(n, 1) || ldata < std::max<int64_t>(n, 1))
        return set_error(c, TMVG_BAD_ARG, "inverse_ata: bad sizes");
    return lu_inverse_ata<double>(c, n, LU, lda, ATA, ldata);
}

tmvg_status tmvg_lu_is_singular_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                    int* singular)
{
    // LUDiv::isSingular (src/TMV_LUD.cpp:204-209): min |U_jj| <= epsilon *
    // max |U_jj| (Abs2 of a real is |x|), scanned in order with strict
    // comparisons as FindMin/MaxAbs2Element do (src/TMV_Vector.cpp:539-600),
    // so a NaN never replaces the running extreme.  O(n): the diagonal is
    // read back and reduced on the host.
    CTX_OR_BAIL(h);
    if (n < 0 || lda < std::max<int64_t>(n, 1) || !singular)
        return set_error(c, TMVG_BAD_ARG, "is_singular: bad arguments");
    *singular = 0;
    if (n == 0) return TMVG_OK;
    double* diag = nullptr;
    if (cudaMallocHost(&diag, sizeof(double) * n) != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, TMVG_OOM, "is_singular: host buffer");
    }
    tmvg_status st = check_cuda(c,
                                cudaMemcpy2DAsync(diag, sizeof(double), LU, (lda + 1) * sizeof(double),
                                                  sizeof(double), n, cudaMemcpyDeviceToHost, c->stream),
                                "is_singular: diag d2h");
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "is_singular sync");
    if (!st) {
        double mn = std::fabs(diag[0]), mx = mn;
        for (int64_t j = 1; j < n; ++j) {
            const double a = std::fabs(diag[j]);
            if (a > mx) mx = a;
            if (a < mn) mn = a;
        }
        *singular = mn <= std::numeric_limits<double>::epsilon() * mx ? 1 : 0;
    }
    cudaFreeHost(diag);
    return st;
}

tmvg_status tmvg_tri_ldiveq_f64(tmvg_handle h, int upper, int unitdiag, int64_t n, const double* T,
                                int64_t tsi, int64_t tsj, int64_t nrhs, double* B, int64_t bsi,
                                int64_t bsj)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrhs < 0) return set_error(c, TMVG_BAD_ARG, "tri_ldiveq: bad sizes");
    return tri_ldiveq<double>(c, n, T, tsi, tsj, upper != 0, unitdiag != 0, nrhs, B, bsi, bsj);
}

tmvg_status tmvg_tri_rdiveq_f64(tmvg_handle h, int upper, int unitdiag, int64_t n, const double* T,
                                int64_t tsi, int64_t tsj, int64_t nrows, double* B, int64_t bsi,
                                int64_t bsj)
{
    // m %= T is T^T.LDivEq(m^T) (include/tmv/TMV_TriMatrix.h:945-946): the
    // transposed triangle (upper <-> lower, strides swapped) divides m^T.
    CTX_OR_BAIL(h);
    if (n < 0 || nrows < 0) return set_error(c, TMVG_BAD_ARG, "tri_rdiveq: bad sizes");
    return tri_ldiveq<double>(c, n, T, tsj, tsi, upper == 0, unitdiag != 0, nrows, B, bsj, bsi);
}

tmvg_status tmvg_multmv_f64(tmvg_handle h, int add, double alpha, int64_t m, int64_t n, const double* A,
                            int64_t sAi, int64_t sAj, const double* x, int64_t incx, double* y,
                            int64_t incy)
{
    CTX_OR_BAIL(h);
    if (m < 0 || n < 0) return set_error(c, TMVG_BAD_ARG, "multmv: bad sizes");
    return multmv(c, add != 0, alpha, m, n, A, sAi, sAj, x, incx, y, incy);
}

tmvg_status tmvg_lu_decompose_z64(tmvg_handle h, int64_t n, double* A, int64_t lda, int64_t* P)
{
    CTX_OR_BAIL(h);
    return zlu_factor(c, n, reinterpret_cast<double2*>(A), lda, P);
}

tmvg_status tmvg_lu_ldiveq_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                               int64_t nrhs, double* B, int64_t ldb)
{
    CTX_OR_BAIL(h);
    return zlu_ldiveq(c, n, reinterpret_cast<const double2*>(LU), lda, P, nrhs,
                      reinterpret_cast<double2*>(B), ldb);
}

tmvg_status tmvg_lu_rdiveq_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                               int64_t nrows, double* B, int64_t ldb)
{
    CTX_OR_BAIL(h);
    return zlu_rdiveq(c, n, reinterpret_cast<const double2*>(LU), lda, P, nrows,
                      reinterpret_cast<double2*>(B), ldb);
}

tmvg_status tmvg_lu_inverse_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                                double* Minv, int64_t ldm)
{
    CTX_OR_BAIL(h);
    return zlu_inverse(c, n, reinterpret_cast<const double2*>(LU), lda, P, reinterpret_cast<double2*>(Minv), ldm);
}


tmvg_status tmvg_multmm_f32_host(tmvg_handle h, int add, float alpha, int64_t m, int64_t n, int64_t k,
                                 const float* A, int64_t sAi, int64_t sAj, const float* B, int64_t sBi,
                                 int64_t sBj, float* C, int64_t sCi, int64_t sCj)
{
    CTX_OR_BAIL(h);
    if (m < 0 || n < 0 || k < 0) return set_error(c, TMVG_BAD_ARG, "multmm: negative size");
    if (m == 0 || n == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(float) * m * k, sizeof(float) * k * n, sizeof(float) * m * n,
                  sizeof(float) * std::max(std::max(m * k, k * n), m * n)});
    if (!io.ok) return set_error(c, TMVG_OOM, "multmm: device buffers");
    DevBuf &dA = io[0], &dB = io[1], &dC = io[2], &tmp = io[3];
    tmvg_status st = h2d_matrix<float>(c, dA.as<float>(), A, m, k, sAi, sAj, tmp.as<float>());
    if (!st) st = h2d_matrix<float>(c, dB.as<float>(), B, k, n, sBi, sBj, tmp.as<float>());
    if (!st && add) st = h2d_matrix<float>(c, dC.as<float>(), C, m, n, sCi, sCj, tmp.as<float>());
    if (!st)
        st = gemm<float>(c, m, n, k, alpha, Mat<const float>{dA.as<float>(), 1, m},
                         Mat<const float>{dB.as<float>(), 1, k}, add ? 1.0f : 0.0f, Mat<float>{dC.as<float>(), 1, m});
    if (!st) st = d2h_matrix<float>(c, C, dC.as<float>(), m, n, sCi, sCj, tmp.as<float>());
    if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "multmm sync");
    return st;
}

tmvg_status tmvg_lu_decompose_f32_host(tmvg_handle h, int64_t n, float* A, int64_t sAi, int64_t sAj,
                                       int64_t* P)
{
    CTX_OR_BAIL(h);
    return lu_decompose_host<float>(c, n, A, sAi, sAj, P,
                                    [&](float* dA, int64_t* dP) { return lu_factor<float>(c, n, dA, n, dP); });
}

tmvg_status tmvg_lu_ldiveq_f32_host(tmvg_handle h, int64_t n, const float* LU, int64_t lda, const int64_t* P,
                                    int64_t nrhs, float* B, int64_t sBi, int64_t sBj)
{
    CTX_OR_BAIL(h);
    return lu_div_host<float>(c, false, n, LU, lda, P, nrhs, B, sBi, sBj,
                              [&](const float* dLU, const int64_t* dP, int64_t o, float* dB, int64_t ldb) {
                                  return lu_ldiveq<float>(c, n, dLU, n, dP, o, dB, 1, ldb);
                              });
}

tmvg_status tmvg_lu_rdiveq_f32_host(tmvg_handle h, int64_t n, const float* LU, int64_t lda, const int64_t* P,
                                    int64_t nrows, float* B, int64_t sBi, int64_t sBj)
{
    CTX_OR_BAIL(h);
    return lu_div_host<float>(c, true, n, LU, lda, P, nrows, B, sBi, sBj,
                              [&](const float* dLU, const int64_t* dP, int64_t o, float* dB, int64_t ldb) {
                                  return lu_rdiveq<float>(c, n, dLU, n, dP, o, dB, 1, ldb);
                              });
}

tmvg_status tmvg_lu_inverse_f32_host(tmvg_handle h, int64_t n, const float* LU, int64_t lda, const int64_t* P,
                                     float* Minv, int64_t msi, int64_t msj)
{
    CTX_OR_BAIL(h);
    return lu_inverse_host<float>(c, n, LU, lda, P, Minv, msi, msj,
                                  [&](const float* dLU, const int64_t* dP, float* dM) {
                                      return lu_inverse<float>(c, n, dLU, n, dP, dM, n);
                                  });
}

tmvg_status tmvg_lu_decompose_z64_host(tmvg_handle h, int64_t n, double* A, int64_t sAi, int64_t sAj,
                                       int64_t* P)
{
    CTX_OR_BAIL(h);
    return lu_decompose_host<double2>(c, n, reinterpret_cast<double2*>(A), sAi, sAj, P,
                                      [&](double2* dA, int64_t* dP) { return zlu_factor(c, n, dA, n, dP); });
}

tmvg_status tmvg_lu_ldiveq_z64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                                    int64_t nrhs, double* B, int64_t sBi, int64_t sBj)
{
    CTX_OR_BAIL(h);
    return lu_div_host<double2>(c, false, n, reinterpret_cast<const double2*>(LU), lda, P, nrhs,
                                reinterpret_cast<double2*>(B), sBi, sBj,
                                [&](const double2* dLU, const int64_t* dP, int64_t o, double2* dB, int64_t ldb) {
                                    return zlu_ldiveq(c, n, dLU, n, dP, o, dB, ldb);
                                });
}

tmvg_status tmvg_lu_rdiveq_z64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                                    int64_t nrows, double* B, int64_t sBi, int64_t sBj)
{
    CTX_OR_BAIL(h);
    return lu_div_host<double2>(c, true, n, reinterpret_cast<const double2*>(LU), lda, P, nrows,
                                reinterpret_cast<double2*>(B), sBi, sBj,
                                [&](const double2* dLU, const int64_t* dP, int64_t o, double2* dB, int64_t ldb) {
                                    return zlu_rdiveq(c, n, dLU, n, dP, o, dB, ldb);
                                });
}

tmvg_status tmvg_lu_inverse_z64_host(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                                     double* Minv, int64_t msi, int64_t msj)
{
    CTX_OR_BAIL(h);
    return lu_inverse_host<double2>(c, n, reinterpret_cast<const double2*>(LU), lda, P,
                                    reinterpret_cast<double2*>(Minv), msi, msj,
                                    [&](const double2* dLU, const int64_t* dP, double2* dM) {
                                        return zlu_inverse(c, n, dLU, n, dP, dM, n);
                                    });
}

tmvg_status tmvg_lu_det_z64(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                            double* det, double* logdet, double* sign)
{
    // LUDiv::det / logDet (src/TMV_LUD.cpp:132-156) with GenDiagMatrix::logDet
    // (src/TMV_DiagMatrix.cpp:59-85) for std::complex<double>: log TMV_ABS(U_jj)
    // summed, the sign multiplied by TMV_SIGN(U_jj, |U_jj|) = U_jj / |U_jj|
    // componentwise (include/tmv/TMV_Base.h:708-716), a zero U_jj gives
    // log(0) and sign 0, the permutation's determinant multiplies the sign.
    // O(n): the diagonal and P are read back and reduced on the host in
    // TMV's order, as for the real determinant.
    CTX_OR_BAIL(h);
    if (n < 0 || lda < std::max<int64_t>(n, 1) || !det || !logdet || !sign)
        return set_error(c, TMVG_BAD_ARG, "det_z: bad arguments");
    std::vector<double> diag(2 * (size_t)std::max<int64_t>(n, 1));
    std::vector<int64_t> hp((size_t)std::max<int64_t>(n, 1));
    tmvg_status st = TMVG_OK;
    if (n > 0) {
        st = check_cuda(c,
                        cudaMemcpy2DAsync(diag.data(), 2 * sizeof(double), LU, 2 * (lda + 1) * sizeof(double),
                                          2 * sizeof(double), n, cudaMemcpyDeviceToHost, c->stream),
                        "det_z: diag d2h");
        if (!st)
            st = check_cuda(c, cudaMemcpyAsync(hp.data(), P, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, c->stream),
                            "det_z: P d2h");
        if (!st) st = check_cuda(c, cudaStreamSynchronize(c->stream), "det_z sync");
    }
    if (st) return st;
    std::complex<double> s(1.0, 0.0);
    double ld = 0.0;
    int pd = 1;
    for (int64_t j = 0; j < n; ++j) {
        const std::complex<double> u(diag[2 * j], diag[2 * j + 1]);
        if (u == std::complex<double>(0.0, 0.0)) {
            ld = std::log(u.real());
            s = 0.0;
        } else {
            // TMV_ABS: the modulus scaled by the larger component
            double xr = u.real(), xi = u.imag();
            const double ar = std::fabs(xr), ai = std::fabs(xi);
            const double sc = ar < ai ? ai : ar;
            xr /= sc;
            xi /= sc;
            const double a = sc * std::sqrt(xr * xr + xi * xi);
            ld += std::log(a);
            const std::complex<double> sg = a > 0 ? std::complex<double>(u.real() / a, u.imag() / a)
                                                  : std::complex<double>(1.0, 0.0);
            s *= sg;
        }
        if (hp[j] != j) pd = -pd;
    }
    s = (double)pd * s;
    *logdet = ld;
    sign[0] = s.real();
    sign[1] = s.imag();
    const std::complex<double> d = s == std::complex<double>(0.0, 0.0) ? std::complex<double>(0.0, 0.0)
                                                                       : s * std::exp(ld);
    det[0] = d.real();
    det[1] = d.imag();
    return TMVG_OK;
}

tmvg_status tmvg_lu_solve_mixed_f64(tmvg_handle h, int64_t n, const double* A, int64_t lda,
                                    int64_t nrhs, const double* B, int64_t ldb, double* X,
                                    int64_t ldx, int max_iter, double tol, tmvg_ir_info* info)
{
    CTX_OR_BAIL(h);
    return lu_solve_mixed(c, n, A, lda, nrhs, B, ldb, X, ldx, max_iter, tol, info);
}

tmvg_status tmvg_lu_solve_mixed_f64_host(tmvg_handle h, int64_t n, const double* A, int64_t nrhs,
                                         const double* B, double* X, int max_iter, double tol,
                                         tmvg_ir_info* info)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrhs < 0) return set_error(c, TMVG_BAD_ARG, "lu_solve_mixed: bad sizes");
    if (n == 0 || nrhs == 0) return TMVG_OK;
    IoBufs io(c, {sizeof(double) * n * n, sizeof(double) * n * nrhs, sizeof(double) * n * nrhs});
    if (!io.ok) return set_error(c, TMVG_OOM, "lu_solve_mixed: device buffers");
    DevBuf &dA = io[0], &dB = io[1], &dX = io[2];
    tmvg_status st = check_cuda(
        c, cudaMemcpyAsync(dA.p, A, sizeof(double) * n * n, cudaMemcpyHostToDevice, c->stream),
        "mixed: A h2d");
    if (!st)
        st = check_cuda(c,
                        cudaMemcpyAsync(dB.p, B, sizeof(double) * n * nrhs, cudaMemcpyHostToDevice,
                                        c->stream),
                        "mixed: B h2d");
    if (!st)
        st = lu_solve_mixed(c, n, dA.as<double>(), n, nrhs, dB.as<double>(), n, dX.as<double>(), n,
                            max_iter, tol, info);
    if (st == TMVG_OK || st == TMVG_NOT_CONVERGED) {
        tmvg_status st2 = check_cuda(c,
                                     cudaMemcpyAsync(X, dX.p, sizeof(double) * n * nrhs,
                                                     cudaMemcpyDeviceToHost, c->stream),
                                     "mixed: X d2h");
        if (!st2) st2 = check_cuda(c, cudaStreamSynchronize(c->stream), "mixed sync");
        if (st2) return st2;
    }
    return st;
}

tmvg_status tmvg_lu_solve_fwd_f64(tmvg_handle h, int64_t n, const double* A, int64_t lda,
                                  int64_t nrhs, const double* B, int64_t ldb, double* X,
                                  int64_t ldx, double* LU, int64_t* P)
{
    return tmvg_divide_f64(h, n, A, lda, nrhs, B, ldb, X, ldx, LU, P);
}

tmvg_status tmvg_lu_solve_bwd_f64(tmvg_handle h, int64_t n, const double* LU, int64_t lda,
                                  const int64_t* P, int64_t nrhs, const double* X, int64_t ldx,
                                  const double* G, int64_t ldg, double* gB, int64_t ldgb,
                                  double* gA, int64_t ldga)
{
    CTX_OR_BAIL(h);
    if (n < 0 || nrhs < 0 || lda < std::max<int64_t>(n, 1) || ldx < std::max<int64_t>(n, 1) ||
        ldg < std::max<int64_t>(n, 1) || (gB && ldgb < std::max<int64_t>(n, 1)) ||
        (gA && ldga < std::max<int64_t>(n, 1)))
        return set_error(c, TMVG_BAD_ARG, "lu_solve_bwd: bad sizes");
    if (n == 0 || (!gB && !gA)) return TMVG_OK;
    double* gb = gB;
    int64_t ldb2 = ldgb;
    if (!gb) {
        gb = (double*)workspace2(c, sizeof(double) * (size_t)n * std::max<int64_t>(nrhs, 1));
        if (!gb) return TMVG_OOM;
        ldb2 = n;
    }
    if (nrhs > 0) {
        // gB = A^-T G: copy G, then gB^T := gB^T (P L U)^-1 (LU_RDivEq on the
        // nrhs x n view gB^T, element (i, j) at gb[i*ldb2 + j])
        tmvg_status st = check_cuda(
            c,
            cudaMemcpy2DAsync(gb, ldb2 * sizeof(double), G, ldg * sizeof(double),
                              n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, c->stream),
            "bwd: copy G");
        if (st) return st;
        st = lu_rdiveq<double>(c, n, LU, lda, P, nrhs, gb, ldb2, 1);
        if (st) return st;
    }
    if (gA) {
        // gA = -gB X^T: (n x nrhs) * (nrhs x n), X^T(i, j) = X[j + i*ldx]
        tmvg_status st = gemm<double>(c, n, n, nrhs, -1.0, Mat<const double>{gb, 1, ldb2},
                                      Mat<const double>{X, ldx, 1}, 0.0, Mat<double>{gA, 1, ldga});
        if (st) return st;
    }
    return check_cuda(c, cudaStreamSynchronize(c->stream), "bwd sync");
}

tmvg_status tmvg_gemm_f32_tf32x3(tmvg_handle h, int64_t m, int64_t n, int64_t k, const float* A,
                                 int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc)
{
    CTX_OR_BAIL(h);
    if (m < 0 || n < 0 || k < 0 || lda < std::max<int64_t>(m, 1) || ldb < std::max<int64_t>(k, 1) ||
        ldc < std::max<int64_t>(m, 1))
        return set_error(c, TMVG_BAD_ARG, "gemm_f32_tf32x3: bad sizes");
    tmvg_status st = gemm_f32_tf32x3_update(c, m, n, k, A, lda, B, ldb, C, ldc);
    if (st) return st;
    return collect_device_error(c, "gemm_f32_tf32x3");
}

}  // extern "C"
