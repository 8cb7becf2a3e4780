// common.cuh -- shared device/host helpers of the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "tmvg.h"

namespace tmvg {

// Number of SMs of the device a context runs on is read at creation; these
// constants only size launch shapes.
constexpr int kWarp = 32;

// Bounded spin: a device-side wait that exceeds this many polls records an
// error code and returns instead of hanging the GPU.  At roughly 100-200 ns a
// poll (with __nanosleep backoff) this is a few seconds.
constexpr unsigned kSpinLimit = 1u << 24;

// Device error word codes (written by kernels, read by the host).
enum DevError : int {
    kDevOk = 0,
    kDevTimeout = 1,
    kDevSingular = 2,
};

// Kernel classes timed by tmvg_timing_enable (the TMVG_KCLASS_* values).
enum KernelClass : int {
    kClsTrailingUpdate = 0,
    kClsPanel = 1,
    kClsTriSolve = 2,
    kClsResidual = 3,
    kClsCount = 4,
};

// One timed span: events recorded on the context's stream around the
// launches of one kernel class, with the algorithmic work they do.
struct TimedSpan {
    cudaEvent_t a, b;
    int cls;
    double bytes, flops;
};

// Per-context state shared by the C entry points.
struct Context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // Grow-only device workspace (bytes) for temporaries of one call.
    void* work = nullptr;
    size_t work_bytes = 0;
    // Device words: [0] error code, [1] aux (e.g. index where a wait gave up),
    // [2..] barrier counters.
    int* dflags = nullptr;
    unsigned* dbar = nullptr;
    int* hflags = nullptr;  // pinned mirror of dflags[0..2)
    int64_t launches = 0;
    std::string last_error;
    // Second grow-only workspace for drivers that call routines which use
    // `work` themselves (mixed-precision solve, batched solve).
    void* work2 = nullptr;
    size_t work2_bytes = 0;
    // Sync-free triangular solves: per-block publication flags (epoch
    // tagged, zeroed at creation) and the block ticket counter.
    unsigned* trsv_flags = nullptr;
    unsigned trsv_epoch = 0;
    unsigned long long* trsv_ticket = nullptr;
    // FP32 inverse-block solves publish each solution entry as one 64-bit
    // word (epoch << 32 | value bits); grow-only, never needs clearing.
    unsigned long long* trsv_pub = nullptr;
    size_t trsv_pub_len = 0;
    // Inverted 64 x 64 diagonal blocks of the many-column sync-free solve
    // (grow-only) and their per-block zero-diagonal flags.
    void* trsv_dinv = nullptr;
    size_t trsv_dinv_bytes = 0;
    // Whether a 16-CTA cluster of the panel kernel can be launched, per
    // element type (-1 unknown, 0 no, 1 yes): [0] double, [1] float.
    int cluster_ok[2] = {-1, -1};
    // The same for the register-resident panel kernel.
    int reg_cluster_ok[2] = {-1, -1};
    // The same for the complex LU's panel cluster, per panel width (32, 16).
    int zpanel_ok[2] = {-1, -1};
    // Third grow-only workspace: operand copies of the tensor-core update.
    void* work3 = nullptr;
    size_t work3_bytes = 0;
    // Device copies of the host entry points' operands (grow-only).
    void* io = nullptr;
    size_t io_bytes = 0;
    // Row-gather lists of the interchange -> permutation conversion
    // (grow-only; its callers keep the permutation in `work`).
    void* perm_lists = nullptr;
    size_t perm_lists_bytes = 0;
    // Kernel-class timing (off unless tmvg_timing_enable turned it on):
    // spans recorded but not yet read, recycled events, and per-class sums.
    bool timing = false;
    std::vector<TimedSpan> spans;
    std::vector<cudaEvent_t> event_pool;
    int64_t t_launches[kClsCount] = {};
    double t_ms[kClsCount] = {};
    double t_bytes[kClsCount] = {};
    double t_flops[kClsCount] = {};
    // Look-ahead of the LU: a high-priority side stream for the panels and
    // the events that order it against `stream` (created on first use).
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_wide = nullptr, ev_panel = nullptr;
    // TMVG_SERIALIZE_LOOKAHEAD=1 at creation: every side-stream panel is
    // waited for on the host before the main stream's next launch, which
    // fixes one extreme interleaving of the two streams (used by tests to
    // show that no cross-stream dependency is missing).
    bool serialize_lookahead = false;
    // TMVG_PANEL_REG2=1 at creation: the register panel updates every
    // column at every step (lu_panel_cluster_reg2_kernel) instead of by
    // leaves (lu_panel_leaf_kernel); the two give bitwise the same factors.
    bool panel_reg2 = false;
    // Failure-path test hooks (tmvg_test_set_wait): the poll limit of the
    // sync-free triangular solve's block-flag waits (0: kSpinLimit), and a
    // number of leading blocks the next such solve never hands out, so their
    // flags are never published (reset after one launch).
    unsigned poll_limit = 0;
    int test_skip_blocks = 0;
};

// The side stream and its events (nullptr-safe to call repeatedly).
tmvg_status ensure_side_stream(Context* c);

// Records CUDA events on c->stream around its scope when timing is on;
// the launches inside the scope count as one span of class `cls`.
class ScopedTimer {
  public:
    ScopedTimer(Context* c, int cls, double bytes, double flops, cudaStream_t stream);
    ScopedTimer(Context* c, int cls, double bytes, double flops)
        : ScopedTimer(c, cls, bytes, flops, c->stream) {}
    ~ScopedTimer();
    ScopedTimer(const ScopedTimer&) = delete;
    ScopedTimer& operator=(const ScopedTimer&) = delete;

  private:
    Context* c_;
    int cls_;
    double bytes_, flops_;
    cudaStream_t stream_;
    cudaEvent_t a_ = nullptr;
};

tmvg_status set_error(Context* c, tmvg_status s, const std::string& msg);
tmvg_status check_cuda(Context* c, cudaError_t e, const char* what);
// Ensure at least `bytes` of workspace; returns nullptr on failure.
void* workspace(Context* c, size_t bytes);
// FP64 FMA rate of the device in TFLOP/s (probe.cu; synchronises).
tmvg_status probe_fp64_rate(Context* c, double* tflops);
void* workspace2(Context* c, size_t bytes);
void* workspace3(Context* c, size_t bytes);
void* perm_lists_buffer(Context* c, size_t bytes);
void* trsv_dinv_buffer(Context* c, size_t bytes);
// Reads and clears the device error word (synchronises the stream).
tmvg_status collect_device_error(Context* c, const char* what);

// ---------------------------------------------------------------------
// Pivot search keys.
//
// TMV's maxAbsElement (src/TMV_Vector.cpp:474-503) scans from the first
// element with `if (|v_i| > max)`, so ties keep the lowest index and a NaN is
// chosen only when it is the first element.  A parallel reduction reproduces
// this with a key per element, compared as (key desc, index asc):
//   first element: |v|, or +inf when v is NaN ("maxabs" mode), or 0 when v is
//                  NaN in the second column of TMV's two-column leaf
//                  (src/TMV_LUDecompose.cpp:306-319), whose scan starts
//                  from max = 0 ("r2" mode);
//   other elements: |v|, or -1 when v is NaN.
// ---------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ double pivot_key(T v, bool first, bool r2mode)
{
    double a = fabs((double)v);
    if (a != a) return first ? (r2mode ? 0.0 : __longlong_as_double(0x7ff0000000000000LL)) : -1.0;
    return a;
}

// (key, index) max-reduction with lowest index on ties.
template <typename I>
__device__ __forceinline__ void pivot_combine(double& k, I& i, double k2, I i2)
{
    if (k2 > k || (k2 == k && i2 < i)) {
        k = k2;
        i = i2;
    }
}

template <typename I>
__device__ __forceinline__ void warp_pivot_reduce(double& k, I& i)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double k2 = __shfl_xor_sync(0xffffffffu, k, off);
        I i2 = __shfl_xor_sync(0xffffffffu, i, off);
        pivot_combine(k, i, k2, i2);
    }
}

// The same keys as ordered 64-bit integers, for reductions that should not
// take FP64 issue slots (a double comparison occupies the FP64 pipe, which
// GB300 issues at 2 per SM per clock): the bits of |v| (non-negative doubles
// order like their bit patterns), the bits of +inf or 0 for a NaN first
// element, -1 for a NaN elsewhere.
template <typename T>
__device__ __forceinline__ long long pivot_ikey(T v, bool first, bool r2mode)
{
    const long long b = __double_as_longlong((double)v) & 0x7fffffffffffffffLL;
    if (b > 0x7ff0000000000000LL) return first ? (r2mode ? 0LL : 0x7ff0000000000000LL) : -1LL;
    return b;
}

__device__ __forceinline__ void pivot_icombine(long long& k, long long& i, long long k2, long long i2)
{
    if (k2 > k || (k2 == k && i2 < i)) {
        k = k2;
        i = i2;
    }
}

__device__ __forceinline__ void warp_pivot_ireduce(long long& k, long long& i)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const long long k2 = __shfl_xor_sync(0xffffffffu, k, off);
        const long long i2 = __shfl_xor_sync(0xffffffffu, i, off);
        pivot_icombine(k, i, k2, i2);
    }
}

// TMV_Underflow for a real pivot magnitude a = |piv| (include/tmv/TMV_Base.h:
// 692-696, where TMV_ABS2 of a real is its absolute value, :330-331):
// a < numeric_limits<T>::min().  NaN never underflows.
template <typename T>
__device__ __forceinline__ bool underflows(double a);
template <>
__device__ __forceinline__ bool underflows<double>(double a) { return a < 2.2250738585072014e-308; }
template <>
__device__ __forceinline__ bool underflows<float>(double a) { return a < 1.1754943508222875e-38; }

// ---------------------------------------------------------------------
// Grid barrier for cooperative launches (all CTAs co-resident).
// `counter` is a monotonically increasing word zeroed before the launch; the
// b-th barrier (0-based) completes when it reaches (b+1)*gridDim.x.  The wait
// is bounded: on timeout it writes kDevTimeout into err[0] and returns false,
// and the caller must leave the kernel.
// ---------------------------------------------------------------------
__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned target, int* err)
{
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(counter, 1u);
        unsigned spins = 0;
        ok = 1;
        while (true) {
            unsigned v = *((volatile unsigned*)counter);
            if (v >= target) break;
            if (*((volatile int*)err) == kDevTimeout) { ok = 0; break; }
            if (++spins > kSpinLimit) {
                atomicExch(err, (int)kDevTimeout);
                ok = 0;
                break;
            }
            if (spins > 64) __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace tmvg
