// gemm_tc.cuh -- FP32-accurate C -= A B on tcgen05 tensor cores (3xTF32).
#pragma once

#include "common.cuh"

namespace tmvg {

// Whether the tensor-core update handles inner dimension K (a multiple of 32
// up to 128, with the tensor-map encoder available).
bool tf32x3_supported(int64_t K);

// x rounded to TF32 (round to nearest, ties away from zero); hi = tf32(x)
// and lo = tf32(x - hi) split an FP32 value for the 3xTF32 product.
__device__ __forceinline__ float tf32_round(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Operand copies of one update in the context's third workspace: A hi/lo
// row-major m x K, B hi/lo column-major K x n (leading dimension K).  A
// caller may split B in column ranges and pass offset pointers to apply.
struct Tf32x3Buffers {
    float *Ahi, *Alo, *Bhi, *Blo;
};
tmvg_status tf32x3_buffers(Context* c, int64_t m, int64_t n, int64_t K, Tf32x3Buffers* b);
// A (m x K, column-major, lda) -> b.Ahi / b.Alo.
tmvg_status tf32x3_split_a(Context* c, int64_t m, int64_t K, const float* A, int64_t lda,
                           const Tf32x3Buffers& b);
// B (K x n, column-major, ldb) -> b.Bhi / b.Blo.
tmvg_status tf32x3_split_b(Context* c, int64_t n, int64_t K, const float* B, int64_t ldb,
                           const Tf32x3Buffers& b);
// C (m x n, column-major, ldc) -= A B from the split copies in b.
tmvg_status tf32x3_apply(Context* c, int64_t m, int64_t n, int64_t K, const Tf32x3Buffers& b, float* C,
                         int64_t ldc);

// C (m x n, column-major, ldc) -= A (m x K, column-major, lda) * B (K x n,
// column-major, ldb), FP32 data, 3xTF32 products accumulated in FP32.
tmvg_status gemm_f32_tf32x3_update(Context* c, int64_t m, int64_t n, int64_t K, const float* A,
                                   int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc);

}  // namespace tmvg
