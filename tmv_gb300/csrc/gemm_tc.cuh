// gemm_tc.cuh -- FP32-accurate C -= A B on tcgen05 tensor cores (3xTF32).
#pragma once

#include "common.cuh"

namespace tmvg {

// Whether the tensor-core update handles inner dimension K (a multiple of 32
// up to 128, with the tensor-map encoder available).
bool tf32x3_supported(int64_t K);

// C (m x n, column-major, ldc) -= A (m x K, column-major, lda) * B (K x n,
// column-major, ldb), FP32 data, 3xTF32 products accumulated in FP32.
tmvg_status gemm_f32_tf32x3_update(Context* c, int64_t m, int64_t n, int64_t K, const float* A,
                                   int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc);

}  // namespace tmvg
