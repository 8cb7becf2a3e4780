// trsv.cuh -- single-launch triangular solves and pivot permutations.
#pragma once

#include "common.cuh"

namespace tmvg {

// Capacity of the per-context block-flag array (64-row blocks): n <= 4M.
constexpr int64_t kTrsvFlagCap = 65536;

// B := T^-1 B for the lower (upper = false) or upper triangle of `tri`
// (strides tsi, tsj; unit diagonal not read when unit), B n x nrhs with
// strides; skip_zero as in tri_solve().  Best for nrhs <= 8.
template <typename T>
tmvg_status trsm_sync_free(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                           bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi, int64_t bsj,
                           bool skip_zero);

// Repeated one-column solves with one triangle: invert its 128 x 128
// diagonal blocks once (dinv: ceil(n/128)*128*128 elements, singular:
// ceil(n/128) ints), then solve x := T^-1 x with one launch per solve.
constexpr int64_t kInvBlock = 128;
template <typename T>
tmvg_status trsv_factor_inverse_blocks(Context* c, int64_t n, const T* tri, int64_t tsi,
                                       int64_t tsj, bool upper, bool unit, T* dinv, int* singular);
// (trsv_with_inverse_blocks: stop, when given, is a device word; a nonzero
// value makes the launch return at once, for solves enqueued ahead by a loop
// that decides on the device when to stop.)
// Both triangles of a packed LU factor (column-major, leading dimension ld)
// in one launch: unit lower L into (dinvL, singL), upper U into (dinvU, singU).
template <typename T>
tmvg_status trsv_lu_inverse_blocks(Context* c, int64_t n, const T* LU, int64_t ld, T* dinvL,
                                   int* singL, T* dinvU, int* singU);
template <typename T>
tmvg_status trsv_with_inverse_blocks(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                                     bool upper, bool unit, const T* dinv, const int* singular,
                                     T* x, int64_t incx, bool skip_zero, const int* stop = nullptr,
                                     const T* mlink = nullptr);
// Link blocks of an FP32 factor for trsv_with_inverse_blocks (mlink, FP32
// only; used when n is a multiple of 128): M_b = Dinv_b T[b, b-1] for both
// triangles (ceil(n/128)*128*128 floats each), computed once per factor
// after trsv_lu_inverse_blocks.
tmvg_status trsv_lu_link_blocks(Context* c, int64_t n, const float* LU, int64_t ld, const float* dinvL,
                                const int* singL, float* mlinkL, const float* dinvU, const int* singU,
                                float* mlinkU);

// Interchange vector P (TMV/LAPACK form) -> gather permutation perm with
// (P B)[i] = B[perm[i]].
tmvg_status pivots_to_perm(Context* c, int64_t n, const int64_t* P, int* perm);

// out[i,:] = in[perm[i],:] (inverse = false) or out[perm[i],:] = in[i,:].
template <typename T>
tmvg_status permute_rows(Context* c, int64_t n, int64_t ncols, const int* perm, const T* in,
                         int64_t isi, int64_t isj, T* out, int64_t osi, int64_t osj, bool inverse);

}  // namespace tmvg
