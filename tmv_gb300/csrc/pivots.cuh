// pivots.cuh -- the interchanges of one panel as a row gather (device side).
#pragma once

#include "common.cuh"

namespace tmvg {

// Largest panel width any factorisation kernel uses.
constexpr int kPairsPanelMax = 128;

// ---------------------------------------------------------------------
// The interchanges of one panel as a row gather.  Applying
// swap(row k+t, row piv[t]) for t = 0..nb-1 in order moves row src[q] to
// row dst[q] for at most 2*nb pairs; only rows k..k+nb-1 and the pivot rows
// change.  One warp replays the swaps on row labels in shared memory: the
// panel block [k, k+nb) is an array, rows outside it (only ever pivot rows;
// a pivot row above the block, which no factorisation produces, is handled
// the same way) live in a short list searched with a ballot.  pairs[0] =
// count, then the dst and src arrays of kMaxPairs each.
// ---------------------------------------------------------------------
constexpr int kMaxPairs = 2 * kPairsPanelMax;

__device__ inline void panel_row_pairs(int64_t k, int nb, const int* piv, int* pairs)
{
    __shared__ int blk[kPairsPanelMax];
    __shared__ int orow[kPairsPanelMax], oval[kPairsPanelMax];
    __shared__ int ocnt;
    const int lane = threadIdx.x & 31;
    for (int t = lane; t < nb; t += 32) blk[t] = (int)(k + t);
    if (lane == 0) ocnt = 0;
    __syncwarp();
    for (int t = 0; t < nb; ++t) {
        const int p = piv[t];
        const int i = (int)(k + t);
        if (p != i) {
            if (p >= k && p < k + nb) {
                if (lane == 0) {
                    const int a = blk[t];
                    blk[t] = blk[p - k];
                    blk[p - k] = a;
                }
            } else {
                const int cnt = ocnt;
                int found = -1;
                for (int q0 = 0; q0 < cnt; q0 += 32) {
                    const int q = q0 + lane;
                    const unsigned m = __ballot_sync(0xffffffffu, q < cnt && orow[q] == p);
                    if (m) { found = q0 + __ffs(m) - 1; break; }
                }
                if (lane == 0) {
                    if (found >= 0) {
                        const int a = blk[t];
                        blk[t] = oval[found];
                        oval[found] = a;
                    } else {
                        orow[cnt] = p;
                        oval[cnt] = blk[t];
                        blk[t] = p;
                        ocnt = cnt + 1;
                    }
                }
            }
        }
        __syncwarp();
    }
    // emit the moved rows: row dst receives the old content of row src
    if (lane == 0) {
        int np = 0;
        int* dst = pairs + 1;
        int* src = pairs + 1 + kMaxPairs;
        for (int t = 0; t < nb; ++t)
            if (blk[t] != k + t) { dst[np] = (int)(k + t); src[np] = blk[t]; ++np; }
        for (int q = 0; q < ocnt; ++q)
            if (oval[q] != orow[q]) { dst[np] = orow[q]; src[np] = oval[q]; ++np; }
        pairs[0] = np;
    }
}

}  // namespace tmvg
