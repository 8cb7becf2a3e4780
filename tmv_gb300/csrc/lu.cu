// lu.cu -- partial-pivoting LU factorisation and LU solves on sm_103a.
//
// Algorithm (right-looking, blocked; the reference is recursive,
// src/TMV_LUDecompose.cpp:217-407, and produces the same factors up to the
// rounding of the trailing updates):
//   for each panel of kPanel columns starting at k:
//     1. lu_panel_kernel: factor A[k:n, k:k+nb] column by column with TMV's
//        pivot rule; the panel lives in the shared memory of up to one CTA
//        per SM, one bounded grid barrier per column;
//     2. laswp_kernel: apply the panel's interchanges to the other columns
//        (TMV: A1.permuteRows(P,0,N1) and A0.permuteRows(P,N1,R));
//     3. tri_diag_kernel: U12 = L11^-1 A12 (TMV: A01 /= A00.lowerTri(UnitDiag));
//     4. gemm: A22 -= L21 U12 (TMV: A11 -= A10*A01 -> MultMM<true>(-1,...)).
//
// Pivot rule (src/TMV_Vector.cpp:474-503, src/TMV_LUDecompose.cpp:274-383):
// first index of the strict maximum |a| over the sub-column, NaN handling as
// described at pivot_key(); a maximum |a| < DBL_MIN (TMV_Underflow,
// include/tmv/TMV_Base.h:692-696) zeroes the sub-column and records P[j] = j.
// The L column is scaled by the reciprocal of the pivot, as TMV's v /= x does
// (include/tmv/TMV_VectorArith.h:104-106).
#include "lu.cuh"
#include "trsv.cuh"

#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

namespace tmvg {

constexpr int kPanelThreads = 256;
constexpr int kPanelMax = 128;  // largest panel width (scratch layout)
constexpr int kTriBlock = 64;   // diagonal block of the blocked triangular solves

// Panel width: 64 columns in FP64, 128 in FP32 (same shared-memory
// footprint, 256 rows x ~33 KB per CTA; wider FP32 panels halve the number
// of trailing updates and so the trailing-matrix traffic).
template <typename T>
constexpr int panel_width() { return sizeof(T) == 8 ? 64 : 128; }

// ---------------------------------------------------------------------
// Columns that TMV factors as the second column of a two-column leaf of its
// recursion (split N1 = R/2, rounded down to a multiple of 64 above 64,
// src/TMV_LUDecompose.cpp:241-245).  Their pivot scan starts from max = 0,
// which only matters for NaN input.
// ---------------------------------------------------------------------
static void leaf_modes(int64_t off, int64_t R, std::vector<unsigned char>& modes)
{
    if (R > 2) {
        int64_t N1 = R / 2;
        if (N1 > 64) N1 = (N1 / 64) * 64;
        leaf_modes(off, N1, modes);
        leaf_modes(off + N1, R - N1, modes);
    } else if (R == 2) {
        modes[off + 1] = 1;
    }
}

// ---------------------------------------------------------------------
// Panel factorisation.
// ---------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
lu_panel_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int nb,
                int64_t* __restrict__ P, const unsigned char* __restrict__ modes,
                int rows_per_cta, double* cand_key, long long* cand_idx,
                T* cand_rows, T* diag_row, unsigned* bar, int* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* rows = reinterpret_cast<T*>(smem_raw);
    const int ldp = nb + 1;
    __shared__ double s_key[kPanelThreads / 32];
    __shared__ long long s_idx[kPanelThreads / 32];
    __shared__ double w_key;
    __shared__ long long w_idx;
    __shared__ T urow[kPanelMax];

    const int G = gridDim.x;
    const int cta = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t m = n - k;
    const int64_t r0 = (int64_t)cta * rows_per_cta;
    const int nr = (int)max((int64_t)0, min((int64_t)rows_per_cta, m - r0));

    for (int t = tid; t < nr * nb; t += kPanelThreads) {
        const int r = t % nr, cc = t / nr;
        rows[r * ldp + cc] = A[(k + r0 + r) + (k + cc) * lda];
    }
    __syncthreads();

    bool prev_uf = false;
    for (int jj = 0; jj < nb; ++jj) {
        const int par = jj & 1;
        const bool r2 = modes[jj] && !prev_uf;

        // 1. this CTA's best candidate among panel rows >= jj
        double bk = -INFINITY;
        long long bi = LLONG_MAX;
        for (int r = tid; r < nr; r += kPanelThreads) {
            const int64_t pr = r0 + r;
            if (pr < jj) continue;
            pivot_combine(bk, bi, pivot_key(rows[r * ldp + jj], pr == jj, r2), (long long)pr);
        }
        warp_pivot_reduce(bk, bi);
        if (lane == 0) { s_key[warp] = bk; s_idx[warp] = bi; }
        __syncthreads();
        if (warp == 0) {
            bk = lane < kPanelThreads / 32 ? s_key[lane] : -INFINITY;
            bi = lane < kPanelThreads / 32 ? s_idx[lane] : LLONG_MAX;
            warp_pivot_reduce(bk, bi);
            if (lane == 0) {
                __stcg(&cand_key[par * G + cta], bk);
                __stcg(&cand_idx[par * G + cta], bi);
                w_idx = bi;  // local use below
            }
        }
        __syncthreads();
        // 2. publish the candidate row and (owner only) the diagonal row
        {
            const long long mine = w_idx;
            if (mine != LLONG_MAX) {
                const int r = (int)(mine - r0);
                for (int cc = tid; cc < nb; cc += kPanelThreads)
                    __stcg(&cand_rows[((int64_t)par * G + cta) * kPanelMax + cc], rows[r * ldp + cc]);
            }
            if (jj >= r0 && jj < r0 + nr) {
                const int r = (int)(jj - r0);
                for (int cc = tid; cc < nb; cc += kPanelThreads)
                    __stcg(&diag_row[par * kPanelMax + cc], rows[r * ldp + cc]);
            }
        }
        if (!grid_barrier(bar, (unsigned)(jj + 1) * (unsigned)G, err)) return;

        // 3. global winner
        if (warp == 0) {
            double kk = -INFINITY;
            long long ii = LLONG_MAX;
            for (int g = lane; g < G; g += 32)
                pivot_combine(kk, ii, __ldcg(&cand_key[par * G + g]), __ldcg(&cand_idx[par * G + g]));
            warp_pivot_reduce(kk, ii);
            if (lane == 0) { w_key = kk; w_idx = ii; }
        }
        __syncthreads();
        const double wk = w_key;
        const long long wi = w_idx;  // panel row of the pivot

        if (underflows<T>(wk)) {
            if (cta == 0 && tid == 0) P[k + jj] = k + jj;
            for (int r = tid; r < nr; r += kPanelThreads)
                if (r0 + r >= jj) rows[r * ldp + jj] = T(0);
            prev_uf = true;
        } else {
            prev_uf = false;
            if (cta == 0 && tid == 0) P[k + jj] = k + wi;
            const int wc = (int)(wi / rows_per_cta);
            for (int cc = tid; cc < nb; cc += kPanelThreads)
                urow[cc] = __ldcg(&cand_rows[((int64_t)par * G + wc) * kPanelMax + cc]);
            __syncthreads();
            if (wi != jj) {
                if (jj >= r0 && jj < r0 + nr) {
                    const int r = (int)(jj - r0);
                    for (int cc = tid; cc < nb; cc += kPanelThreads) rows[r * ldp + cc] = urow[cc];
                }
                if (wi >= r0 && wi < r0 + nr) {
                    const int r = (int)(wi - r0);
                    for (int cc = tid; cc < nb; cc += kPanelThreads)
                        rows[r * ldp + cc] = __ldcg(&diag_row[par * kPanelMax + cc]);
                }
            }
            __syncthreads();
            const T inv = T(1) / urow[jj];
            for (int r = tid; r < nr; r += kPanelThreads) {
                if (r0 + r <= jj) continue;
                T* rw = rows + r * ldp;
                const T l = rw[jj] * inv;
                rw[jj] = l;
                for (int cc = jj + 1; cc < nb; ++cc) rw[cc] -= l * urow[cc];
            }
        }
        __syncthreads();
    }

    for (int t = tid; t < nr * nb; t += kPanelThreads) {
        const int r = t % nr, cc = t / nr;
        A[(k + r0 + r) + (k + cc) * lda] = rows[r * ldp + cc];
    }
}

// ---------------------------------------------------------------------
// Row interchanges.
// ---------------------------------------------------------------------
// Interchanges P[k..k+nb) applied to columns [0, ncols) except [skip0, skip1).
template <typename T>
__global__ void laswp_kernel(T* __restrict__ A, int64_t lda, int64_t ncols, int64_t k, int nb,
                             const int64_t* __restrict__ P, int64_t skip0, int64_t skip1)
{
    __shared__ int64_t sp[kPanelMax];
    for (int t = threadIdx.x; t < nb; t += blockDim.x) sp[t] = P[k + t];
    __syncthreads();
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= ncols || (c >= skip0 && c < skip1)) return;
    T* col = A + c * lda;
    for (int t = 0; t < nb; ++t) {
        const int64_t i = k + t, p = sp[t];
        if (p != i) {
            const T a = col[i];
            col[i] = col[p];
            col[p] = a;
        }
    }
}

// General interchanges on a strided matrix (one thread per column).
template <typename T>
__global__ void pivot_rows_kernel(int64_t ncols, T* __restrict__ B, int64_t bsi, int64_t bsj,
                                  const int64_t* __restrict__ P, int64_t i1, int64_t i2, bool reverse)
{
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    T* col = B + c * bsj;
    if (!reverse) {
        for (int64_t i = i1; i < i2; ++i) {
            const int64_t p = P[i];
            if (p != i) { const T a = col[i * bsi]; col[i * bsi] = col[p * bsi]; col[p * bsi] = a; }
        }
    } else {
        for (int64_t i = i2; i > i1;) {
            --i;
            const int64_t p = P[i];
            if (p != i) { const T a = col[i * bsi]; col[i * bsi] = col[p * bsi]; col[p * bsi] = a; }
        }
    }
}

// ---------------------------------------------------------------------
// Triangular solve of one diagonal block (w <= kTriBlock rows) for many
// right-hand sides: each thread substitutes one column, held in shared
// memory.  Lower: x_i = (b_i - sum_{j<i} T_ij x_j) / T_ii; upper the mirror,
// with the sums taken in the order TMV's column-oriented vector solve applies
// its updates (src/TMV_TriDiv_V.cpp:148-236, 322-398).
// skip_zero reproduces that solve's "if (*bj != 0)" test: a zero diagonal
// only raises SINGULAR where it would divide a nonzero; the division is then
// a true division.  Otherwise (TMV's row-major leaves,
// src/TMV_TriDiv_M.cpp:58-188) every zero diagonal is singular and the row
// is multiplied by the reciprocal.
// ---------------------------------------------------------------------
constexpr int kTriCols = 64;
template <typename T>
__global__ void __launch_bounds__(kTriCols)
tri_diag_kernel(int w, const T* __restrict__ tri, int64_t tsi, int64_t tsj, bool upper,
                bool unit, int64_t nrhs, T* __restrict__ B, int64_t bsi, int64_t bsj,
                bool skip_zero, int* err)
{
    // dynamic shared memory: Ts[w][w+1] then Xs[w][kTriCols+1]
    extern __shared__ __align__(16) unsigned char tri_smem[];
    T* Tsb = reinterpret_cast<T*>(tri_smem);
    T* Xsb = Tsb + w * (w + 1);
#define Ts(i, j) Tsb[(i) * (w + 1) + (j)]
#define Xs(i, j) Xsb[(i) * (kTriCols + 1) + (j)]
    const int tid = threadIdx.x;
    const int64_t c0 = (int64_t)blockIdx.x * kTriCols;
    const int ncb = (int)min((int64_t)kTriCols, nrhs - c0);

    for (int t = tid; t < w * w; t += kTriCols) {
        const int i = t % w, j = t / w;
        const bool need = upper ? (j >= i) : (i >= j);
        Ts(i, j) = need ? tri[i * tsi + j * tsj] : T(0);
    }
    if (bsi == 1) {
        for (int t = tid; t < w * ncb; t += kTriCols) {
            const int i = t % w, cl = t / w;
            Xs(i, cl) = B[i + (c0 + cl) * bsj];
        }
    } else {
        for (int t = tid; t < w * ncb; t += kTriCols) {
            const int cl = t % ncb, i = t / ncb;
            Xs(i, cl) = B[i * bsi + (c0 + cl) * bsj];
        }
    }
    __syncthreads();

    if (tid < ncb) {
        bool sing = false;
        if (!upper) {
            for (int i = 0; i < w; ++i) {
                T s = Xs(i, tid);
                for (int j = 0; j < i; ++j) s -= Ts(i, j) * Xs(j, tid);
                if (!unit) {
                    const T d = Ts(i, i);
                    if (skip_zero) {
                        if (s != T(0)) {
                            if (d == T(0)) sing = true;
                            else s = s / d;
                        }
                    } else {
                        if (d == T(0)) sing = true;
                        else s = s * (T(1) / d);
                    }
                }
                Xs(i, tid) = s;
            }
        } else {
            for (int i = w - 1; i >= 0; --i) {
                T s = Xs(i, tid);
                for (int j = w - 1; j > i; --j) s -= Ts(i, j) * Xs(j, tid);
                if (!unit) {
                    const T d = Ts(i, i);
                    if (skip_zero) {
                        if (s != T(0)) {
                            if (d == T(0)) sing = true;
                            else s = s / d;
                        }
                    } else {
                        if (d == T(0)) sing = true;
                        else s = s * (T(1) / d);
                    }
                }
                Xs(i, tid) = s;
            }
        }
        if (sing) atomicCAS(err, (int)kDevOk, (int)kDevSingular);
    }
    __syncthreads();
    if (bsi == 1) {
        for (int t = tid; t < w * ncb; t += kTriCols) {
            const int i = t % w, cl = t / w;
            B[i + (c0 + cl) * bsj] = Xs(i, cl);
        }
    } else {
        for (int t = tid; t < w * ncb; t += kTriCols) {
            const int cl = t % ncb, i = t / ncb;
            B[i * bsi + (c0 + cl) * bsj] = Xs(i, cl);
        }
    }
}
#undef Ts
#undef Xs

// Strided copy out(i, j) = in(i, j).
template <typename T>
__global__ void copy_kernel(int64_t m, int64_t n, const T* __restrict__ in, int64_t isi,
                            int64_t isj, T* __restrict__ out, int64_t osi, int64_t osj)
{
    const int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % m, j = t / m;
        out[i * osi + j * osj] = in[i * isi + j * isj];
    }
}

template <typename T>
tmvg_status copy_matrix(Context* c, int64_t m, int64_t n, const T* in, int64_t isi, int64_t isj,
                        T* out, int64_t osi, int64_t osj)
{
    if (m <= 0 || n <= 0) return TMVG_OK;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(m * n, 256), 8 * c->num_sms);
    copy_kernel<T><<<blocks, 256, 0, c->stream>>>(m, n, in, isi, isj, out, osi, osj);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "copy launch");
}

// ---------------------------------------------------------------------
// Host drivers.
// ---------------------------------------------------------------------
template <typename T>
static tmvg_status launch_tri_diag(Context* c, int w, const T* tri, int64_t tsi, int64_t tsj,
                                   bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi,
                                   int64_t bsj, bool skip_zero)
{
    if (nrhs <= 0 || w <= 0) return TMVG_OK;
    const int64_t blocks = ceil_div(nrhs, kTriCols);
    if (blocks > INT_MAX) return set_error(c, TMVG_UNSUPPORTED, "tri solve: too many columns");
    const size_t smem = sizeof(T) * ((size_t)w * (w + 1) + (size_t)w * (kTriCols + 1));
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(tri_diag_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(T) * (kTriBlock * (kTriBlock + 1) + kTriBlock * (kTriCols + 1))));
    tri_diag_kernel<T><<<(unsigned)blocks, kTriCols, smem, c->stream>>>(
        w, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip_zero, c->dflags);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "tri_diag launch");
}

template <typename T>
tmvg_status tri_solve(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                      bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi, int64_t bsj,
                      bool skip_zero)
{
    if (n <= 0 || nrhs <= 0) return TMVG_OK;
    tmvg_status st;
    if (!upper) {
        for (int64_t kb = 0; kb < n; kb += kTriBlock) {
            const int w = (int)std::min<int64_t>(kTriBlock, n - kb);
            st = launch_tri_diag<T>(c, w, tri + kb * tsi + kb * tsj, tsi, tsj, false, unit, nrhs,
                                    B + kb * bsi, bsi, bsj, skip_zero);
            if (st) return st;
            if (kb + w < n) {
                st = gemm<T>(c, n - kb - w, nrhs, w, T(-1),
                             Mat<const T>{tri + (kb + w) * tsi + kb * tsj, tsi, tsj},
                             Mat<const T>{B + kb * bsi, bsi, bsj}, T(1),
                             Mat<T>{B + (kb + w) * bsi, bsi, bsj});
                if (st) return st;
            }
        }
    } else {
        const int64_t last = ((n - 1) / kTriBlock) * kTriBlock;
        for (int64_t kb = last; kb >= 0; kb -= kTriBlock) {
            const int w = (int)std::min<int64_t>(kTriBlock, n - kb);
            st = launch_tri_diag<T>(c, w, tri + kb * tsi + kb * tsj, tsi, tsj, true, unit, nrhs,
                                    B + kb * bsi, bsi, bsj, skip_zero);
            if (st) return st;
            if (kb > 0) {
                st = gemm<T>(c, kb, nrhs, w, T(-1), Mat<const T>{tri + kb * tsj, tsi, tsj},
                             Mat<const T>{B + kb * bsi, bsi, bsj}, T(1), Mat<T>{B, bsi, bsj});
                if (st) return st;
            }
        }
    }
    return TMVG_OK;
}

template <typename T>
tmvg_status apply_pivots(Context* c, int64_t ncols, T* B, int64_t bsi, int64_t bsj,
                         const int64_t* P, int64_t i1, int64_t i2, bool reverse)
{
    if (ncols <= 0 || i2 <= i1) return TMVG_OK;
    pivot_rows_kernel<T><<<(unsigned)ceil_div(ncols, 128), 128, 0, c->stream>>>(
        ncols, B, bsi, bsj, P, i1, i2, reverse);
    ++c->launches;
    return check_cuda(c, cudaGetLastError(), "pivot_rows launch");
}

template <typename T>
tmvg_status lu_factor(Context* c, int64_t n, T* A, int64_t lda, int64_t* P)
{
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return set_error(c, TMVG_BAD_ARG, "lu: bad n/lda");
    if (n == 0) return TMVG_OK;
    const int nbmax = panel_width<T>();

    // Panel geometry: one CTA per 256 rows up to one per SM.
    const int64_t G_full = std::min<int64_t>(c->num_sms, ceil_div(n, kPanelThreads));
    const int64_t rows_full = ceil_div(n, G_full);
    const size_t smem_full = (size_t)rows_full * (nbmax + 1) * sizeof(T);
    if (smem_full > 200 * 1024)
        return set_error(c, TMVG_UNSUPPORTED, "lu: matrix too tall for the shared-memory panel");

    // Workspace: modes (n bytes), candidate keys/indices/rows, diag rows.
    const size_t off_key = 0;
    const size_t off_idx = off_key + sizeof(double) * 2 * G_full;
    const size_t off_rows = (off_idx + sizeof(long long) * 2 * G_full + 255) & ~size_t(255);
    const size_t off_diag = off_rows + sizeof(T) * 2 * G_full * kPanelMax;
    const size_t off_modes = (off_diag + sizeof(T) * 2 * kPanelMax + 255) & ~size_t(255);
    const size_t bytes = off_modes + (size_t)n;
    unsigned char* ws = (unsigned char*)workspace(c, bytes);
    if (!ws) return TMVG_OOM;
    double* cand_key = (double*)(ws + off_key);
    long long* cand_idx = (long long*)(ws + off_idx);
    T* cand_rows = (T*)(ws + off_rows);
    T* diag_row = (T*)(ws + off_diag);
    unsigned char* modes = ws + off_modes;
    {
        std::vector<unsigned char> hm((size_t)n, 0);
        leaf_modes(0, n, hm);
        tmvg_status st = check_cuda(
            c, cudaMemcpyAsync(modes, hm.data(), (size_t)n, cudaMemcpyHostToDevice, c->stream),
            "lu: modes upload");
        if (st) return st;
        // the host vector must outlive the copy
        st = check_cuda(c, cudaStreamSynchronize(c->stream), "lu: modes sync");
        if (st) return st;
    }

    static bool attr_set[2] = {false, false};
    const int ai = sizeof(T) == 8 ? 0 : 1;
    if (!attr_set[ai]) {
        cudaFuncSetAttribute(lu_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        attr_set[ai] = true;
    }

    for (int64_t k = 0; k < n; k += nbmax) {
        const int nb = (int)std::min<int64_t>(nbmax, n - k);
        const int64_t m = n - k;
        const int G = (int)std::min<int64_t>(c->num_sms, ceil_div(m, kPanelThreads));
        const int rows_per_cta = (int)ceil_div(m, G);
        const size_t smem = (size_t)rows_per_cta * (nb + 1) * sizeof(T);
        tmvg_status st = check_cuda(c, cudaMemsetAsync(c->dbar, 0, sizeof(unsigned), c->stream),
                                    "lu: barrier reset");
        if (st) return st;
        T* Ap = A;
        int64_t* Pp = P;
        const unsigned char* mp = modes + k;
        int64_t ldav = lda, nv = n, kv = k;
        int nbv = nb, rpc = rows_per_cta;
        unsigned* bar = c->dbar;
        int* err = c->dflags;
        void* args[] = {&Ap, &ldav, &nv, &kv, &nbv, &Pp, &mp, &rpc, &cand_key, &cand_idx,
                        &cand_rows, &diag_row, &bar, &err};
        st = check_cuda(c,
                        cudaLaunchCooperativeKernel((const void*)lu_panel_kernel<T>, dim3(G),
                                                    dim3(kPanelThreads), args, smem, c->stream),
                        "lu: panel launch");
        if (st) return st;
        ++c->launches;

        // interchanges on the other columns
        if (n > nb) {
            laswp_kernel<T><<<(unsigned)ceil_div(n, 128), 128, 0, c->stream>>>(A, lda, n, k, nb, P,
                                                                              k, k + nb);
            ++c->launches;
            st = check_cuda(c, cudaGetLastError(), "lu: laswp launch");
            if (st) return st;
        }
        if (k + nb < n) {
            const int64_t rest = n - k - nb;
            st = tri_solve<T>(c, nb, A + k + k * lda, 1, lda, false, true, rest,
                              A + k + (k + nb) * lda, 1, lda, false);
            if (st) return st;
            st = gemm<T>(c, rest, rest, nb, T(-1), Mat<const T>{A + (k + nb) + k * lda, 1, lda},
                         Mat<const T>{A + k + (k + nb) * lda, 1, lda}, T(1),
                         Mat<T>{A + (k + nb) + (k + nb) * lda, 1, lda});
            if (st) return st;
        }
    }
    return collect_device_error(c, "lu_factor");
}

// Triangular solve of the pivoted right-hand sides: the single-launch
// sync-free kernel for few columns, the blocked product-based solve for many.
template <typename T>
static tmvg_status tri_any(Context* c, int64_t n, const T* tri, int64_t tsi, int64_t tsj,
                           bool upper, bool unit, int64_t nrhs, T* B, int64_t bsi, int64_t bsj,
                           bool skip_zero)
{
    if (nrhs <= 8)
        return trsm_sync_free<T>(c, n, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip_zero);
    return tri_solve<T>(c, n, tri, tsi, tsj, upper, unit, nrhs, B, bsi, bsj, skip_zero);
}

template <typename T>
tmvg_status lu_ldiveq(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                      int64_t nrhs, T* B, int64_t bsi, int64_t bsj)
{
    // src/TMV_LUDiv.cpp:186-226: m.permuteRows(P); m /= L(unit); m /= U.
    // The interchanges are applied as one gather into a dense column-major
    // scratch, which is solved and copied back.
    if (n <= 0 || nrhs <= 0) return TMVG_OK;
    const size_t pbytes = (sizeof(int) * (size_t)n + 255) & ~size_t(255);
    unsigned char* ws = (unsigned char*)workspace(c, pbytes + sizeof(T) * (size_t)n * nrhs);
    if (!ws) return TMVG_OOM;
    int* perm = (int*)ws;
    T* X = (T*)(ws + pbytes);
    tmvg_status st = pivots_to_perm(c, n, P, perm);
    if (st) return st;
    st = permute_rows<T>(c, n, nrhs, perm, B, bsi, bsj, X, 1, n, false);
    if (st) return st;
    // Column-major B (or one column) takes TMV's vector path: skip semantics.
    st = tri_any<T>(c, n, LU, 1, lda, false, true, nrhs, X, 1, n, true);
    if (st) return st;
    st = tri_any<T>(c, n, LU, 1, lda, true, false, nrhs, X, 1, n, true);
    if (st) return st;
    st = copy_matrix<T>(c, n, nrhs, X, 1, n, B, bsi, bsj);
    if (st) return st;
    return collect_device_error(c, "lu_ldiveq");
}

template <typename T>
tmvg_status lu_rdiveq(Context* c, int64_t n, const T* LU, int64_t lda, const int64_t* P,
                      int64_t nrows, T* B, int64_t bsi, int64_t bsj)
{
    // src/TMV_LUDiv.cpp:370-411: m %= U; m %= L; m.reversePermuteCols(P), with
    // m %= T computed as T^T.LDivEq(m^T) (include/tmv/TMV_TriMatrix.h:945-946).
    if (n <= 0 || nrows <= 0) return TMVG_OK;
    const size_t pbytes = (sizeof(int) * (size_t)n + 255) & ~size_t(255);
    unsigned char* ws = (unsigned char*)workspace(c, pbytes + sizeof(T) * (size_t)n * nrows);
    if (!ws) return TMVG_OOM;
    int* perm = (int*)ws;
    T* X = (T*)(ws + pbytes);  // m^T, n x nrows column-major
    // m^T: element (i, j) = B[j*bsi + i*bsj]
    tmvg_status st = copy_matrix<T>(c, n, nrows, B, bsj, bsi, X, 1, n);
    if (st) return st;
    // One row of m is one vector (skip semantics); otherwise m^T is
    // row-major in TMV and its row-major leaves check every diagonal.
    const bool skip = (nrows == 1);
    st = tri_any<T>(c, n, LU, lda, 1, false, false, nrows, X, 1, n, skip);
    if (st) return st;
    st = tri_any<T>(c, n, LU, lda, 1, true, true, nrows, X, 1, n, skip);
    if (st) return st;
    // reversePermuteCols(P): undo the interchanges, i.e. scatter by perm
    st = pivots_to_perm(c, n, P, perm);
    if (st) return st;
    st = permute_rows<T>(c, n, nrows, perm, X, 1, n, B, bsj, bsi, true);
    if (st) return st;
    return collect_device_error(c, "lu_rdiveq");
}

template tmvg_status lu_factor<double>(Context*, int64_t, double*, int64_t, int64_t*);
template tmvg_status lu_factor<float>(Context*, int64_t, float*, int64_t, int64_t*);
template tmvg_status tri_solve<double>(Context*, int64_t, const double*, int64_t, int64_t, bool,
                                       bool, int64_t, double*, int64_t, int64_t, bool);
template tmvg_status tri_solve<float>(Context*, int64_t, const float*, int64_t, int64_t, bool,
                                      bool, int64_t, float*, int64_t, int64_t, bool);
template tmvg_status apply_pivots<double>(Context*, int64_t, double*, int64_t, int64_t,
                                          const int64_t*, int64_t, int64_t, bool);
template tmvg_status apply_pivots<float>(Context*, int64_t, float*, int64_t, int64_t,
                                         const int64_t*, int64_t, int64_t, bool);
template tmvg_status lu_ldiveq<double>(Context*, int64_t, const double*, int64_t, const int64_t*,
                                       int64_t, double*, int64_t, int64_t);
template tmvg_status lu_rdiveq<double>(Context*, int64_t, const double*, int64_t, const int64_t*,
                                       int64_t, double*, int64_t, int64_t);
template tmvg_status lu_ldiveq<float>(Context*, int64_t, const float*, int64_t, const int64_t*,
                                      int64_t, float*, int64_t, int64_t);
template tmvg_status copy_matrix<double>(Context*, int64_t, int64_t, const double*, int64_t,
                                         int64_t, double*, int64_t, int64_t);
template tmvg_status copy_matrix<float>(Context*, int64_t, int64_t, const float*, int64_t,
                                        int64_t, float*, int64_t, int64_t);

}  // namespace tmvg

// =====================================================================
// LU factorisation without device allocation.
//
// Some callers of this library cannot allocate device memory: programs whose
// device memory is owned entirely by another allocator (a framework's caching
// allocator or a fixed arena that must not see cudaMalloc behind its back),
// and code paths where an allocation's latency or failure is not acceptable.
// tmvg_lu_decompose_f64_noalloc serves them: it runs the same kernels as
// tmvg_lu_decompose_f64 but takes every scratch word from the file-scope
// array below, which each GPU that loads this library holds until the process
// exits (kNoAllocBytes, about 343 KiB).  It needs no tmvg_handle (creating one
// allocates).  Limits: n <= kNoAllocMaxN = 16384 (larger n returns
// TMVG_UNSUPPORTED before any device work); at most kNoAllocMaxCtas = 160
// panel CTAs are used.
// =====================================================================
namespace tmvg {
namespace {
constexpr int64_t kNoAllocMaxN = 16384;
constexpr int kNoAllocMaxCtas = 160;
constexpr size_t kNaOffErr = 0;    // int[2]: device error word + aux
constexpr size_t kNaOffBar = 64;   // unsigned: grid-barrier counter
constexpr size_t kNaOffKey = 256;  // double[2 * kNoAllocMaxCtas]
constexpr size_t kNaOffIdx = kNaOffKey + sizeof(double) * 2 * kNoAllocMaxCtas;
constexpr size_t kNaOffRows = kNaOffIdx + sizeof(long long) * 2 * kNoAllocMaxCtas;
constexpr size_t kNaOffDiag = kNaOffRows + sizeof(double) * 2 * kNoAllocMaxCtas * kPanelMax;
constexpr size_t kNaOffModes = kNaOffDiag + sizeof(double) * 2 * kPanelMax;
constexpr size_t kNoAllocBytes = kNaOffModes + kNoAllocMaxN;
constexpr int kNoAllocMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_lu_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array on `device` (which must be current).
// The host-side name of a __device__ array is only a stand-in, so the
// address is asked of the runtime once per device and cached.
static unsigned char* noalloc_scratch(int device, tmvg_status* st)
{
    static std::mutex mu;
    static unsigned char* addr[kNoAllocMaxDevices] = {};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 0 || device >= kNoAllocMaxDevices) {
        *st = TMVG_UNSUPPORTED;
        return nullptr;
    }
    if (!addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_lu_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            *st = TMVG_CUDA_ERROR;
            return nullptr;
        }
        addr[device] = static_cast<unsigned char*>(p);
    }
    *st = TMVG_OK;
    return addr[device];
}

}  // namespace tmvg

extern "C" tmvg_status tmvg_lu_decompose_f64_noalloc(int64_t n, double* A, int64_t lda, int64_t* P,
                                                     void* stream)
{
    using namespace tmvg;
    if (n < 0 || lda < std::max<int64_t>(n, 1)) return TMVG_BAD_ARG;
    if (n > kNoAllocMaxN) return TMVG_UNSUPPORTED;
    if (n == 0) return TMVG_OK;
    if (!A || !P) return TMVG_BAD_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return TMVG_NO_DEVICE;
    }
    tmvg_status st = TMVG_OK;
    unsigned char* s = noalloc_scratch(dev, &st);
    if (!s) return st;

    // A context on the stack: no workspace, flags and barrier in the scratch.
    Context c;
    c.device = dev;
    c.num_sms = std::min(sms, kNoAllocMaxCtas);
    c.stream = static_cast<cudaStream_t>(stream);
    c.dflags = reinterpret_cast<int*>(s + kNaOffErr);
    c.dbar = reinterpret_cast<unsigned*>(s + kNaOffBar);
    double* cand_key = reinterpret_cast<double*>(s + kNaOffKey);
    long long* cand_idx = reinterpret_cast<long long*>(s + kNaOffIdx);
    double* cand_rows = reinterpret_cast<double*>(s + kNaOffRows);
    double* diag_row = reinterpret_cast<double*>(s + kNaOffDiag);
    unsigned char* modes = s + kNaOffModes;

    // The array keeps the last call's contents: clear the error words.
    st = check_cuda(&c, cudaMemsetAsync(s, 0, 256, c.stream), "noalloc: clear");
    if (st) return st;
    {
        std::vector<unsigned char> hm((size_t)n, 0);
        leaf_modes(0, n, hm);
        st = check_cuda(&c, cudaMemcpyAsync(modes, hm.data(), (size_t)n, cudaMemcpyHostToDevice, c.stream),
                        "noalloc: modes");
        if (st) return st;
        st = check_cuda(&c, cudaStreamSynchronize(c.stream), "noalloc: modes sync");
        if (st) return st;
    }
    const int nbmax = panel_width<double>();
    cudaFuncSetAttribute(lu_panel_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    for (int64_t k = 0; k < n; k += nbmax) {
        const int nb = (int)std::min<int64_t>(nbmax, n - k);
        const int64_t m = n - k;
        const int G = (int)std::min<int64_t>(c.num_sms, ceil_div(m, kPanelThreads));
        const int rows_per_cta = (int)ceil_div(m, G);
        const size_t smem = (size_t)rows_per_cta * (nb + 1) * sizeof(double);
        st = check_cuda(&c, cudaMemsetAsync(c.dbar, 0, sizeof(unsigned), c.stream), "noalloc: barrier");
        if (st) return st;
        double* Ap = A;
        int64_t* Pp = P;
        const unsigned char* mp = modes + k;
        int64_t ldav = lda, nv = n, kv = k;
        int nbv = nb, rpc = rows_per_cta;
        unsigned* bar = c.dbar;
        int* err = c.dflags;
        void* args[] = {&Ap, &ldav, &nv, &kv, &nbv, &Pp, &mp, &rpc, &cand_key, &cand_idx,
                        &cand_rows, &diag_row, &bar, &err};
        st = check_cuda(&c,
                        cudaLaunchCooperativeKernel((const void*)lu_panel_kernel<double>, dim3(G),
                                                    dim3(kPanelThreads), args, smem, c.stream),
                        "noalloc: panel launch");
        if (st) return st;
        if (n > nb) {
            laswp_kernel<double><<<(unsigned)ceil_div(n, 128), 128, 0, c.stream>>>(A, lda, n, k, nb, P,
                                                                                  k, k + nb);
            st = check_cuda(&c, cudaGetLastError(), "noalloc: laswp launch");
            if (st) return st;
        }
        if (k + nb < n) {
            const int64_t rest = n - k - nb;
            st = tri_solve<double>(&c, nb, A + k + k * lda, 1, lda, false, true, rest,
                                   A + k + (k + nb) * lda, 1, lda, false);
            if (st) return st;
            st = gemm<double>(&c, rest, rest, nb, -1.0, Mat<const double>{A + (k + nb) + k * lda, 1, lda},
                              Mat<const double>{A + k + (k + nb) * lda, 1, lda}, 1.0,
                              Mat<double>{A + (k + nb) + (k + nb) * lda, 1, lda});
            if (st) return st;
        }
    }
    int code[2] = {0, 0};
    st = check_cuda(&c, cudaMemcpyAsync(code, c.dflags, sizeof(code), cudaMemcpyDeviceToHost, c.stream),
                    "noalloc: status");
    if (st) return st;
    st = check_cuda(&c, cudaStreamSynchronize(c.stream), "noalloc: sync");
    if (st) return st;
    if (code[0] == kDevTimeout) return TMVG_TIMEOUT;
    if (code[0] != kDevOk) return TMVG_CUDA_ERROR;
    return TMVG_OK;
}
