// shim_lu.cpp -- tmv::LU_Decompose (src/TMV_LUDecompose.cpp:514-559) and
// tmv::LU_LDivEq / LU_RDivEq (src/TMV_LUDiv.cpp:186-226, 370-411) and
// tmv::LU_Inverse (src/TMV_LUInverse.cpp:236-299) for every instantiation of
// TMV_LUDecompose.inst, TMV_LUDiv.inst and TMV_LUInverse.inst.  double,
// float and std::complex<double> problems go to the GPU (a rectangular
// LU_Decompose through a padded square factorisation, below), with the
// factors and the right-hand sides of one type; the other instantiations
// (integer, complex<float>, and divisions that mix a real factor with complex
// right-hand sides) run TMV's own CPU code.
#include <complex>
#include <string>
#include <vector>

#include "TMV_LUDiv.h"
#include "shim_common.h"
#include "tmv/TMV_LUD.h"
#include "tmv/TMV_TriDiv.h"
#include "tmv/TMV_TriMatrix.h"

#ifdef INST_INT
#undef INST_INT
#endif

namespace tmv {

namespace {

static_assert(sizeof(ptrdiff_t) == sizeof(int64_t), "LP64 pivots");

// The C ABI's host-view entry points for one element type.
template <class T>
struct Gpu;

template <>
struct Gpu<double> {
    static tmvg_status lu(tmvg_handle h, int64_t n, double* A, int64_t si, int64_t sj, int64_t* P)
    {
        return tmvg_lu_decompose_f64_host(h, n, A, si, sj, P);
    }
    static tmvg_status ldiv(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                            int64_t o, double* B, int64_t si, int64_t sj)
    {
        return tmvg_lu_ldiveq_f64_host(h, n, LU, lda, P, o, B, si, sj);
    }
    static tmvg_status rdiv(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                            int64_t o, double* B, int64_t si, int64_t sj)
    {
        return tmvg_lu_rdiveq_f64_host(h, n, LU, lda, P, o, B, si, sj);
    }
    static tmvg_status inv(tmvg_handle h, int64_t n, const double* LU, int64_t lda, const int64_t* P,
                           double* M, int64_t si, int64_t sj)
    {
        return tmvg_lu_inverse_f64_host(h, n, LU, lda, P, M, si, sj);
    }
};

template <>
struct Gpu<float> {
    static tmvg_status lu(tmvg_handle h, int64_t n, float* A, int64_t si, int64_t sj, int64_t* P)
    {
        return tmvg_lu_decompose_f32_host(h, n, A, si, sj, P);
    }
    static tmvg_status ldiv(tmvg_handle h, int64_t n, const float* LU, int64_t lda, const int64_t* P,
                            int64_t o, float* B, int64_t si, int64_t sj)
    {
        return tmvg_lu_ldiveq_f32_host(h, n, LU, lda, P, o, B, si, sj);
    }
    static tmvg_status rdiv(tmvg_handle h, int64_t n, const float* LU, int64_t lda, const int64_t* P,
                            int64_t o, float* B, int64_t si, int64_t sj)
    {
        return tmvg_lu_rdiveq_f32_host(h, n, LU, lda, P, o, B, si, sj);
    }
    static tmvg_status inv(tmvg_handle h, int64_t n, const float* LU, int64_t lda, const int64_t* P,
                           float* M, int64_t si, int64_t sj)
    {
        return tmvg_lu_inverse_f32_host(h, n, LU, lda, P, M, si, sj);
    }
};

// std::complex<double> is two doubles (real, imaginary): the C ABI's
// interleaved layout; strides stay in complex elements.
template <>
struct Gpu<std::complex<double> > {
    using Z = std::complex<double>;
    static double* d(Z* p) { return reinterpret_cast<double*>(p); }
    static const double* d(const Z* p) { return reinterpret_cast<const double*>(p); }
    static tmvg_status lu(tmvg_handle h, int64_t n, Z* A, int64_t si, int64_t sj, int64_t* P)
    {
        return tmvg_lu_decompose_z64_host(h, n, d(A), si, sj, P);
    }
    static tmvg_status ldiv(tmvg_handle h, int64_t n, const Z* LU, int64_t lda, const int64_t* P,
                            int64_t o, Z* B, int64_t si, int64_t sj)
    {
        return tmvg_lu_ldiveq_z64_host(h, n, d(LU), lda, P, o, d(B), si, sj);
    }
    static tmvg_status rdiv(tmvg_handle h, int64_t n, const Z* LU, int64_t lda, const int64_t* P,
                            int64_t o, Z* B, int64_t si, int64_t sj)
    {
        return tmvg_lu_rdiveq_z64_host(h, n, d(LU), lda, P, o, d(B), si, sj);
    }
    static tmvg_status inv(tmvg_handle h, int64_t n, const Z* LU, int64_t lda, const int64_t* P,
                           Z* M, int64_t si, int64_t sj)
    {
        return tmvg_lu_inverse_z64_host(h, n, d(LU), lda, P, d(M), si, sj);
    }
};

template <class T>
constexpr bool on_gpu = std::is_same<T, double>::value || std::is_same<T, float>::value ||
                        std::is_same<T, std::complex<double> >::value;

template <class T>
void gpu_lu_decompose(MatrixView<T> A, ptrdiff_t* P);

// LU_Decompose of an M x N matrix, M != N (TMV factors its R = min(M,N)
// columns, src/TMV_LUDecompose.cpp:217-235, and writes R interchanges).  The
// GPU factors the S x S matrix, S = max(M,N), that holds A in its top-left
// block, the identity in its trailing (S-R) x (S-R) block and zeros
// elsewhere.  Steps j < R see exactly TMV's columns (the padding adds no
// candidate larger than a real one: its entries in those columns are zero),
// so the first R pivots and A's factors are TMV's.  A wide A is then done
// (steps j >= R touch only padding rows).  For a tall A the steps j >= R may
// interchange rows >= R of the factored columns, so those interchanges are
// undone on A's columns, last first.  Shapes far from square would pad to
// far more memory than A holds: above 16 M N padded elements (and S > 4096)
// the call throws tmv::Error rather than leave the GPU.
template <class T>
void gpu_lu_decompose_rect(MatrixView<T> A, ptrdiff_t* P)
{
    const ptrdiff_t M = A.colsize(), N = A.rowsize();
    const ptrdiff_t R = std::min(M, N), S = std::max(M, N);
    if ((double)S * (double)S > 16.0 * (double)M * (double)N && S > 4096)
        throw Error("tmv::LU_Decompose: a " + std::to_string(M) + " x " + std::to_string(N) +
                    " matrix is too far from square for the GPU path");
    Matrix<T, ColMajor> Ap(S, S, T(0));
    Ap.subMatrix(0, M, 0, N) = A;
    for (ptrdiff_t t = R; t < S; ++t) Ap(t, t) = T(1);
    std::vector<ptrdiff_t> Pp(S);
    gpu_lu_decompose<T>(Ap.view(), Pp.data());
    if (M > N)
        for (ptrdiff_t j = S - 1; j >= R; --j)
            if (Pp[j] != j) Ap.subMatrix(0, S, 0, N).swapRows(j, Pp[j]);
    A = Ap.subMatrix(0, M, 0, N);
    for (ptrdiff_t j = 0; j < R; ++j) P[j] = Pp[j];
}

template <class T>
void gpu_lu_decompose(MatrixView<T> A, ptrdiff_t* P)
{
    using namespace tmvg_shim;
    if (A.colsize() != A.rowsize()) {
        if (A.colsize() > 0 && A.rowsize() > 0) gpu_lu_decompose_rect<T>(A, P);
        return;
    }
    if (!dense_view(A)) {
        Matrix<T, ColMajor> At(A);
        gpu_lu_decompose<T>(At.view(), P);
        A = At;
        return;
    }
    check(Gpu<T>::lu(gpu(), A.colsize(), A.ptr(), A.stepi(), A.stepj(), reinterpret_cast<int64_t*>(P)),
          "tmv::LU_Decompose");
}

template <class T>
void gpu_lu_div(bool right, const GenMatrix<T>& LUx, const ptrdiff_t* P, MatrixView<T> m)
{
    using namespace tmvg_shim;
    if (!(LUx.iscm() && !LUx.isconj())) {
        Matrix<T, ColMajor> LUc(LUx);
        gpu_lu_div<T>(right, LUc, P, m);
        return;
    }
    if (!dense_view(m)) {
        Matrix<T, ColMajor> mt(m);
        gpu_lu_div<T>(right, LUx, P, mt.view());
        m = mt;
        return;
    }
    const ptrdiff_t n = LUx.colsize();
    const int64_t* p = reinterpret_cast<const int64_t*>(P);
    tmvg_status s = right ? Gpu<T>::rdiv(gpu(), n, LUx.cptr(), LUx.stepj(), p, m.colsize(), m.ptr(),
                                         m.stepi(), m.stepj())
                          : Gpu<T>::ldiv(gpu(), n, LUx.cptr(), LUx.stepj(), p, m.rowsize(), m.ptr(),
                                         m.stepi(), m.stepj());
    if (s == TMVG_SINGULAR) throw SingularUpperTriMatrix<T>(LUx.upperTri());
    check(s, right ? "tmv::LU_RDivEq" : "tmv::LU_LDivEq");
}

template <class T>
void gpu_lu_inverse(const GenMatrix<T>& LUx, const ptrdiff_t* P, MatrixView<T> minv)
{
    using namespace tmvg_shim;
    if (!(LUx.iscm() && !LUx.isconj())) {
        Matrix<T, ColMajor> LUc(LUx);
        gpu_lu_inverse<T>(LUc, P, minv);
        return;
    }
    if (!dense_view(minv)) {
        Matrix<T, ColMajor> mt(minv.colsize(), minv.rowsize());
        gpu_lu_inverse<T>(LUx, P, mt.view());
        minv = mt;
        return;
    }
    tmvg_status s = Gpu<T>::inv(gpu(), LUx.colsize(), LUx.cptr(), LUx.stepj(),
                                reinterpret_cast<const int64_t*>(P), minv.ptr(), minv.stepi(), minv.stepj());
    if (s == TMVG_SINGULAR) throw SingularUpperTriMatrix<T>(LUx.upperTri());
    check(s, "tmv::LU_Inverse");
}

}  // namespace

template <class T>
void LU_Decompose(MatrixView<T> A, ptrdiff_t* P)
{
    if constexpr (on_gpu<T>) gpu_lu_decompose<T>(A, P);
    else TMVG_CPU_LU_Decompose(A, P);
}

template <class T, class T1>
void LU_LDivEq(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> m)
{
    if constexpr (std::is_same<T, T1>::value && on_gpu<T>) gpu_lu_div<T>(false, LUx, P, m);
    else TMVG_CPU_LU_LDivEq(LUx, P, m);
}

template <class T, class T1>
void LU_RDivEq(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> m)
{
    if constexpr (std::is_same<T, T1>::value && on_gpu<T>) gpu_lu_div<T>(true, LUx, P, m);
    else TMVG_CPU_LU_RDivEq(LUx, P, m);
}

template <class T, class T1>
void LU_Inverse(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> minv)
{
    if constexpr (std::is_same<T, T1>::value && on_gpu<T>) gpu_lu_inverse<T>(LUx, P, minv);
    else TMVG_CPU_LU_Inverse(LUx, P, minv);
}

#define InstFile "TMV_LUDecompose.inst"
#include "TMV_Inst.h"
#undef InstFile

#define InstFile "TMV_LUDiv.inst"
#include "TMV_Inst.h"
#undef InstFile

#define InstFile "TMV_LUInverse.inst"
#include "TMV_Inst.h"
#undef InstFile

}  // namespace tmv
