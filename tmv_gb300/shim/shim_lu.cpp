// shim_lu.cpp -- tmv::LU_Decompose (src/TMV_LUDecompose.cpp:514-559) and
// tmv::LU_LDivEq / LU_RDivEq (src/TMV_LUDiv.cpp:186-226, 370-411) and
// tmv::LU_Inverse (src/TMV_LUInverse.cpp:236-299) for every instantiation of
// TMV_LUDecompose.inst, TMV_LUDiv.inst and TMV_LUInverse.inst.  Real double
// problems go to the GPU (a rectangular LU_Decompose through a padded square
// factorisation, below); the other types run TMV's own CPU code.
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

static void gpu_lu_decompose(MatrixView<double> A, ptrdiff_t* P);

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
static void gpu_lu_decompose_rect(MatrixView<double> A, ptrdiff_t* P)
{
    const ptrdiff_t M = A.colsize(), N = A.rowsize();
    const ptrdiff_t R = std::min(M, N), S = std::max(M, N);
    if ((double)S * (double)S > 16.0 * (double)M * (double)N && S > 4096)
        throw Error("tmv::LU_Decompose: a " + std::to_string(M) + " x " + std::to_string(N) +
                    " matrix is too far from square for the GPU path");
    Matrix<double, ColMajor> Ap(S, S, 0.0);
    Ap.subMatrix(0, M, 0, N) = A;
    for (ptrdiff_t t = R; t < S; ++t) Ap(t, t) = 1.0;
    std::vector<ptrdiff_t> Pp(S);
    gpu_lu_decompose(Ap.view(), Pp.data());
    if (M > N)
        for (ptrdiff_t j = S - 1; j >= R; --j)
            if (Pp[j] != j) Ap.subMatrix(0, S, 0, N).swapRows(j, Pp[j]);
    A = Ap.subMatrix(0, M, 0, N);
    for (ptrdiff_t j = 0; j < R; ++j) P[j] = Pp[j];
}

static void gpu_lu_decompose(MatrixView<double> A, ptrdiff_t* P)
{
    using namespace tmvg_shim;
    if (A.colsize() != A.rowsize()) {
        if (A.colsize() > 0 && A.rowsize() > 0) gpu_lu_decompose_rect(A, P);
        return;
    }
    if (!dense_view(A)) {
        Matrix<double, ColMajor> At(A);
        gpu_lu_decompose(At.view(), P);
        A = At;
        return;
    }
    static_assert(sizeof(ptrdiff_t) == sizeof(int64_t), "LP64 pivots");
    check(tmvg_lu_decompose_f64_host(gpu(), A.colsize(), A.ptr(), A.stepi(), A.stepj(),
                                     reinterpret_cast<int64_t*>(P)),
          "tmv::LU_Decompose");
}

template <class T>
void LU_Decompose(MatrixView<T> A, ptrdiff_t* P)
{
    if constexpr (std::is_same<T, double>::value) gpu_lu_decompose(A, P);
    else TMVG_CPU_LU_Decompose(A, P);
}

static void gpu_lu_div(bool right, const GenMatrix<double>& LUx, const ptrdiff_t* P,
                       MatrixView<double> m)
{
    using namespace tmvg_shim;
    if (!(LUx.iscm() && !LUx.isconj())) {
        Matrix<double, ColMajor> LUc(LUx);
        gpu_lu_div(right, LUc, P, m);
        return;
    }
    if (!dense_view(m)) {
        Matrix<double, ColMajor> mt(m);
        gpu_lu_div(right, LUx, P, mt.view());
        m = mt;
        return;
    }
    const ptrdiff_t n = LUx.colsize();
    const int64_t* p = reinterpret_cast<const int64_t*>(P);
    tmvg_status s = right
        ? tmvg_lu_rdiveq_f64_host(gpu(), n, LUx.cptr(), LUx.stepj(), p, m.colsize(), m.ptr(),
                                  m.stepi(), m.stepj())
        : tmvg_lu_ldiveq_f64_host(gpu(), n, LUx.cptr(), LUx.stepj(), p, m.rowsize(), m.ptr(),
                                  m.stepi(), m.stepj());
    if (s == TMVG_SINGULAR) throw SingularUpperTriMatrix<double>(LUx.upperTri());
    check(s, right ? "tmv::LU_RDivEq" : "tmv::LU_LDivEq");
}

template <class T, class T1>
void LU_LDivEq(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> m)
{
    if constexpr (std::is_same<T, double>::value && std::is_same<T1, double>::value)
        gpu_lu_div(false, LUx, P, m);
    else
        TMVG_CPU_LU_LDivEq(LUx, P, m);
}

template <class T, class T1>
void LU_RDivEq(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> m)
{
    if constexpr (std::is_same<T, double>::value && std::is_same<T1, double>::value)
        gpu_lu_div(true, LUx, P, m);
    else
        TMVG_CPU_LU_RDivEq(LUx, P, m);
}

static void gpu_lu_inverse(const GenMatrix<double>& LUx, const ptrdiff_t* P, MatrixView<double> minv)
{
    using namespace tmvg_shim;
    if (!(LUx.iscm() && !LUx.isconj())) {
        Matrix<double, ColMajor> LUc(LUx);
        gpu_lu_inverse(LUc, P, minv);
        return;
    }
    if (!dense_view(minv)) {
        Matrix<double, ColMajor> mt(minv.colsize(), minv.rowsize());
        gpu_lu_inverse(LUx, P, mt.view());
        minv = mt;
        return;
    }
    tmvg_status s = tmvg_lu_inverse_f64_host(gpu(), LUx.colsize(), LUx.cptr(), LUx.stepj(),
                                             reinterpret_cast<const int64_t*>(P), minv.ptr(),
                                             minv.stepi(), minv.stepj());
    if (s == TMVG_SINGULAR) throw SingularUpperTriMatrix<double>(LUx.upperTri());
    check(s, "tmv::LU_Inverse");
}

template <class T, class T1>
void LU_Inverse(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> minv)
{
    if constexpr (std::is_same<T, double>::value && std::is_same<T1, double>::value)
        gpu_lu_inverse(LUx, P, minv);
    else
        TMVG_CPU_LU_Inverse(LUx, P, minv);
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
