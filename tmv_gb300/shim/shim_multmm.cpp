// shim_multmm.cpp -- tmv::MultMM<add,T,Ta,Tb> (src/TMV_MultMM.cpp:405-477)
// for every instantiation of src/TMV_MultMM.inst.  Real double products go to
// the GPU (tmvg_multmm_f64_host: host views in, host views out, synchronous,
// as TMV's call is); the other types run TMV's own CPU code.
#include "shim_common.h"

namespace tmv {

static void gpu_multmm(bool add, double alpha, const GenMatrix<double>& A,
                       const GenMatrix<double>& B, MatrixView<double> C)
{
    using namespace tmvg_shim;
    // Strided or conjugated views go through dense copies, as TMV's MultMM
    // does with its temporaries (src/TMV_MultMM.cpp:431-454).
    if (!dense_view(A)) {
        Matrix<double, ColMajor> At(A);
        gpu_multmm(add, alpha, At, B, C);
        return;
    }
    if (!dense_view(B)) {
        Matrix<double, ColMajor> Bt(B);
        gpu_multmm(add, alpha, A, Bt, C);
        return;
    }
    if (!dense_view(C)) {
        Matrix<double, ColMajor> Ct(C);
        gpu_multmm(add, alpha, A, B, Ct.view());
        C = Ct;
        return;
    }
    check(tmvg_multmm_f64_host(gpu(), add ? 1 : 0, alpha, C.colsize(), C.rowsize(), A.rowsize(),
                               A.cptr(), A.stepi(), A.stepj(), B.cptr(), B.stepi(), B.stepj(),
                               C.ptr(), C.stepi(), C.stepj()),
          "tmv::MultMM");
}

template <bool add, class T, class Ta, class Tb>
void MultMM(const T alpha, const GenMatrix<Ta>& A, const GenMatrix<Tb>& B, MatrixView<T> C)
{
    if constexpr (std::is_same<T, double>::value && std::is_same<Ta, double>::value &&
                  std::is_same<Tb, double>::value) {
        gpu_multmm(add, alpha, A, B, C);
    } else {
        TMVG_CPU_MultMM<add>(alpha, A, B, C);
    }
}

#define InstFile "TMV_MultMM.inst"
#include "TMV_Inst.h"
#undef InstFile

}  // namespace tmv
