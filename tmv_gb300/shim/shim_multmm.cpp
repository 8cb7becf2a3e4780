// shim_multmm.cpp -- tmv::MultMM<add,T,Ta,Tb> (src/TMV_MultMM.cpp:405-477)
// for every instantiation of src/TMV_MultMM.inst.  Real double and float
// products (all three operands of one type) go to the GPU
// (tmvg_multmm_f64_host / tmvg_multmm_f32_host: host views in, host views
// out, synchronous, as TMV's call is); the other types run TMV's own CPU code.
#include "shim_common.h"

namespace tmv {

namespace {

tmvg_status gpu_call(double alpha, bool add, const GenMatrix<double>& A, const GenMatrix<double>& B,
                     MatrixView<double> C)
{
    return tmvg_multmm_f64_host(tmvg_shim::gpu(), add ? 1 : 0, alpha, C.colsize(), C.rowsize(),
                                A.rowsize(), A.cptr(), A.stepi(), A.stepj(), B.cptr(), B.stepi(),
                                B.stepj(), C.ptr(), C.stepi(), C.stepj());
}

tmvg_status gpu_call(float alpha, bool add, const GenMatrix<float>& A, const GenMatrix<float>& B,
                     MatrixView<float> C)
{
    return tmvg_multmm_f32_host(tmvg_shim::gpu(), add ? 1 : 0, alpha, C.colsize(), C.rowsize(),
                                A.rowsize(), A.cptr(), A.stepi(), A.stepj(), B.cptr(), B.stepi(),
                                B.stepj(), C.ptr(), C.stepi(), C.stepj());
}

template <class T>
void gpu_multmm(bool add, T alpha, const GenMatrix<T>& A, const GenMatrix<T>& B, MatrixView<T> C)
{
    using namespace tmvg_shim;
    // Strided or conjugated views go through dense copies, as TMV's MultMM
    // does with its temporaries (src/TMV_MultMM.cpp:431-454).
    if (!dense_view(A)) {
        Matrix<T, ColMajor> At(A);
        gpu_multmm<T>(add, alpha, At, B, C);
        return;
    }
    if (!dense_view(B)) {
        Matrix<T, ColMajor> Bt(B);
        gpu_multmm<T>(add, alpha, A, Bt, C);
        return;
    }
    if (!dense_view(C)) {
        Matrix<T, ColMajor> Ct(C);
        gpu_multmm<T>(add, alpha, A, B, Ct.view());
        C = Ct;
        return;
    }
    check(gpu_call(alpha, add, A, B, C), "tmv::MultMM");
}

}  // namespace

template <bool add, class T, class Ta, class Tb>
void MultMM(const T alpha, const GenMatrix<Ta>& A, const GenMatrix<Tb>& B, MatrixView<T> C)
{
    if constexpr ((std::is_same<T, double>::value || std::is_same<T, float>::value) &&
                  std::is_same<Ta, T>::value && std::is_same<Tb, T>::value) {
        gpu_multmm<T>(add, alpha, A, B, C);
    } else {
        TMVG_CPU_MultMM<add>(alpha, A, B, C);
    }
}

#define InstFile "TMV_MultMM.inst"
#include "TMV_Inst.h"
#undef InstFile

}  // namespace tmv
