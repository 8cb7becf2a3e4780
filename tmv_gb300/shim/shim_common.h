// shim_common.h -- shared pieces of the TMV drop-in: the process-wide GPU
// context and the names under which TMV's own CPU implementations of the
// replaced routines stay available for the types this library does not
// accelerate (float, int and complex instantiations).
//
// The drop-in is built by tmv_gb300/shim/Makefile from the TMV sources: every
// TMV translation unit is compiled unchanged except TMV_MultMM.cpp,
// TMV_LUDecompose.cpp, TMV_LUDiv.cpp and TMV_LUInverse.cpp, which are compiled with their entry
// points renamed to the TMVG_CPU_ names below; the shim translation units
// then define the original entry points for exactly the instantiation lists
// of TMV's .inst files.
#ifndef TMVG_SHIM_COMMON_H
#define TMVG_SHIM_COMMON_H

#include <new>
#include <string>
#include <type_traits>

#include "TMV.h"
#include "tmvg.h"

namespace tmv {

template <bool add, typename T, typename Ta, typename Tb>
void TMVG_CPU_MultMM(const T alpha, const GenMatrix<Ta>& A, const GenMatrix<Tb>& B,
                     MatrixView<T> C);
template <typename T>
void TMVG_CPU_LU_Decompose(MatrixView<T> A, ptrdiff_t* P);
template <typename T, typename T1>
void TMVG_CPU_LU_LDivEq(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> m);
template <typename T, typename T1>
void TMVG_CPU_LU_RDivEq(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> m);
template <typename T, typename T1>
void TMVG_CPU_LU_Inverse(const GenMatrix<T1>& LUx, const ptrdiff_t* P, MatrixView<T> minv);

namespace tmvg_shim {

// One context per process, on device $TMVG_DEVICE (default 0).  Every call
// counts one entry into the GPU path; with $TMVG_SHIM_STATS set the count is
// printed to stderr when the process exits ("tmvg drop-in: N GPU calls").
tmvg_handle gpu();

// TMV's error conventions (include/tmv/TMV_Base.h:502-648): allocation
// failures are std::bad_alloc, everything else a tmv::Error.
inline void check(tmvg_status s, const char* what)
{
    if (s == TMVG_OK) return;
    if (s == TMVG_OOM) throw std::bad_alloc();
    std::string msg = std::string(what) + ": " + tmvg_status_string(s) + " (" +
                      tmvg_last_error(gpu()) + ")";
    throw Error(msg);
}

// Views the C ABI takes directly: column- or row-major, non-conjugated.
template <typename T>
inline bool dense_view(const GenMatrix<T>& m)
{
    return !m.isconj() && (m.iscm() || m.isrm());
}

}  // namespace tmvg_shim
}  // namespace tmv

#endif
