// ref_capi.cpp -- extern "C" binding of TMV 0.76's own public surface.
//
// TEST INFRASTRUCTURE ONLY.  This file is compiled together with the TMV
// reference sources into oracle/_ref/libtmvref.so by oracle/Makefile, and is
// loaded only by the fixture generator (tests/golden/make_golden.py) and by the
// CPU tests that pin the C restatement (oracle/tmv_oracle.c) against TMV itself.
// Nothing in the product links it.
//
// Every entry point reaches TMV through the calls a TMV user (or TMV's own
// LUDiv) makes:
//   tmvref_multmm        C = alpha*A*B / C += alpha*A*B  (tmv::Matrix expression
//                        surface -> ProdMM::assignToM -> MultMM<add>,
//                        include/tmv/TMV_MatrixArith.h:701-810, src/TMV_MultMM.cpp:405)
//   tmvref_lu_decompose  LU_Decompose(MatrixView<T>, ptrdiff_t*) (src/TMV_LUDecompose.cpp:514)
//   tmvref_lu_ldiveq     LU_LDivEq (src/TMV_LUDiv.cpp:186)
//   tmvref_lu_rdiveq     LU_RDivEq (src/TMV_LUDiv.cpp:370)
//   tmvref_divide        m.divideUsing(tmv::LU); m.saveDiv(); X = B/m (src/TMV_LUD.cpp:74-120)
//   tmvref_rdivide       X = B % m (LUDiv::doRDiv, src/TMV_LUD.cpp:122-130)
//   tmvref_det           m.det(), m.logDet(&s) (src/TMV_LUD.cpp:132-190)
//   tmvref_batched_divide  one B_i/A_i per system, OpenMP over systems.
//   tmvref_band_lu_decompose, tmvref_band_lu_ldiveq, tmvref_band_lu_rdiveq
//                        LU_Decompose(BandMatrixView<T>, ptrdiff_t*, ptrdiff_t)
//                        (src/TMV_BandLUDecompose.cpp:383) and LU_LDivEq /
//                        LU_RDivEq on band factors (src/TMV_BandLUDiv.cpp:
//                        811-851; m row-major for RDivEq) over TMV's
//                        column-major band storage; tmvref_band_batched_solve
//                        both over a batch, OpenMP over systems.
//   tmvref_lu_decompose_z, tmvref_lu_ldiveq_z, tmvref_lu_rdiveq_z, tmvref_det_z,
//   tmvref_inverse_z, tmvref_multmm_z
//                        the same for std::complex<double> (column-major,
//                        interleaved entries).
//
// Status: 0 ok, 1 tmv::Singular thrown, 2 other tmv::Error, 3 other exception.

#include "TMV.h"
#include "TMV_Band.h"
#include "TMV_BandLUDiv.h"
#include "TMV_LUDiv.h"
#include <omp.h>
#include <algorithm>
#include <cstring>

namespace {

template <class F>
int guarded(F f)
{
    try {
        f();
    } catch (tmv::Singular&) {
        return 1;
    } catch (tmv::Error&) {
        return 2;
    } catch (...) {
        return 3;
    }
    return 0;
}

tmv::StorageType stor_of(int rowmajor)
{ return rowmajor ? tmv::RowMajor : tmv::ColMajor; }

}  // namespace

extern "C" {

int tmvref_version(void) { return 76; }

void tmvref_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

int tmvref_max_threads(void) { return omp_get_max_threads(); }

int tmvref_multmm(int add, double alpha, ptrdiff_t m, ptrdiff_t n, ptrdiff_t k,
                  const double* A, ptrdiff_t sAi, ptrdiff_t sAj,
                  const double* B, ptrdiff_t sBi, ptrdiff_t sBj,
                  double* C, ptrdiff_t sCi, ptrdiff_t sCj)
{
    return guarded([&] {
        tmv::ConstMatrixView<double> Av = tmv::MatrixViewOf(A, m, k, sAi, sAj);
        tmv::ConstMatrixView<double> Bv = tmv::MatrixViewOf(B, k, n, sBi, sBj);
        tmv::MatrixView<double> Cv = tmv::MatrixViewOf(C, m, n, sCi, sCj);
        if (add) Cv += alpha * Av * Bv;
        else Cv = alpha * Av * Bv;
    });
}

int tmvref_lu_decompose(ptrdiff_t n, double* A, ptrdiff_t sAi, ptrdiff_t sAj,
                        ptrdiff_t* P)
{
    return guarded([&] {
        tmv::MatrixView<double> Av = tmv::MatrixViewOf(A, n, n, sAi, sAj);
        tmv::LU_Decompose(Av, P);
    });
}

int tmvref_lu_decompose_z(ptrdiff_t n, double* A, ptrdiff_t lda, ptrdiff_t* P)
{
    return guarded([&] {
        typedef std::complex<double> Z;
        tmv::MatrixView<Z> Av = tmv::MatrixViewOf(reinterpret_cast<Z*>(A), n, n, 1, lda);
        tmv::LU_Decompose(Av, P);
    });
}

int tmvref_lu_ldiveq_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                       ptrdiff_t nrhs, double* B, ptrdiff_t ldb)
{
    return guarded([&] {
        typedef std::complex<double> Z;
        tmv::ConstMatrixView<Z> LUv = tmv::MatrixViewOf(reinterpret_cast<const Z*>(LU), n, n, 1, lda);
        tmv::MatrixView<Z> Bv = tmv::MatrixViewOf(reinterpret_cast<Z*>(B), n, nrhs, 1, ldb);
        tmv::LU_LDivEq(LUv, P, Bv);
    });
}

int tmvref_lu_rdiveq_z(ptrdiff_t n, const double* LU, ptrdiff_t lda, const ptrdiff_t* P,
                       ptrdiff_t nrows, double* B, ptrdiff_t ldb)
{
    return guarded([&] {
        typedef std::complex<double> Z;
        tmv::ConstMatrixView<Z> LUv = tmv::MatrixViewOf(reinterpret_cast<const Z*>(LU), n, n, 1, lda);
        tmv::MatrixView<Z> Bv = tmv::MatrixViewOf(reinterpret_cast<Z*>(B), nrows, n, 1, ldb);
        tmv::LU_RDivEq(LUv, P, Bv);
    });
}

// det and logDet of a complex matrix through LUDiv (src/TMV_LUD.cpp:132-156)
int tmvref_det_z(ptrdiff_t n, const double* A, double* det, double* logdet, double* sign)
{
    return guarded([&] {
        typedef std::complex<double> Z;
        tmv::Matrix<Z, tmv::ColMajor> m(n, n);
        std::memcpy(m.ptr(), A, sizeof(Z) * n * n);
        m.divideUsing(tmv::LU);
        const Z d = m.det();
        Z s;
        *logdet = m.logDet(&s);
        det[0] = d.real();
        det[1] = d.imag();
        sign[0] = s.real();
        sign[1] = s.imag();
    });
}

// Band LU over TMV's column-major band storage: element (i,j) at a[i + j*ldab]
// for j-hu <= i <= j+lo, hu = min(lo+hi, n-1).  The fill diagonals hi+1..hu
// are zeroed first, as BandLUDiv's copy of A into its wider band leaves them.
// algo 0 factors the column-major view (NonLapBandLU_Decompose); algo 1
// (lo = hi = 1) copies the matrix into the diagonal-major storage BandLUDiv
// gives a tridiagonal matrix, so that TMV runs NonLapTriDiagLU_Decompose and
// the row-oriented upper solve, and copies the factors back.
static void band_zero_fill(ptrdiff_t n, ptrdiff_t hi, ptrdiff_t hu, double* a, ptrdiff_t ldab)
{
    for (ptrdiff_t j = 0; j < n; ++j)
        for (ptrdiff_t d = hi + 1; d <= hu; ++d)
            if (j - d >= 0) a[(j - d) + j * ldab] = 0.0;
}

static void band_to_dm(ptrdiff_t n, ptrdiff_t hu, const double* a, ptrdiff_t ldab,
                       tmv::BandMatrix<double, tmv::DiagMajor>& D)
{
    for (ptrdiff_t j = 0; j < n; ++j)
        for (ptrdiff_t i = std::max<ptrdiff_t>(0, j - hu); i <= std::min(n - 1, j + 1); ++i)
            D(i, j) = a[i + j * ldab];
}

int tmvref_band_lu_decompose(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, double* a,
                             ptrdiff_t ldab, ptrdiff_t* P)
{
    return guarded([&] {
        if (n == 0) return;
        const ptrdiff_t hu = std::min(lo + hi, n - 1);
        band_zero_fill(n, hi, hu, a, ldab);
        if (algo == 1) {
            tmv::BandMatrix<double, tmv::DiagMajor> D(n, n, 1, hu, 0.0);
            band_to_dm(n, hu, a, ldab, D);
            tmv::LU_Decompose(D.view(), P, hi);
            for (ptrdiff_t j = 0; j < n; ++j)
                for (ptrdiff_t i = std::max<ptrdiff_t>(0, j - hu); i <= std::min(n - 1, j + 1); ++i)
                    a[i + j * ldab] = D(i, j);
            return;
        }
        tmv::BandMatrixView<double> A(a, n, n, lo, hu, 1, ldab, ldab + 1, tmv::NonConj);
        tmv::LU_Decompose(A, P, hi);
    });
}

int tmvref_band_lu_ldiveq(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, const double* lu,
                          ptrdiff_t ldab, const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                          ptrdiff_t ldb)
{
    return guarded([&] {
        if (n == 0 || nrhs == 0) return;
        const ptrdiff_t hu = std::min(lo + hi, n - 1);
        tmv::MatrixView<double> Bv = tmv::MatrixViewOf(B, n, nrhs, 1, ldb);
        if (algo == 1) {
            tmv::BandMatrix<double, tmv::DiagMajor> D(n, n, 1, hu, 0.0);
            band_to_dm(n, hu, lu, ldab, D);
            tmv::LU_LDivEq(D, P, Bv);
            return;
        }
        tmv::ConstBandMatrixView<double> LU(lu, n, n, lo, hu, 1, ldab, ldab + 1, tmv::NonConj);
        tmv::LU_LDivEq(LU, P, Bv);
    });
}

int tmvref_band_lu_rdiveq(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo, const double* lu,
                          ptrdiff_t ldab, const ptrdiff_t* P, ptrdiff_t nrhs, double* B,
                          ptrdiff_t ldb)
{
    return guarded([&] {
        if (n == 0 || nrhs == 0) return;
        const ptrdiff_t hu = std::min(lo + hi, n - 1);
        tmv::MatrixView<double> Mv = tmv::MatrixViewOf(B, nrhs, n, ldb, 1);
        if (algo == 1) {
            tmv::BandMatrix<double, tmv::DiagMajor> D(n, n, 1, hu, 0.0);
            band_to_dm(n, hu, lu, ldab, D);
            tmv::LU_RDivEq(D, P, Mv);
            return;
        }
        tmv::ConstBandMatrixView<double> LU(lu, n, n, lo, hu, 1, ldab, ldab + 1, tmv::NonConj);
        tmv::LU_RDivEq(LU, P, Mv);
    });
}

// B /= A for a tmv::BandMatrix A (lo, hi; column-major storage), through
// BandLUDiv as TMV's division operators run it (src/TMV_BandLUD.cpp:85-146,
// 217-222): A's band given in the layout above with hu = hi (no fill slots
// needed), B n x nrhs column-major.
int tmvref_band_divide(ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, const double* a, ptrdiff_t ldab,
                       ptrdiff_t nrhs, double* B, ptrdiff_t ldb)
{
    return guarded([&] {
        if (n == 0 || nrhs == 0) return;
        tmv::BandMatrix<double> A(n, n, lo, hi, 0.0);
        for (ptrdiff_t j = 0; j < n; ++j)
            for (ptrdiff_t i = std::max<ptrdiff_t>(0, j - hi); i <= std::min(n - 1, j + lo); ++i)
                A(i, j) = a[i + j * ldab];
        tmv::MatrixView<double> Bv = tmv::MatrixViewOf(B, n, nrhs, 1, ldb);
        Bv /= A;
    });
}

// The batched band workload through TMV, OpenMP over systems.
int tmvref_band_batched_solve(ptrdiff_t count, ptrdiff_t n, ptrdiff_t lo, ptrdiff_t hi, int algo,
                              double* ab, ptrdiff_t ldab, ptrdiff_t sab, ptrdiff_t* P, ptrdiff_t sp,
                              ptrdiff_t nrhs, double* B, ptrdiff_t ldb, ptrdiff_t sb, int* status)
{
#pragma omp parallel for schedule(static)
    for (ptrdiff_t s = 0; s < count; ++s) {
        int rc = tmvref_band_lu_decompose(n, lo, hi, algo, ab + s * sab, ldab, P + s * sp);
        if (rc == 0)
            rc = tmvref_band_lu_ldiveq(n, lo, hi, algo, ab + s * sab, ldab, P + s * sp, nrhs, B + s * sb, ldb);
        status[s] = rc;
    }
    return 0;
}

int tmvref_lu_ldiveq(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                     const ptrdiff_t* P, ptrdiff_t nrhs,
                     double* B, ptrdiff_t sBi, ptrdiff_t sBj)
{
    return guarded([&] {
        tmv::ConstMatrixView<double> LUv = tmv::MatrixViewOf(LU, n, n, 1, lda);
        tmv::MatrixView<double> Bv = tmv::MatrixViewOf(B, n, nrhs, sBi, sBj);
        tmv::LU_LDivEq(LUv, P, Bv);
    });
}

int tmvref_lu_rdiveq(ptrdiff_t n, const double* LU, ptrdiff_t lda,
                     const ptrdiff_t* P, ptrdiff_t nrows,
                     double* B, ptrdiff_t sBi, ptrdiff_t sBj)
{
    return guarded([&] {
        tmv::ConstMatrixView<double> LUv = tmv::MatrixViewOf(LU, n, n, 1, lda);
        tmv::MatrixView<double> Bv = tmv::MatrixViewOf(B, nrows, n, sBi, sBj);
        tmv::LU_RDivEq(LUv, P, Bv);
    });
}

// A: n x n, storage rowmajor?RM:CM (dense).  B, X: n x nrhs column-major.
// LU_out (n*n, the stored factor in LUDiv's own storage order, i.e. the
// factor of A for column-major input and of A^T for row-major input) and
// P_out (n) may be null.
int tmvref_divide(ptrdiff_t n, int rowmajor, const double* A, ptrdiff_t nrhs,
                  const double* B, double* X, double* LU_out, ptrdiff_t* P_out)
{
    return guarded([&] {
        if (rowmajor) {
            tmv::Matrix<double, tmv::RowMajor> m(
                tmv::MatrixViewOf(A, n, n, tmv::RowMajor));
            m.divideUsing(tmv::LU);
            m.saveDiv();
            m.setDiv();
            tmv::Matrix<double, tmv::ColMajor> Bm(
                tmv::MatrixViewOf(B, n, nrhs, tmv::ColMajor));
            tmv::MatrixViewOf(X, n, nrhs, tmv::ColMajor) = Bm / m;
            if (LU_out) tmv::MatrixViewOf(LU_out, n, n, tmv::ColMajor) = m.lud().getLU();
            if (P_out) std::memcpy(P_out, m.lud().getP().getValues(), n * sizeof(ptrdiff_t));
        } else {
            tmv::Matrix<double, tmv::ColMajor> m(
                tmv::MatrixViewOf(A, n, n, tmv::ColMajor));
            m.divideUsing(tmv::LU);
            m.saveDiv();
            m.setDiv();
            tmv::Matrix<double, tmv::ColMajor> Bm(
                tmv::MatrixViewOf(B, n, nrhs, tmv::ColMajor));
            tmv::MatrixViewOf(X, n, nrhs, tmv::ColMajor) = Bm / m;
            if (LU_out) tmv::MatrixViewOf(LU_out, n, n, tmv::ColMajor) = m.lud().getLU();
            if (P_out) std::memcpy(P_out, m.lud().getP().getValues(), n * sizeof(ptrdiff_t));
        }
    });
}

// X = W % A  (X A = W): W, X are nrows x n column-major, A n x n column-major.
int tmvref_rdivide(ptrdiff_t n, const double* A, ptrdiff_t nrows,
                   const double* W, double* X)
{
    return guarded([&] {
        tmv::Matrix<double, tmv::ColMajor> m(
            tmv::MatrixViewOf(A, n, n, tmv::ColMajor));
        m.divideUsing(tmv::LU);
        m.saveDiv();
        tmv::Matrix<double, tmv::ColMajor> Wm(
            tmv::MatrixViewOf(W, nrows, n, tmv::ColMajor));
        tmv::MatrixViewOf(X, nrows, n, tmv::ColMajor) = Wm % m;
    });
}

int tmvref_det(ptrdiff_t n, const double* A, double* det, double* logdet,
               double* sign)
{
    return guarded([&] {
        tmv::Matrix<double, tmv::ColMajor> m(
            tmv::MatrixViewOf(A, n, n, tmv::ColMajor));
        m.divideUsing(tmv::LU);
        m.saveDiv();
        *det = m.det();
        double s = 0;
        *logdet = m.logDet(&s);
        *sign = s;
    });
}

int tmvref_multmv(int add, double alpha, ptrdiff_t m, ptrdiff_t n, const double* A,
                  ptrdiff_t sAi, ptrdiff_t sAj, const double* x, ptrdiff_t incx, double* y,
                  ptrdiff_t incy)
{
    // y = alpha*A*x / y += alpha*A*x on views (MultMV<add>)
    return guarded([&] {
        tmv::ConstMatrixView<double> Av = tmv::MatrixViewOf(A, m, n, sAi, sAj);
        tmv::ConstVectorView<double> xv = tmv::VectorViewOf(x, n, incx);
        tmv::VectorView<double> yv = tmv::VectorViewOf(y, m, incy);
        if (add) yv += alpha * Av * xv;
        else yv = alpha * Av * xv;
    });
}

int tmvref_tri_ldiveq(int upper, int unitdiag, ptrdiff_t n, const double* T, ptrdiff_t tsi,
                      ptrdiff_t tsj, ptrdiff_t nrhs, double* B, ptrdiff_t bsi, ptrdiff_t bsj)
{
    // m /= U or m /= L (TriLDivEq) on views
    return guarded([&] {
        tmv::ConstMatrixView<double> Tv = tmv::MatrixViewOf(T, n, n, tsi, tsj);
        tmv::MatrixView<double> Bv = tmv::MatrixViewOf(B, n, nrhs, bsi, bsj);
        const tmv::DiagType dt = unitdiag ? tmv::UnitDiag : tmv::NonUnitDiag;
        if (upper) Bv /= Tv.upperTri(dt);
        else Bv /= Tv.lowerTri(dt);
    });
}

// C = alpha A B / C += alpha A B for complex views (the same expression
// surface as tmvref_multmm)
int tmvref_multmm_z(int add, const double* alpha, ptrdiff_t m, ptrdiff_t n, ptrdiff_t k,
                    const double* A, ptrdiff_t sAi, ptrdiff_t sAj, const double* B, ptrdiff_t sBi,
                    ptrdiff_t sBj, double* C, ptrdiff_t sCi, ptrdiff_t sCj)
{
    return guarded([&] {
        typedef std::complex<double> Z;
        const Z al(alpha[0], alpha[1]);
        tmv::ConstMatrixView<Z> Av = tmv::MatrixViewOf(reinterpret_cast<const Z*>(A), m, k, sAi, sAj);
        tmv::ConstMatrixView<Z> Bv = tmv::MatrixViewOf(reinterpret_cast<const Z*>(B), k, n, sBi, sBj);
        tmv::MatrixView<Z> Cv = tmv::MatrixViewOf(reinterpret_cast<Z*>(C), m, n, sCi, sCj);
        if (add) Cv += al * Av * Bv;
        else Cv = al * Av * Bv;
    });
}

// m.inverse() of a complex matrix (LUDiv::doMakeInverse -> LU_Inverse)
int tmvref_inverse_z(ptrdiff_t n, const double* A, double* minv)
{
    return guarded([&] {
        typedef std::complex<double> Z;
        tmv::Matrix<Z, tmv::ColMajor> m(n, n);
        std::memcpy(m.ptr(), A, sizeof(Z) * n * n);
        m.divideUsing(tmv::LU);
        tmv::MatrixViewOf(reinterpret_cast<Z*>(minv), n, n, tmv::ColMajor) = m.inverse();
    });
}

int tmvref_inverse(ptrdiff_t n, const double* A, double* minv, double* ata, int* singular)
{
    // m.inverse() (LUDiv::doMakeInverse -> LU_Inverse), m.makeInverseATA()
    // and m.isSingular() on an LU-divided copy of A
    return guarded([&] {
        tmv::Matrix<double, tmv::ColMajor> m(
            tmv::MatrixViewOf(A, n, n, tmv::ColMajor));
        m.divideUsing(tmv::LU);
        m.saveDiv();
        m.setDiv();
        if (singular) *singular = m.isSingular() ? 1 : 0;
        if (minv) tmv::MatrixViewOf(minv, n, n, tmv::ColMajor) = m.inverse();
        if (ata) {
            tmv::Matrix<double, tmv::ColMajor> t(n, n);
            m.makeInverseATA(t);
            tmv::MatrixViewOf(ata, n, n, tmv::ColMajor) = t;
        }
    });
}

// Ragged batch: system i has order n[i], nrhs[i] right-hand sides, A_i at
// A + a_off[i] (column-major n_i x n_i), B_i at B + b_off[i] (column-major
// n_i x nrhs_i).  X_i = B_i / A_i is written over B_i.  status[i] per system.
int tmvref_batched_divide(ptrdiff_t count, const ptrdiff_t* n, const ptrdiff_t* nrhs,
                          const ptrdiff_t* a_off, const ptrdiff_t* b_off,
                          const double* A, double* B, int* status)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (ptrdiff_t i = 0; i < count; ++i) {
        const ptrdiff_t ni = n[i], ri = nrhs[i];
        status[i] = guarded([&] {
            tmv::Matrix<double, tmv::ColMajor> m(
                tmv::MatrixViewOf(A + a_off[i], ni, ni, tmv::ColMajor));
            tmv::MatrixView<double> Bv =
                tmv::MatrixViewOf(B + b_off[i], ni, ri, tmv::ColMajor);
            Bv /= m;
        });
    }
    return 0;
}

}  // extern "C"
