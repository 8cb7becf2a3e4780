// dropin_demo.cpp -- unmodified TMV user code linked against the drop-in:
// C = A*B, A.divideUsing(tmv::LU), x = b/A, X = B/A, Y = W%A, det.  With a
// GPU the double-precision work runs on it; prints residual checks and exits
// non-zero if one fails.  Without a device every GPU call throws
// tmv::Error("... no cuda device ..."), which the demo reports (exit 2).
#include <cmath>
#include <cstdio>

#include "TMV.h"

int main()
{
    try {
        const int n = 300, nrhs = 5;
        tmv::Matrix<double> A(n, n), B(n, nrhs), W(nrhs, n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) A(i, j) = std::sin(1.0 + i * 0.37 + j * 1.3) + (i == j ? 20.0 : 0.0);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < nrhs; ++j) { B(i, j) = std::cos(i + 2.0 * j); W(j, i) = std::sin(i - j); }

        tmv::Matrix<double> C = A * B;                      // MultMM<false>
        tmv::Matrix<double> C2(n, nrhs);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < nrhs; ++j) {
                double s = 0;
                for (int k = 0; k < n; ++k) s += A(i, k) * B(k, j);
                C2(i, j) = s;
            }
        const double eprod = Norm(C - C2) / Norm(C2);

        A.divideUsing(tmv::LU);
        A.saveDiv();
        tmv::Matrix<double> X = B / A;                      // LU_Decompose + LU_LDivEq
        tmv::Matrix<double> Y = W % A;                      // LU_RDivEq
        const double eX = Norm(A * X - B) / Norm(B);
        const double eY = Norm(Y * A - W) / Norm(W);
        std::printf("product rel err %.3e  B/A resid %.3e  W%%A resid %.3e  det %.6e\n", eprod,
                    eX, eY, A.det());
        return (eprod < 1e-13 && eX < 1e-13 && eY < 1e-13) ? 0 : 1;
    } catch (tmv::Error& e) {
        std::printf("tmv::Error: %s\n", e.what());
        return 2;
    }
}
