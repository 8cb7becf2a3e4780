// tmv_surface.cpp -- a TMV user program (TMV's public API only) that runs the
// surface of the dense hot path on inputs read from a directory and writes
// every result back as raw column-major doubles.  The drop-in tests build it
// twice from this one source: linked to stock TMV and linked to the GB300
// drop-in, then compare the two outputs.
//
//   tmv_surface <dir>
//     in:  <dir>/in.bin   int64 n, k, p, then column-major doubles
//                         A (n x k), B (k x p), M (n x n), R (n x p),
//                         W (p x n), b (n), S (n x n, singular)
//     out: <dir>/<name>.bin for each result, <dir>/results.txt with one line
//          "<name> ok" or "<name> throw <exception kind>" per step.
//
// Surface covered (include/tmv/TMV_MatrixArith.h:701-730, 980-1010,
// 1145-1227; src/TMV_LUD.cpp:37-262; src/TMV_BaseMatrix.cpp:31-293):
// C = A*B in the CCC, RCC, CRC layouts and into a row-major C; C += x*A*B and
// C -= A*B; a product of strided views; m.divideUsing(tmv::LU), saveDiv,
// X = R/m, x = b/m, Y = W%m, X /= m, det, logDet, inverse, isSingular, the LU
// factors and pivots; the same solves on a row-major m (TMV's istrans path);
// LU_Decompose of a tall and a wide matrix (include/tmv/TMV_LUD.h:79); and
// the solve of a singular m, which must throw.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "TMV.h"

namespace {

std::string g_dir;
std::ofstream g_log;

template <class M>
void save(const std::string& name, const M& m)
{
    std::vector<double> v;
    v.reserve(m.colsize() * m.rowsize());
    for (ptrdiff_t j = 0; j < (ptrdiff_t)m.rowsize(); ++j)
        for (ptrdiff_t i = 0; i < (ptrdiff_t)m.colsize(); ++i) v.push_back(m(i, j));
    std::ofstream f(g_dir + "/" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
}

void save_vec(const std::string& name, const std::vector<double>& v);

void save_v(const std::string& name, const tmv::Vector<double>& x)
{
    std::vector<double> v(x.size());
    for (ptrdiff_t i = 0; i < (ptrdiff_t)x.size(); ++i) v[i] = x(i);
    save_vec(name, v);
}

void save_vec(const std::string& name, const std::vector<double>& v)
{
    std::ofstream f(g_dir + "/" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
}

template <class F>
void step(const char* name, F f)
{
    try {
        f();
        g_log << name << " ok\n";
    } catch (tmv::Singular&) {
        g_log << name << " throw Singular\n";
    } catch (tmv::Error& e) {
        g_log << name << " throw Error " << e.what() << "\n";
    } catch (std::exception& e) {
        g_log << name << " throw std " << e.what() << "\n";
    }
    g_log.flush();
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 2) {
        std::fprintf(stderr, "usage: tmv_surface <dir>\n");
        return 2;
    }
    g_dir = argv[1];
    std::ifstream in(g_dir + "/in.bin", std::ios::binary);
    int64_t dims[3];
    in.read(reinterpret_cast<char*>(dims), sizeof(dims));
    const ptrdiff_t n = dims[0], k = dims[1], p = dims[2];
    auto read = [&](ptrdiff_t rows, ptrdiff_t cols) {
        tmv::Matrix<double> m(rows, cols);
        std::vector<double> v(rows * cols);
        in.read(reinterpret_cast<char*>(v.data()), v.size() * sizeof(double));
        for (ptrdiff_t j = 0; j < cols; ++j)
            for (ptrdiff_t i = 0; i < rows; ++i) m(i, j) = v[i + j * rows];
        return m;
    };
    const tmv::Matrix<double> A = read(n, k), B = read(k, p), M = read(n, n), R = read(n, p),
                              W = read(p, n), bm = read(n, 1), S = read(n, n);
    if (!in) {
        std::fprintf(stderr, "short input\n");
        return 2;
    }
    const tmv::Vector<double> b = bm.col(0);
    g_log.open(g_dir + "/results.txt");

    // products: MultMM<false> / MultMM<true> in each layout
    const tmv::Matrix<double, tmv::RowMajor> Ar = A, Br = B;
    step("prod_ccc", [&] { tmv::Matrix<double> C = A * B; save("prod_ccc", C); });
    step("prod_rcc", [&] { tmv::Matrix<double> C = Ar * B; save("prod_rcc", C); });
    step("prod_crc", [&] { tmv::Matrix<double> C = A * Br; save("prod_crc", C); });
    step("prod_rm_c", [&] {
        tmv::Matrix<double, tmv::RowMajor> C = Ar * Br;
        save("prod_rm_c", C);
    });
    step("prod_add", [&] {
        tmv::Matrix<double> C = A * B;
        C += 0.75 * A * B;
        C -= Ar * B;
        save("prod_add", C);
    });
    step("prod_views", [&] {
        // every other row of A times every other column of B (n2 and p2
        // of them: TMV's strided subMatrix holds (i2 - i1) / istep rows),
        // and a transpose
        const ptrdiff_t n2 = (n + 1) / 2, p2 = (p + 1) / 2;
        tmv::Matrix<double> C = A.subMatrix(0, 2 * n2, 0, k, 2, 1) *
                                B.subMatrix(0, k, 0, 2 * p2, 1, 2);
        tmv::Matrix<double> D = B.transpose() * A.transpose();
        save("prod_views", C);
        save("prod_transpose", D);
    });

    // LU: divideUsing(LU), saveDiv, the solves and the LUDiv queries
    tmv::Matrix<double> m = M;
    m.divideUsing(tmv::LU);
    m.saveDiv();
    step("lu_ldiv", [&] { tmv::Matrix<double> X = R / m; save("lu_ldiv", X); });
    step("lu_ldiv_vec", [&] { tmv::Vector<double> x = b / m; save_v("lu_ldiv_vec", x); });
    step("lu_rdiv", [&] { tmv::Matrix<double> Y = W % m; save("lu_rdiv", Y); });
    step("lu_ldiveq", [&] {
        tmv::Matrix<double> X = R;
        X /= m;
        save("lu_ldiveq", X);
    });
    step("lu_factors", [&] {
        save("lu_factors", m.lud().getLU());
        std::vector<double> P(n);
        const ptrdiff_t* pv = m.lud().getP().getValues();
        for (ptrdiff_t i = 0; i < n; ++i) P[i] = (double)pv[i];
        save_vec("lu_pivots", P);
    });
    step("lu_det", [&] {
        double sign = 0;
        const double ld = m.logDet(&sign);
        save_vec("lu_det", {m.det(), ld, sign, m.isSingular() ? 1.0 : 0.0});
    });
    step("lu_inverse", [&] { tmv::Matrix<double> Mi = m.inverse(); save("lu_inverse", Mi); });

    // a row-major matrix: TMV factors its transpose (istrans)
    tmv::Matrix<double, tmv::RowMajor> mr = M;
    mr.divideUsing(tmv::LU);
    step("rm_ldiv", [&] { tmv::Matrix<double> X = R / mr; save("rm_ldiv", X); });
    step("rm_rdiv", [&] { tmv::Matrix<double> Y = W % mr; save("rm_rdiv", Y); });

    // LU_Decompose of rectangular matrices (TMV factors min(M,N) columns)
    auto rect = [&](const char* name, tmv::Matrix<double> T) {
        step(name, [&] {
            const ptrdiff_t r = std::min(T.colsize(), T.rowsize());
            std::vector<ptrdiff_t> P(r);
            tmv::LU_Decompose(T.view(), P.data());
            save(name, T);
            save_vec(std::string(name) + "_pivots", std::vector<double>(P.begin(), P.end()));
        });
    };
    rect("lu_tall", A);
    rect("lu_wide", A.transpose());

    // a singular matrix: factorisation succeeds, the solve throws
    tmv::Matrix<double> s = S;
    s.divideUsing(tmv::LU);
    step("singular_ldiv", [&] { tmv::Vector<double> x = b / s; save_v("singular_ldiv", x); });
    step("singular_det", [&] { save_vec("singular_det", {s.det(), s.isSingular() ? 1.0 : 0.0}); });
    return 0;
}
