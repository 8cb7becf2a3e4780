// tmv_surface.cpp -- a TMV user program (TMV's public API only) that runs the
// surface of the dense hot path on inputs read from a directory and writes
// every result back as raw column-major doubles.  The drop-in tests build it
// twice from this one source: linked to stock TMV and linked to the GB300
// drop-in, then compare the two outputs.
//
//   tmv_surface <dir>
//     in:  <dir>/in.bin   int64 n, k, p, then column-major doubles
//                         A (n x k), B (k x p), M (n x n), R (n x p),
//                         W (p x n), b (n), S (n x n, singular), then
//                         complex<double> (real, imaginary interleaved)
//                         Mz (n x n), Rz (n x p), Wz (p x n)
//     out: <dir>/<name>.bin for each result, <dir>/results.txt with one line
//          "<name> ok" or "<name> throw <exception kind>" per step.
//
// Surface covered (include/tmv/TMV_MatrixArith.h:701-730, 980-1010,
// 1145-1227; src/TMV_LUD.cpp:37-262; src/TMV_BaseMatrix.cpp:31-293):
// C = A*B in the CCC, RCC, CRC layouts and into a row-major C; C += x*A*B and
// C -= A*B; a product of strided views; m.divideUsing(tmv::LU), saveDiv,
// X = R/m, x = b/m, Y = W%m, X /= m, det, logDet, inverse, isSingular, the LU
// factors and pivots; the same solves on a row-major m (TMV's istrans path);
// LU_Decompose of a tall and a wide matrix (include/tmv/TMV_LUD.h:79); the
// solve of a singular m, which must throw; and the same product and LU
// surface for tmv::Matrix<float> and tmv::Matrix<std::complex<double> >.
#include <algorithm>
#include <complex>
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

template <class M>
void save_z(const std::string& name, const M& m)
{
    std::vector<double> v;
    for (ptrdiff_t j = 0; j < (ptrdiff_t)m.rowsize(); ++j)
        for (ptrdiff_t i = 0; i < (ptrdiff_t)m.colsize(); ++i) {
            const std::complex<double> z = m(i, j);
            v.push_back(z.real());
            v.push_back(z.imag());
        }
    std::ofstream f(g_dir + "/" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
}

template <class M>
void save_f(const std::string& name, const M& m)
{
    std::vector<double> v;
    for (ptrdiff_t j = 0; j < (ptrdiff_t)m.rowsize(); ++j)
        for (ptrdiff_t i = 0; i < (ptrdiff_t)m.colsize(); ++i) v.push_back((double)m(i, j));
    std::ofstream f(g_dir + "/" + name + ".bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
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
    auto readz = [&](ptrdiff_t rows, ptrdiff_t cols) {
        tmv::Matrix<std::complex<double> > m(rows, cols);
        std::vector<double> v(2 * rows * cols);
        in.read(reinterpret_cast<char*>(v.data()), v.size() * sizeof(double));
        for (ptrdiff_t j = 0; j < cols; ++j)
            for (ptrdiff_t i = 0; i < rows; ++i)
                m(i, j) = std::complex<double>(v[2 * (i + j * rows)], v[2 * (i + j * rows) + 1]);
        return m;
    };
    const tmv::Matrix<std::complex<double> > Mz = readz(n, n), Rz = readz(n, p), Wz = readz(p, n);
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

    // float: MultMM<float> and the LU surface on the same data, rounded
    auto tofloat = [](const tmv::Matrix<double>& d) {
        tmv::Matrix<float> f(d.colsize(), d.rowsize());
        for (ptrdiff_t j = 0; j < (ptrdiff_t)d.rowsize(); ++j)
            for (ptrdiff_t i = 0; i < (ptrdiff_t)d.colsize(); ++i) f(i, j) = (float)d(i, j);
        return f;
    };
    const tmv::Matrix<float> Af = tofloat(A), Bf = tofloat(B), Mf = tofloat(M), Rf = tofloat(R),
                             Wf = tofloat(W);
    step("f_prod", [&] {
        tmv::Matrix<float> C = Af * Bf;
        C += 0.5f * Af * Bf;
        save_f("f_prod", C);
    });
    tmv::Matrix<float> mf = Mf;
    mf.divideUsing(tmv::LU);
    mf.saveDiv();
    step("f_ldiv", [&] { tmv::Matrix<float> X = Rf / mf; save_f("f_ldiv", X); });
    step("f_rdiv", [&] { tmv::Matrix<float> Y = Wf % mf; save_f("f_rdiv", Y); });
    step("f_inverse", [&] { tmv::Matrix<float> Mi = mf.inverse(); save_f("f_inverse", Mi); });
    step("f_factors", [&] {
        save_f("f_factors", mf.lud().getLU());
        const ptrdiff_t* pv = mf.lud().getP().getValues();
        save_vec("f_pivots", std::vector<double>(pv, pv + n));
    });

    // complex<double>: LU_Decompose, LU_LDivEq, LU_RDivEq, LU_Inverse, det
    tmv::Matrix<std::complex<double> > mz = Mz;
    mz.divideUsing(tmv::LU);
    mz.saveDiv();
    step("z_ldiv", [&] { tmv::Matrix<std::complex<double> > X = Rz / mz; save_z("z_ldiv", X); });
    step("z_rdiv", [&] { tmv::Matrix<std::complex<double> > Y = Wz % mz; save_z("z_rdiv", Y); });
    step("z_inverse", [&] { tmv::Matrix<std::complex<double> > Mi = mz.inverse(); save_z("z_inverse", Mi); });
    step("z_factors", [&] {
        save_z("z_factors", mz.lud().getLU());
        const ptrdiff_t* pv = mz.lud().getP().getValues();
        save_vec("z_pivots", std::vector<double>(pv, pv + n));
        const std::complex<double> d = mz.det();
        save_vec("z_det", {d.real(), d.imag()});
    });
    tmv::Matrix<std::complex<double>, tmv::RowMajor> mzr = Mz;
    mzr.divideUsing(tmv::LU);
    step("z_rm_ldiv", [&] { tmv::Matrix<std::complex<double> > X = Rz / mzr; save_z("z_rm_ldiv", X); });
    return 0;
}
