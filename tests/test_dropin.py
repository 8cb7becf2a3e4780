"""The link-time drop-in under unmodified TMV (tmv_gb300/shim), on the CPU.

Builds libtmv_gb300_dropin.so from a TMV source tree ($TMV_REFERENCE, or the
copy in third_party/tmv that the build stages) and checks that TMV's own entry
points for real double data now come from the shim, that TMV's CPU code stays
reachable under the renamed names for the other types, that the surface
program of the GPU drop-in tests runs against stock TMV, and that a program
linked to the drop-in reports a missing GPU through TMV's exception type.  No
GPU needed (tests/test_gpu_dropin.py runs the same programs on one).
"""
import subprocess

import numpy as np
import pytest

from tmv_gb300.build import tmv_source_dir

TMV = tmv_source_dir()

pytestmark = pytest.mark.skipif(TMV is None,
                                reason="no TMV source tree ($TMV_REFERENCE or third_party/tmv)")


@pytest.fixture(scope="module")
def dropin():
    from tmv_gb300.build import build_dropin

    return build_dropin(TMV)


def symbols(path, defined_only=True):
    args = ["nm", "-C"] + (["--defined-only"] if defined_only else []) + [str(path)]
    return subprocess.run(args, capture_output=True, text=True, check=True).stdout


def test_double_entry_points_come_from_the_shim(dropin):
    mm = symbols(dropin / "shim_multmm.o")
    assert ("tmv::MultMM<false, double, double, double>(double, tmv::GenMatrix<double> const&, "
            "tmv::GenMatrix<double> const&, tmv::MatrixView<double, 0>)") in mm
    assert "tmv::MultMM<true, double, double, double>" in mm
    lu = symbols(dropin / "shim_lu.o")
    assert "tmv::LU_Decompose<double>(tmv::MatrixView<double, 0>, long*)" in lu
    assert "tmv::LU_LDivEq<double, double>" in lu and "tmv::LU_RDivEq<double, double>" in lu
    assert "tmv::LU_Inverse<double, double>" in lu
    # the shim reaches the GPU only through the C ABI
    undef = subprocess.run(["nm", "-u", str(dropin / "shim_multmm.o")], capture_output=True,
                           text=True).stdout
    assert "tmvg_multmm_f64_host" in undef


def test_tmv_cpu_code_kept_under_renamed_entry_points(dropin):
    cpu = symbols(dropin / "cpu_TMV_MultMM.o")
    assert "tmv::TMVG_CPU_MultMM<false, std::complex<double>" in cpu
    assert "tmv::MultMM<" not in cpu.replace("TMVG_CPU_MultMM<", "")
    lib = symbols(dropin / "libtmv_gb300_dropin.so")
    assert "tmv::TMVG_CPU_LU_Decompose<float>" in lib
    assert "tmv::TMVG_CPU_LU_LDivEq<std::complex<double>, double>" in lib
    assert "tmv::TMVG_CPU_LU_Inverse<std::complex<double>, std::complex<double> >" in lib


def test_unmodified_tmv_program_links_and_reports(dropin):
    r = subprocess.run([str(dropin / "dropin_demo")], capture_output=True, text=True, timeout=120)
    # without a GPU: TMV's Error carrying the C ABI's status; with one: 0
    if r.returncode == 2:
        assert "tmv::Error" in r.stdout and "tmvg_create" in r.stdout
    else:
        assert r.returncode == 0, r.stdout


def test_surface_program_runs_on_stock_tmv(dropin, tmp_path):
    """The GPU drop-in test's program, linked to stock TMV: every step runs,
    the singular solve throws tmv::Singular, and the product agrees with
    numpy."""
    import test_gpu_dropin as T

    exe = tmp_path / "tmv_surface_stock"
    subprocess.run(["g++", "-O2", "-std=gnu++17", "-w", "-DNOBLAS", "-DNOLAP", "-DTMV_NDEBUG",
                    f"-I{TMV}/include", "-fopenmp", "-o", str(exe), T.SURFACE, f"-L{dropin}",
                    "-ltmv_stock", f"-Wl,-rpath,{dropin}"], check=True)
    n, k, p = 40, 17, 3
    T.write_inputs(tmp_path, np.random.default_rng(5), n, k, p)
    steps, _ = T.run(exe, tmp_path)
    assert steps["singular_ldiv"] == "throw Singular"
    assert all(v == "ok" for s, v in steps.items() if s != "singular_ldiv"), steps
    raw = np.fromfile(tmp_path / "in.bin", dtype=np.float64)[3:]
    A = raw[:n * k].reshape((n, k), order="F")
    B = raw[n * k:n * k + k * p].reshape((k, p), order="F")
    C = T.load(tmp_path, "prod_ccc", (n, p))
    assert np.abs(C - A @ B).max() <= 1e-13 * np.abs(A @ B).max()
    for name, shape in T.result_shapes(n, k, p).items():  # every result has its size
        assert T.load(tmp_path, name, shape).shape == shape
    for name, shape in T.float_shapes(n, k, p).items():
        assert T.load(tmp_path, name, shape).shape == shape
    for name, shape in T.complex_shapes(n, k, p).items():
        assert T.load_z(tmp_path, name, shape).shape == shape


def test_stock_tmv_wide_lu_differs_only_in_its_last_row(dropin, tmp_path):
    """Stock TMV's LU_Decompose of a wide matrix (M < N) reproduces A except
    in the last row beyond column M: its two-row recursion leaf updates U(1,
    2:N) with U(0,1) where L(1,0) belongs (src/TMV_LUDecompose.cpp:349-355).
    This pins the one place where the drop-in's (correct) result and TMV's
    differ, which the GPU drop-in test leaves out of its comparison."""
    import test_gpu_dropin as T

    exe = tmp_path / "tmv_surface_stock"
    subprocess.run(["g++", "-O2", "-std=gnu++17", "-w", "-DNOBLAS", "-DNOLAP", "-DTMV_NDEBUG",
                    f"-I{TMV}/include", "-fopenmp", "-o", str(exe), T.SURFACE, f"-L{dropin}",
                    "-ltmv_stock", f"-Wl,-rpath,{dropin}"], check=True)
    n, k, p = 40, 17, 3
    T.write_inputs(tmp_path, np.random.default_rng(12), n, k, p)
    T.run(exe, tmp_path)
    raw = np.fromfile(tmp_path / "in.bin", dtype=np.float64)[3:]
    A = raw[:n * k].reshape((n, k), order="F")
    M = A.T
    R = T.plu(T.load(tmp_path, "lu_wide", (k, n)), T.load(tmp_path, "lu_wide_pivots", None).astype(np.int64))
    bad = np.abs(R - M) > 1e-12 * np.abs(M).max()
    rows, cols = np.nonzero(bad)
    assert len(rows) > 0 and set(rows.tolist()) <= {k - 1} and cols.min() >= k
    Rt = T.plu(T.load(tmp_path, "lu_tall", (n, k)), T.load(tmp_path, "lu_tall_pivots", None).astype(np.int64))
    assert np.abs(Rt - A).max() <= 1e-13 * np.abs(A).max()
