"""The C ABI library builds, loads and exports every declared entry point
(no GPU work: nothing here launches a kernel)."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_in_headers():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(tmvg_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    from tmv_gb300 import _lib
    from tmv_gb300.build import LIB, build_library

    if not LIB.exists():
        build_library()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    import ctypes

    names = declared_in_headers()
    assert len(names) >= 20
    for name in sorted(names):
        assert hasattr(lib, name), name
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)


def test_python_binding_covers_the_header():
    from tmv_gb300 import _lib

    assert declared_in_headers() <= set(_lib.declared_symbols())


def test_status_strings(lib):
    assert lib.tmvg_version() >= 1
    assert lib.tmvg_status_string(0) == b"ok"
    assert lib.tmvg_status_string(1) == b"singular"
    assert lib.tmvg_status_string(2) == b"not converged"


def test_null_handle_is_rejected(lib):
    # entry points check their handle before touching the device
    assert lib.tmvg_synchronize(None) == 3
    assert lib.tmvg_lu_decompose_f64(None, 4, None, 4, None) == 3
    # the complex<double> entry points too
    import ctypes as C

    lib.tmvg_lu_decompose_z64.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
    assert lib.tmvg_lu_decompose_z64(None, 4, None, 4, None) == 3
    for name in ("tmvg_lu_ldiveq_z64", "tmvg_lu_rdiveq_z64"):
        f = getattr(lib, name)
        f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                      C.c_int64]
        assert f(None, 4, None, 4, None, 1, None, 4) == 3
    lib.tmvg_lu_inverse_z64.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                        C.c_void_p, C.c_int64]
    assert lib.tmvg_lu_inverse_z64(None, 4, None, 4, None, None, 4) == 3


def test_library_is_sm103a_only():
    # the build passes exactly one -gencode for sm_103a
    from tmv_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
