"""The no-allocation LU entry point (tmvg_lu_decompose_f64_noalloc).

Some callers cannot allocate device memory: their device memory belongs to
another allocator (a framework's caching allocator, a fixed arena) or an
allocation is not acceptable on their code path.  For them the library has
one extra entry point that factors with scratch taken from a static device
array instead of cudaMalloc.  These tests call it through the C ABI: twice in
a row, each result compared with the regular entry point's; with the free
device memory read around calls that nothing else interleaves, which must not
change; and with a size above its stated limit, which is refused.  The file
is collected last, so a run that stops at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import to_dev, to_host

pytestmark = pytest.mark.gpu


def _noalloc(lib, A, P, n, stream):
    return lib.tmvg_lu_decompose_f64_noalloc(n, C.c_void_p(A.data_ptr()), n,
                                             C.c_void_p(P.data_ptr()), C.c_void_p(stream))


def test_noalloc_lu_matches_regular_entry_point(dev):
    import torch

    from tmv_gb300 import _lib, linalg

    lib = _lib.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(2024)
    for n in (700, 1300):  # two calls in a row, different sizes
        a = rng.standard_normal((n, n))
        A1 = to_dev(a, dev, "F")
        P1 = torch.empty(n, dtype=torch.int64, device=dev)
        st = _noalloc(lib, A1, P1, n, stream)
        assert st == 0, _lib.STATUS.get(st, st)
        A2 = to_dev(a, dev, "F")
        P2 = linalg.lu_decompose(A2)
        torch.cuda.synchronize()
        lu1, lu2 = to_host(A1), to_host(A2)
        assert np.array_equal(to_host(P1), to_host(P2))
        assert np.abs(lu1 - lu2).max() <= 1e-12 * max(np.abs(lu2).max(), 1.0)


def test_noalloc_lu_leaves_free_device_memory_unchanged(dev):
    """Free device memory (cudaMemGetInfo) is the same before and after a call.

    Each size is factored once first, so that the kernels it launches are
    loaded before the measured call (module loading may take device memory);
    the measured calls then run with no handle and no other library call in
    between, on inputs allocated beforehand."""
    import torch

    from tmv_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(77)
    sizes = (900, 1700)
    mats = {n: rng.standard_normal((n, n)) for n in sizes}
    for n in sizes:  # warm-up: load every kernel each size uses
        A = to_dev(mats[n], dev, "F")
        P = torch.empty(n, dtype=torch.int64, device=dev)
        assert _noalloc(lib, A, P, n, stream) == 0
    bufs = {n: (to_dev(mats[n], dev, "F"), torch.empty(n, dtype=torch.int64, device=dev))
            for n in sizes}
    torch.cuda.synchronize()
    for n in sizes:
        free0, _ = torch.cuda.mem_get_info(dev)
        assert _noalloc(lib, *bufs[n], n, stream) == 0
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info(dev)
        assert free1 == free0, f"n={n}: free device memory changed by {free0 - free1} bytes"


def test_noalloc_rejects_sizes_above_its_limit():
    from tmv_gb300 import _lib

    lib = _lib.load()
    # refused on the host before any device work (8 = TMVG_UNSUPPORTED)
    assert lib.tmvg_lu_decompose_f64_noalloc(16385, None, 16385, None, None) == 8
    assert lib.tmvg_lu_decompose_f64_noalloc(-1, None, 1, None, None) == 3
