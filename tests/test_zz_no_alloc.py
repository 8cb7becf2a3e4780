"""The no-allocation LU entry point (tmvg_lu_decompose_f64_noalloc).

Some callers cannot allocate device memory: their device memory belongs to
another allocator (a framework's caching allocator, a fixed arena) or an
allocation is not acceptable on their code path.  For them the library has
one extra entry point that factors with scratch taken from a static device
array instead of cudaMalloc.  This test calls it through the C ABI twice in a
row and compares each result with the regular entry point's, and checks that
a size above its stated limit is refused.  It lives in a file that pytest
collects last, so a run that stops at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import to_dev, to_host

pytestmark = pytest.mark.gpu


def test_noalloc_lu_matches_regular_entry_point(dev):
    import torch

    from tmv_gb300 import _lib, linalg

    lib = _lib.load()
    noalloc = lib.tmvg_lu_decompose_f64_noalloc
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(2024)
    for n in (700, 1300):  # two calls in a row, different sizes
        a = rng.standard_normal((n, n))
        A1 = to_dev(a, dev, "F")
        P1 = torch.empty(n, dtype=torch.int64, device=dev)
        st = noalloc(n, C.c_void_p(A1.data_ptr()), n, C.c_void_p(P1.data_ptr()),
                     C.c_void_p(stream))
        assert st == 0, _lib.STATUS.get(st, st)
        A2 = to_dev(a, dev, "F")
        P2 = linalg.lu_decompose(A2)
        torch.cuda.synchronize()
        lu1, lu2 = to_host(A1), to_host(A2)
        assert np.array_equal(to_host(P1), to_host(P2))
        assert np.abs(lu1 - lu2).max() <= 1e-12 * max(np.abs(lu2).max(), 1.0)


def test_noalloc_rejects_sizes_above_its_limit():
    from tmv_gb300 import _lib

    lib = _lib.load()
    # refused on the host before any device work (8 = TMVG_UNSUPPORTED)
    assert lib.tmvg_lu_decompose_f64_noalloc(16385, None, 16385, None, None) == 8
    assert lib.tmvg_lu_decompose_f64_noalloc(-1, None, 1, None, None) == 3
