"""Failure path of a bounded device-side wait, without a GPU fault.

The sync-free triangular solve hands its 64-row blocks to CTAs by ticket, and
each block waits (bounded) for the publication flags of the blocks before it.
tmvg_test_set_wait shortens that wait and makes the next solve start its
tickets at block 1, so block 0 is never solved and its flag is never set: the
wait must give up, the call must return TMVG_TIMEOUT (TMV's error path for a
failed solve is an exception, src/TMV_TriDiv_M.cpp:78-84; here it is the
status code the drop-in turns into tmv::Error), and the same handle must then
solve correctly.  No kernel traps or spins without a limit.
"""
import ctypes as C
import time

import numpy as np
import pytest

from helpers import rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu

TIMEOUT = 5


def _tri_call(h, T, B, upper=False):
    n = T.shape[0]
    return h.call("tmvg_tri_ldiveq_f64", int(upper), 0, n, C.c_void_p(T.data_ptr()), T.stride(0),
                  T.stride(1), B.shape[1], C.c_void_p(B.data_ptr()), B.stride(0), B.stride(1))


@pytest.mark.parametrize("upper", [False, True])
def test_unpublished_block_times_out_and_handle_recovers(dev, orc, upper):
    import torch

    from tmv_gb300 import linalg

    rng = np.random.default_rng(91)
    n, nrhs = 700, 3
    t = np.tril(rng.standard_normal((n, n))) if not upper else np.triu(rng.standard_normal((n, n)))
    t[np.diag_indices(n)] = 4.0 + rng.random(n)
    b = rng.standard_normal((n, nrhs))
    h = linalg.handle(dev.index or 0)
    T = to_dev(t, dev, "F")

    B = to_dev(b, dev, "F")
    torch.cuda.synchronize()
    h.check(h.call("tmvg_test_set_wait", 2000, 1), "test_set_wait")
    try:
        t0 = time.perf_counter()
        st = _tri_call(h, T, B, upper)
        dt = time.perf_counter() - t0
        msg = h.lib.tmvg_last_error(h.h)
    finally:
        # the skip resets itself after one launch; restore the default limit
        h.check(h.call("tmvg_test_set_wait", 0, 0), "test_set_wait")
    assert st == TIMEOUT, (st, msg)
    assert b"timed out" in msg
    assert dt < 10.0

    B = to_dev(b, dev, "F")
    assert _tri_call(h, T, B, upper) == 0
    torch.cuda.synchronize()
    bo = np.asfortranarray(b.copy())
    assert orc.tri_ldiveq(upper, False, np.asfortranarray(t), bo) == 0
    assert rel_frob(to_host(B), bo) <= 1e-12
    # and the handle's other paths still run: an LU solve on the same handle
    X, LU, P = linalg.divide(to_dev(t + t.T, dev, "F"), to_dev(b, dev, "F"))
    assert np.isfinite(to_host(X)).all()


def test_test_hook_rejects_negative_skip(dev):
    from tmv_gb300 import linalg

    h = linalg.handle(dev.index or 0)
    assert h.call("tmvg_test_set_wait", 0, -1) == 3  # TMVG_BAD_ARG


def test_refinement_solve_wait_times_out_and_handle_recovers(dev):
    """The same hook on the mixed solve's streamed FP32 triangular solve
    (n = 512: whole 128-row blocks, each CTA waiting on tagged words of the
    blocks before it): its first launch starts at ticket 1, block 0 never
    publishes, the wait on it gives up after 2000 polls, the solve returns
    TMVG_TIMEOUT, and the next solve on the same handle converges."""
    from tmv_gb300 import TmvgError, linalg

    rng = np.random.default_rng(92)
    n = 512
    a = rng.standard_normal((n, n)) + 4.0 * np.sqrt(n) * np.eye(n)
    b = rng.standard_normal(n)
    h = linalg.handle(dev.index or 0)
    A = to_dev(a, dev, "F")
    B = to_dev(b.reshape(n, 1), dev, "F")
    h.check(h.call("tmvg_test_set_wait", 2000, 1), "test_set_wait")
    try:
        t0 = time.perf_counter()
        with pytest.raises(TmvgError) as ei:
            linalg.solve_mixed(A, B)
        dt = time.perf_counter() - t0
    finally:
        h.check(h.call("tmvg_test_set_wait", 0, 0), "test_set_wait")
    assert ei.value.status == TIMEOUT
    assert "timed out" in str(ei.value)
    assert dt < 10.0
    X, info = linalg.solve_mixed(A, B)
    assert info.converged == 1
    x = to_host(X)[:, 0]
    assert np.abs(a @ x - b).max() <= 1e-12 * (np.abs(a).sum(axis=1).max() * np.abs(x).max())
