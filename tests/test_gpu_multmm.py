"""MultMM on the GPU against the oracle and TMV's exact integer product pins."""
import numpy as np
import pytest

from helpers import arith8_operands, rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu

LAYOUTS = [("F", "F"), ("F", "C"), ("C", "F"), ("C", "C")]  # CCC, CRC, RCC, RRC


def _multmm(dev, add, alpha, a, b, c0, la, lb, lc="F"):
    import torch

    from tmv_gb300 import linalg

    A = to_dev(a, dev, la)
    B = to_dev(b, dev, lb)
    C = to_dev(c0, dev, lc)
    linalg.multmm(add, alpha, A, B, C)
    torch.cuda.synchronize()
    return to_host(C)


@pytest.mark.parametrize("la,lb", LAYOUTS)
def test_arith8_integer_products_exact(dev, la, lb):
    # tests/TMV_TestMatrixArith_8.cpp:327-396: sizes {2,5,77,637}, every
    # product of integer-valued operands is exact in FP64 -> bitwise equality.
    sizes = [2, 5, 77, 637]
    for m in sizes:
        for n in sizes:
            for k in sizes:
                a, b = arith8_operands(m, n, k)
                exact = (a.astype(np.int64) @ b.astype(np.int64)).astype(np.float64)
                c = _multmm(dev, False, 1.0, a, b, np.zeros((m, n)), la, lb)
                assert np.array_equal(c, exact), (m, n, k, la, lb)


@pytest.mark.parametrize("la,lb", LAYOUTS)
@pytest.mark.parametrize("lc", ["F", "C"])
def test_random_layouts_vs_oracle(dev, orc, la, lb, lc):
    rng = np.random.default_rng(11)
    for (m, n, k) in [(1, 1, 1), (3, 7, 2), (16, 16, 16), (33, 65, 17), (200, 130, 301)]:
        a = rng.uniform(-1, 1, (m, k))
        b = rng.uniform(-1, 1, (k, n))
        c0 = rng.uniform(-1, 1, (m, n))
        for add, alpha in [(False, 1.0), (True, -1.0), (True, 2.5), (False, -0.75)]:
            ref = np.asfortranarray(c0.copy())
            orc.multmm(add, alpha, np.asfortranarray(a), np.asfortranarray(b), ref)
            got = _multmm(dev, add, alpha, a, b, c0, la, lb, lc)
            assert rel_frob(got, ref) <= 1e-13, (m, n, k, add, alpha)


def test_config1_gemm_1024(dev, orc):
    # FP64 C = A*B, M=N=K=1024, A,B ~ U[-1,1] column-major; within 1e-13
    # relative Frobenius error of TMV's block product.
    rng = np.random.default_rng(1)
    a = rng.uniform(-1, 1, (1024, 1024))
    b = rng.uniform(-1, 1, (1024, 1024))
    ref = np.zeros((1024, 1024), order="F")
    orc.multmm(False, 1.0, np.asfortranarray(a), np.asfortranarray(b), ref)
    got = _multmm(dev, False, 1.0, a, b, np.zeros((1024, 1024)), "F", "F")
    assert rel_frob(got, ref) <= 1e-13


def test_empty_and_degenerate(dev):
    import torch

    from tmv_gb300 import linalg

    # k = 0: C = 0 (add = False) or unchanged (add = True)
    c0 = np.arange(12.0).reshape(3, 4)
    got = _multmm(dev, False, 1.0, np.zeros((3, 0)), np.zeros((0, 4)), c0, "F", "F")
    assert np.array_equal(got, np.zeros((3, 4)))
    got = _multmm(dev, True, 1.0, np.zeros((3, 0)), np.zeros((0, 4)), c0, "F", "F")
    assert np.array_equal(got, c0)
    # alpha = 0 with add leaves C
    got = _multmm(dev, True, 0.0, np.ones((3, 5)), np.ones((5, 4)), c0, "F", "F")
    assert np.array_equal(got, c0)
    # m = 0 / n = 0 are no-ops
    A = torch.zeros((0, 5), dtype=torch.float64, device=dev)
    B = torch.zeros((5, 4), dtype=torch.float64, device=dev)
    C = torch.zeros((0, 4), dtype=torch.float64, device=dev)
    linalg.multmm(False, 1.0, A, B, C)


def test_host_entry_matches_device(dev, orc):
    # tmvg_multmm_f64_host: host buffers, copies inside the call
    import ctypes as C

    from tmv_gb300 import linalg

    rng = np.random.default_rng(5)
    a = np.asfortranarray(rng.uniform(-1, 1, (70, 40)))
    b = np.ascontiguousarray(rng.uniform(-1, 1, (40, 55)))  # row-major B
    c = np.asfortranarray(rng.uniform(-1, 1, (70, 55)))
    ref = c.copy(order="F")
    orc.multmm(True, 1.5, a, b, ref)
    h = linalg.handle(0)
    h.check(h.call("tmvg_multmm_f64_host", 1, 1.5, 70, 55, 40, C.c_void_p(a.ctypes.data), 1, 70,
                   C.c_void_p(b.ctypes.data), 55, 1, C.c_void_p(c.ctypes.data), 1, 70))
    assert rel_frob(c, ref) <= 1e-13
