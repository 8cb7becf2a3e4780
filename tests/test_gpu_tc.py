"""The tcgen05 3xTF32 update C -= A B against an FP64 reference (FP32 accuracy)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128, 64), (1000, 777, 64), (300, 90, 32), (513, 1025, 128), (4000, 130, 96),
          (129, 257, 64), (8, 8, 32)]


def tc_update(dev, a, b, c):
    import torch

    from tmv_gb300 import linalg

    A = torch.from_numpy(np.ascontiguousarray(a.T)).to(dev).t()  # column-major
    B = torch.from_numpy(np.ascontiguousarray(b.T)).to(dev).t()
    Cd = torch.from_numpy(np.ascontiguousarray(c.T)).to(dev).t()
    m, k = a.shape
    n = b.shape[1]
    h = linalg.handle(dev.index)
    h.check(h.call("tmvg_gemm_f32_tf32x3", m, n, k, C.c_void_p(A.data_ptr()), A.stride(1),
                   C.c_void_p(B.data_ptr()), B.stride(1), C.c_void_p(Cd.data_ptr()), Cd.stride(1)),
            "tf32x3")
    torch.cuda.synchronize()
    return Cd.cpu().numpy()


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_tf32x3_update_has_fp32_accuracy(dev, m, n, k):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((k, n)).astype(np.float32)
    c = rng.standard_normal((m, n)).astype(np.float32)
    got = tc_update(dev, a, b, c)
    ref = c.astype(np.float64) - a.astype(np.float64) @ b.astype(np.float64)
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64) + np.abs(c)
    err = np.abs(got - ref) / scale
    # FP32 accuracy: k products of 2^-22 relative error plus FP32 rounding;
    # a single TF32 product would be ~2^-11.
    assert err.max() <= 4e-6, err.max()


def test_rejects_unsupported_depth(dev):
    from tmv_gb300 import TmvgError

    with pytest.raises(TmvgError):
        tc_update(dev, np.ones((64, 40), np.float32), np.ones((40, 64), np.float32),
                  np.zeros((64, 64), np.float32))
