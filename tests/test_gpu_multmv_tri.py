"""y (+)= alpha A x and standalone triangular division on the GPU.

MultMV<add> (src/TMV_MultMV.cpp:1134-1175) and TriLDivEq for upper and lower
triangles (src/TMV_TriDiv_M.cpp:583-710) through the C ABI, against TMV's own
outputs on their special cases (tests/golden/multmv_tri.npz) and against the
oracle over layouts and sizes; integer-valued operands are exact; at full
size (A 8192 x 8192, 512 MiB) the product agrees with an FP64 torch matmul.
"""
from pathlib import Path

import numpy as np
import pytest

from helpers import arith8_operands, diag_shift_matrix, rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def dev_matrix(a, dev, layout):
    import torch

    if layout == "S":  # every other row, every third column of a larger buffer
        m, n = a.shape
        big = np.zeros((2 * m + 1, 3 * n + 2))
        big[: 2 * m : 2, : 3 * n : 3] = a
        t = torch.from_numpy(big).to(dev)
        return t[: 2 * m : 2, : 3 * n : 3]
    return to_dev(a, dev, layout)


def test_multmv_matches_tmv_special_cases(dev):
    import torch

    from tmv_gb300 import linalg

    g = np.load(GOLD / "multmv_tri.npz")
    a, x, y0 = g["mv_A"], g["mv_x"], g["mv_y0"]
    for lay in ("F", "C"):
        for add in (0, 1):
            A = to_dev(a, dev, lay)
            xd = torch.from_numpy(x).to(dev)
            y = torch.from_numpy(y0.copy()).to(dev)
            linalg.multmv(bool(add), 0.5, A, xd, y)
            yh, ref = to_host(y), g[f"mv_{lay}_{add}"]
            # a NaN in a column whose x_j is 0 reaches y in the row form only
            assert np.array_equal(np.isnan(yh), np.isnan(ref)), (lay, add)
            ok = ~np.isnan(ref)
            assert np.abs(yh[ok] - ref[ok]).max() <= 1e-13 * np.abs(ref[ok]).max()


@pytest.mark.parametrize("m,n", [(1, 1), (1, 9), (9, 1), (5, 3), (77, 40), (40, 77), (513, 1500),
                                 (3000, 257), (2049, 2049)])
@pytest.mark.parametrize("layout", ["F", "C", "S"])
def test_multmv_matches_oracle(dev, orc, m, n, layout):
    import torch

    from tmv_gb300 import linalg

    rng = np.random.default_rng(m * 7919 + n)
    a = rng.standard_normal((m, n))
    x = rng.standard_normal(n)
    y0 = rng.standard_normal(m)
    A = dev_matrix(a, dev, layout)
    if layout == "S":  # the same strided view on the host
        big = np.zeros((2 * m + 1, 3 * n + 2))
        big[: 2 * m : 2, : 3 * n : 3] = a
        Ah = big[: 2 * m : 2, : 3 * n : 3]
    else:
        Ah = np.asfortranarray(a) if layout == "F" else np.ascontiguousarray(a)
    for add, alpha in ((False, 1.0), (True, -0.75), (False, 2.5)):
        yo = y0.copy()
        orc.multmv(add, alpha, Ah, x, yo)
        y = torch.from_numpy(y0.copy()).to(dev)
        linalg.multmv(add, alpha, A, torch.from_numpy(x).to(dev), y)
        # FP64: 1e-13 of |alpha| |A| |x| (+ |y|), summation order differs
        scale = abs(alpha) * np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(y0).max()
        assert np.abs(to_host(y) - yo).max() <= 1e-13 * scale


def test_multmv_exact_integers_and_edges(dev):
    import torch

    from tmv_gb300 import linalg

    # integer operands of TMV's product test: every sum is exact in FP64
    a, b = arith8_operands(637, 300, 77)
    for lay in ("F", "C"):
        A = to_dev(a, dev, lay)
        x = torch.from_numpy(b[:, 0].copy()).to(dev)
        y = torch.empty(637, dtype=torch.float64, device=dev)
        linalg.multmv(False, 1.0, A, x, y)
        assert np.array_equal(to_host(y), a @ b[:, 0])
    # alpha = 0 leaves A unread (a NaN matrix): y = 0, or y unchanged with add
    A = torch.full((50, 30), float("nan"), dtype=torch.float64, device=dev)
    x = torch.ones(30, dtype=torch.float64, device=dev)
    y = torch.arange(50, dtype=torch.float64, device=dev)
    linalg.multmv(True, 0.0, A, x, y)
    assert np.array_equal(to_host(y), np.arange(50.0))
    linalg.multmv(False, 0.0, A, x, y)
    assert not to_host(y).any()
    # x and y sharing storage: y = A y
    rng = np.random.default_rng(5)
    a = rng.standard_normal((300, 300))
    v = rng.standard_normal(300)
    yv = torch.from_numpy(v.copy()).to(dev)
    linalg.multmv(False, 1.0, to_dev(a, dev, "F"), yv, yv)
    assert np.abs(to_host(yv) - a @ v).max() <= 1e-13 * np.abs(a @ v).max()


def test_tri_ldiveq_matches_tmv_special_cases(dev):
    import torch

    from tmv_gb300 import linalg
    from tmv_gb300._lib import SingularError

    g = np.load(GOLD / "multmv_tri.npz")
    U, b = g["tri_U"], g["tri_b"]
    Ud = to_dev(U, dev, "F")
    for name, B in (("v", to_dev(b[:, :1], dev, "F")), ("F", to_dev(b, dev, "F")), ("C", to_dev(b, dev, "C"))):
        if int(g[f"tri_{name}_rc"]) == 0:
            linalg.tri_ldiveq(Ud, True, False, B)
            torch.cuda.synchronize()
            assert rel_frob(to_host(B), g[f"tri_{name}"]) <= 1e-13, name
        else:
            with pytest.raises(SingularError):
                linalg.tri_ldiveq(Ud, True, False, B)


@pytest.mark.parametrize("n", [1, 7, 64, 65, 200, 700])
@pytest.mark.parametrize("nrhs", [1, 5, 100])
def test_tri_ldiveq_rdiveq_match_oracle(dev, orc, n, nrhs):
    from tmv_gb300 import linalg

    rng = np.random.default_rng(n * 131 + nrhs)
    T = np.asfortranarray(diag_shift_matrix(rng, n, 2.0 * np.sqrt(n)))
    Td = to_dev(T, dev, "F")
    for upper in (True, False):
        for unit in (True, False):
            b = rng.standard_normal((n, nrhs))
            for lay in ("F", "C"):
                Bo = np.array(b, order=lay, copy=True)  # b itself stays untouched
                assert orc.tri_ldiveq(upper, unit, T, Bo) == 0
                Bd = to_dev(b, dev, lay)
                linalg.tri_ldiveq(Td, upper, unit, Bd)
                assert rel_frob(to_host(Bd), Bo) <= 1e-12, (upper, unit, lay)
            # m %= T: X T = W, through the transposed triangle
            w = rng.standard_normal((nrhs, n))
            Wd = to_dev(w, dev, "F")
            linalg.tri_rdiveq(Td, upper, unit, Wd)
            Wt = np.array(w.T, order="F", copy=True)
            Tt = np.array(T.T, order="F", copy=True)
            assert orc.tri_ldiveq(not upper, unit, Tt, Wt) == 0
            assert rel_frob(to_host(Wd), Wt.T) <= 1e-12, (upper, unit, "rdiv")


def test_matrix_surface_tri_and_vector(dev):
    import torch

    from tmv_gb300.matrix import Matrix, UnitDiag

    rng = np.random.default_rng(8)
    a = diag_shift_matrix(rng, 120, 25.0)
    m = Matrix(a, device=dev)
    v = rng.standard_normal(120)
    y = m * torch.from_numpy(v).to(dev)
    assert np.abs(to_host(y) - a @ v).max() <= 1e-13 * np.abs(a @ v).max()
    b = rng.standard_normal((120, 4))
    X = (Matrix(b, device=dev) / m.upperTri()).numpy()
    assert rel_frob(np.triu(a) @ X, b) <= 1e-13
    # a unit-lower triangle with N(0,1) entries is exponentially ill
    # conditioned; scale its strict lower part
    low = np.tril(rng.standard_normal((120, 120)), -1) * (0.5 / np.sqrt(120)) + 7.0 * np.eye(120)
    L = np.tril(low, -1) + np.eye(120)
    Y = (Matrix(b.T.copy(), device=dev) % Matrix(low, device=dev).lowerTri(UnitDiag)).numpy()
    assert rel_frob(Y @ L, b.T) <= 1e-13


def test_multmv_full_size(dev):
    # A 8192 x 8192 (512 MiB): the refinement residual's operand size
    import torch

    from tmv_gb300 import linalg

    g = torch.Generator(device=dev).manual_seed(11)
    A = torch.randn((8192, 8192), dtype=torch.float64, device=dev, generator=g).t()  # column-major
    x = torch.randn(8192, dtype=torch.float64, device=dev, generator=g)
    y = torch.empty(8192, dtype=torch.float64, device=dev)
    linalg.multmv(False, 1.0, A, x, y)
    ref = A @ x
    assert (torch.linalg.norm(y - ref) / torch.linalg.norm(ref)).item() <= 1e-14
    yr = torch.empty(8192, dtype=torch.float64, device=dev)
    linalg.multmv(False, 1.0, A.t(), x, yr)  # row-major view
    ref2 = A.t() @ x
    assert (torch.linalg.norm(yr - ref2) / torch.linalg.norm(ref2)).item() <= 1e-14
