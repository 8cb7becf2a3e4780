"""LU_Decompose / LU_LDivEq for complex<double> on the GPU against the
oracle's complex restatement (itself pinned to TMV's complex instantiations
and to tests/golden/complex_lu.npz)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a, dev):
    import torch

    return torch.from_numpy(np.asfortranarray(a)).to(dev).t().contiguous().t()


def _host(t):
    return np.asfortranarray(t.cpu().numpy())


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 64, 65, 127, 128, 130, 300, 1024, 1500])
def test_complex_lu_and_solve_match_oracle(dev, orc, n):
    import torch

    from tmv_gb300 import linalg

    rng = np.random.default_rng(700 + n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    lu_o = np.asfortranarray(a.copy())
    p_o = orc.lu_decompose_z(lu_o)
    A = _dev(a, dev)
    P = linalg.lu_decompose_z(A)
    torch.cuda.synchronize()
    assert np.array_equal(P.cpu().numpy(), p_o)
    assert np.abs(_host(A) - lu_o).max() <= 1e-12 * np.abs(lu_o).max()
    b = rng.standard_normal((n, 4)) + 1j * rng.standard_normal((n, 4))
    x_o = np.asfortranarray(b.copy())
    orc.ldiveq_z(lu_o, p_o, x_o)
    X = _dev(b, dev)
    linalg.lu_ldiveq_z(A, P, X)
    x = _host(X)
    assert np.abs(x - x_o).max() <= 1e-11 * np.abs(x_o).max()
    scale = np.abs(a).sum(axis=1).max() * np.abs(x).max()
    assert np.abs(a @ x - b).max() <= 1e-13 * scale


def test_complex_golden_and_pivot_rule(dev):
    # TMV's own complex factors and solutions, and the pivot-rule cases
    # (exact arithmetic: bitwise)
    from pathlib import Path

    import torch

    from tmv_gb300 import linalg

    g = np.load(Path(__file__).resolve().parent / "golden" / "complex_lu.npz")
    for n in [1, 4, 17, 65]:
        A = _dev(g[f"a{n}"], dev)
        P = linalg.lu_decompose_z(A)
        torch.cuda.synchronize()
        assert np.array_equal(P.cpu().numpy(), g[f"P{n}"]), n
        LU = g[f"LU{n}"]
        assert np.abs(_host(A) - LU).max() <= 1e-12 * np.abs(LU).max(), n
        X = _dev(g[f"b{n}"], dev)
        linalg.lu_ldiveq_z(A, P, X)
        assert np.abs(_host(X) - g[f"X{n}"]).max() <= 1e-11 * np.abs(g[f"X{n}"]).max(), n
    for q in range(3):
        A = _dev(g[f"s{q}"], dev)
        P = linalg.lu_decompose_z(A)
        torch.cuda.synchronize()
        assert np.array_equal(P.cpu().numpy(), g[f"sP{q}"])
        np.testing.assert_array_equal(_host(A), g[f"sLU{q}"])


def test_complex_singular_solve_raises(dev, orc):
    from tmv_gb300 import _lib, linalg

    a = np.array([[1 + 1j, 2, 0], [0, 0, 0], [3j, 1, 0]], dtype=np.complex128)  # zero column 2
    A = _dev(a, dev)
    P = linalg.lu_decompose_z(A)
    lu_o = np.asfortranarray(a.copy())
    p_o = orc.lu_decompose_z(lu_o)
    assert np.array_equal(P.cpu().numpy(), p_o)
    np.testing.assert_array_equal(_host(A), lu_o)
    X = _dev(np.ones((3, 1), dtype=np.complex128), dev)
    with pytest.raises(_lib.SingularError):
        linalg.lu_ldiveq_z(A, P, X)
    # the context stays usable
    Y = _dev(np.eye(3, dtype=np.complex128)[:, :1] * 0, dev)
    linalg.lu_ldiveq_z(A, P, Y)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 65, 130])
def test_complex_rdiveq_and_det_match_oracle(dev, orc, n):
    # b % m and det / logDet from the GPU factors, against the oracle's
    # restatement applied to the same factors
    import torch

    from tmv_gb300 import linalg

    rng = np.random.default_rng(800 + n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = _dev(a, dev)
    P = linalg.lu_decompose_z(A)
    torch.cuda.synchronize()
    lu, p = _host(A), P.cpu().numpy()
    for rows in [1, 3]:
        w = rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))
        y_o = np.asfortranarray(w.copy())
        orc.rdiveq_z(lu, p, y_o)
        Y = _dev(w, dev)
        linalg.lu_rdiveq_z(A, P, Y)
        y = _host(Y)
        # the same operations in the same order on the same factors
        np.testing.assert_array_equal(y, y_o)
        scale = np.abs(a).sum(axis=0).max() * np.abs(y).max()
        assert np.abs(y @ a - w).max() <= 1e-13 * scale
    det, logdet, sign = linalg.lu_det_z(A, P)
    d_o, l_o, s_o = orc.lu_det_z(lu, p)
    assert abs(det - d_o) <= 1e-13 * abs(d_o) and abs(logdet - l_o) <= 1e-13 * max(1.0, abs(l_o))
    assert abs(sign - s_o) <= 1e-14
    assert abs(det - np.linalg.det(a)) <= 1e-10 * abs(np.linalg.det(a))


def test_complex_rdiveq_golden_and_singular(dev):
    from pathlib import Path

    import torch

    from tmv_gb300 import _lib, linalg

    g = np.load(Path(__file__).resolve().parent / "golden" / "complex_lu.npz")
    for n in [1, 4, 17, 65]:
        A = _dev(g[f"a{n}"], dev)
        P = linalg.lu_decompose_z(A)
        Y = _dev(g[f"w{n}"], dev)
        linalg.lu_rdiveq_z(A, P, Y)
        torch.cuda.synchronize()
        assert np.abs(_host(Y) - g[f"Y{n}"]).max() <= 1e-11 * np.abs(g[f"Y{n}"]).max(), n
        det, logdet, sign = linalg.lu_det_z(A, P)
        # a product of n diagonal entries, each within rounding of TMV's
        assert abs(det - g[f"det{n}"][0]) <= 1e-11 * abs(g[f"det{n}"][0]), n
        assert abs(sign - g[f"sign{n}"][0]) <= 1e-11, n
    a = np.array([[1 + 1j, 2, 0], [0, 0, 0], [3j, 1, 0]], dtype=np.complex128)
    A = _dev(a, dev)
    P = linalg.lu_decompose_z(A)
    assert linalg.lu_det_z(A, P) == (0j, -np.inf, 0j)
    with pytest.raises(_lib.SingularError):
        linalg.lu_rdiveq_z(A, P, _dev(np.ones((1, 3), dtype=np.complex128), dev))


def test_complex_inverse_matches_tmv(dev):
    # m.inverse() against TMV's own (complex_lu.npz), A A^-1 = I, singular
    from pathlib import Path

    import torch

    from tmv_gb300 import _lib, linalg

    g = np.load(Path(__file__).resolve().parent / "golden" / "complex_lu.npz")
    for n in [1, 4, 17, 65]:
        a = g[f"a{n}"]
        A = _dev(a, dev)
        P = linalg.lu_decompose_z(A)
        M = linalg.lu_inverse_z(A, P)
        torch.cuda.synchronize()
        m = _host(M)
        inv = g[f"inv{n}"]
        assert np.abs(m - inv).max() <= 1e-11 * np.abs(inv).max(), n
        assert np.abs(a @ m - np.eye(n)).max() <= 1e-12 * np.abs(a).sum(axis=1).max() * np.abs(m).max() * n
    a = np.array([[1 + 1j, 2, 0], [0, 0, 0], [3j, 1, 0]], dtype=np.complex128)
    A = _dev(a, dev)
    P = linalg.lu_decompose_z(A)
    with pytest.raises(_lib.SingularError):
        linalg.lu_inverse_z(A, P)


def test_complex_lu_narrow_panel_large(dev):
    """n = 6400 takes the 16-column panels (a 32-column panel's rows exceed
    shared memory): P L U = A to rounding, |L| <= 1 (partial pivoting), and a
    solve's normwise backward error at most 1e-14."""
    import torch

    from tmv_gb300 import linalg

    n = 6400
    g = torch.Generator(device=dev).manual_seed(21)
    A = torch.complex(torch.randn((n, n), dtype=torch.float64, device=dev, generator=g),
                      torch.randn((n, n), dtype=torch.float64, device=dev, generator=g))
    A = A.t().contiguous().t()
    LU = A.clone()
    P = linalg.lu_decompose_z(LU)
    b = torch.complex(torch.randn((n, 2), dtype=torch.float64, device=dev, generator=g),
                      torch.randn((n, 2), dtype=torch.float64, device=dev, generator=g)).t().contiguous().t()
    x = b.clone()
    linalg.lu_ldiveq_z(LU, P, x)
    Pc = P.cpu().numpy()
    assert (Pc >= np.arange(n)).all() and (Pc < n).all()
    L = torch.tril(LU, -1)
    assert float(L.abs().max()) <= 1.0 + 1e-12
    berr = float((A @ x - b).abs().max() / (A.abs().sum(dim=1).max() * x.abs().max()))
    assert berr <= 1e-14, berr
