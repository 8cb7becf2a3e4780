"""The GPU path against outputs of TMV itself (tests/golden/, made by
tests/golden/make_golden.py from TMV 0.76 compiled from its sources)."""
from pathlib import Path

import numpy as np
import pytest

from helpers import arith8_operands, rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    return np.load(GOLD / name, allow_pickle=False)


def gpu_lu(dev, a):
    import torch

    from tmv_gb300 import linalg

    A = to_dev(a, dev, "F")
    P = linalg.lu_decompose(A)
    torch.cuda.synchronize()
    return to_host(A), to_host(P)


def test_arith8_stored_products(dev):
    import torch

    from tmv_gb300 import linalg

    g = load("arith8.npz")
    for key in [k for k in g.files if k.startswith("C_")]:
        m, n, k, lay = key[2:].split("_")
        m, n, k = int(m), int(n), int(k)
        a, b = arith8_operands(m, n, k)
        C = torch.zeros((n, m), dtype=torch.float64, device=dev).t()
        linalg.multmm(False, 1.0, to_dev(a, dev, lay[0]), to_dev(b, dev, lay[1]), C)
        assert np.array_equal(to_host(C), g[key]), key


def test_square4_and_bign100(dev):
    import torch

    from tmv_gb300 import linalg

    for name, mkey, bkey in [("square4.npz", "m", "b"), ("bign100.npz", "M", "R")]:
        g = load(name)
        m = g[mkey]
        lu, p = gpu_lu(dev, m)
        assert np.array_equal(p, g["P"]), name
        assert np.abs(lu - g["LU"]).max() <= 1e-12 * np.abs(g["LU"]).max(), name
        n = m.shape[0]
        X, LU, P = linalg.divide(to_dev(m, dev, "F"), to_dev(g[bkey].reshape(n, 1), dev, "F"))
        assert rel_frob(to_host(X), g["X"]) <= 1e-12, name
        Y = to_dev(g[bkey].reshape(1, n), dev, "F")
        linalg.lu_rdiveq(LU, P, Y)
        assert rel_frob(to_host(Y), g["Y"]) <= 1e-12, name
    g = load("square4.npz")
    LU = to_dev(g["LU"], dev, "F")
    det, logdet, sign = linalg.lu_det(LU, torch.from_numpy(g["P"]).to(dev))
    assert abs(det - float(g["det"])) <= 1e-10 * 28800 and sign == 1.0


def test_random_and_special(dev):
    g = load("random_lu.npz")
    for n in [1, 2, 3, 4, 5, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129]:
        lu, p = gpu_lu(dev, g[f"A{n}"])
        assert np.array_equal(p, g[f"P{n}"]), n
        if f"LU{n}" in g.files:
            assert np.abs(lu - g[f"LU{n}"]).max() <= 1e-12 * max(np.abs(g[f"LU{n}"]).max(), 1), n
    s = load("special.npz")
    for name in sorted(k[2:] for k in s.files if k.startswith("A_")):
        lu, p = gpu_lu(dev, s["A_" + name])
        assert np.array_equal(p, s["P_" + name]), name
        ref = s["LU_" + name]
        assert np.array_equal(np.isnan(lu), np.isnan(ref)), name
        ok = ~np.isnan(ref)
        scale = max(np.abs(ref[ok]).max() if ok.any() else 1.0, 1.0)
        assert np.abs(lu[ok] - ref[ok]).max() <= 1e-12 * scale, name


def test_decomp200_reconstruction(dev):
    g = load("decomp200.npz")
    for mt in (0, 3):
        lu, p = gpu_lu(dev, g[f"m{mt}"])
        k = 200 if mt == 0 else 5
        assert np.array_equal(p[:k], g[f"P{mt}"][:k]), mt
