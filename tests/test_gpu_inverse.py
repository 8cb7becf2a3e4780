"""m.inverse(), m.makeInverseATA() and m.isSingular() on the GPU.

LU_Inverse (src/TMV_LUInverse.cpp:236-299), LUDiv::doMakeInverseATA and
LUDiv::isSingular (src/TMV_LUD.cpp:172-209) through the C ABI, against TMV's
own results (tests/golden/inverse.npz) and the oracle; at n = 4096 (the
dense-solve workload's matrix) through A * A^-1 = I and the symmetry of
(A^T A)^-1.
"""
from pathlib import Path

import numpy as np
import pytest

from helpers import diag_shift_matrix, rel_frob, to_dev, to_host

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def factors(dev, a):
    from tmv_gb300 import linalg

    A = to_dev(a, dev, "F")
    P = linalg.lu_decompose(A)
    return A, P


def test_inverse_matches_tmv_fixtures(dev):
    from tmv_gb300 import linalg
    from tmv_gb300._lib import TmvgError

    g = np.load(GOLD / "inverse.npz")
    for name in ["sq4", "r96", "sing6"]:
        LU, P = factors(dev, g[name])
        assert linalg.lu_is_singular(LU) == bool(g[name + "_singular"]), name
        if int(g[name + "_rc"]) == 0:
            # FP64: 1e-12 relative Frobenius against TMV's inverse
            assert rel_frob(to_host(linalg.lu_inverse(LU, P)), g[name + "_inv"]) <= 1e-12, name
            assert rel_frob(to_host(linalg.lu_inverse_ata(LU)), g[name + "_ata"]) <= 1e-12, name
        elif (to_host(LU).diagonal() == 0).any():
            # an exact zero U(j,j): TMV throws SingularUpperTriMatrix
            with pytest.raises(TmvgError) as e:
                linalg.lu_inverse(LU, P)
            assert e.value.status == 1  # TMVG_SINGULAR


@pytest.mark.parametrize("n", [1, 2, 5, 63, 64, 65, 130, 257, 600])
def test_inverse_matches_oracle(dev, orc, n):
    from tmv_gb300 import linalg

    rng = np.random.default_rng(4400 + n)
    a = diag_shift_matrix(rng, n, 2.0 * np.sqrt(n))
    LU, P = factors(dev, a)
    lu_h, p_h = to_host(LU), to_host(P)
    LUo = np.asfortranarray(a.copy())
    Po = orc.lu_decompose(LUo)
    assert np.array_equal(p_h, Po)
    inv_o = orc.lu_inverse(LUo, Po)
    ata_o = orc.lu_inverse_ata(LUo)
    inv_g = to_host(linalg.lu_inverse(LU, P))
    ata_g = to_host(linalg.lu_inverse_ata(LU))
    assert rel_frob(inv_g, inv_o) <= 1e-12
    assert rel_frob(ata_g, ata_o) <= 1e-12
    assert linalg.lu_is_singular(LU) == orc.lu_is_singular(lu_h)
    # the same inverse twice: no state carried between calls
    assert np.array_equal(to_host(linalg.lu_inverse(LU, P)), inv_g)


def test_inverse_full_size_properties(dev):
    # n = 4096 with 4 sqrt(n) on the diagonal (the FP64 LU workload's
    # matrix): ||A A^-1 - I||_F <= 1e-12 sqrt(n), (A^T A)^-1 symmetric and
    # equal to A^-1 A^-T
    import torch

    from tmv_gb300 import linalg

    n = 4096
    rng = np.random.default_rng(20240610)
    a = diag_shift_matrix(rng, n, 4.0 * np.sqrt(n))
    A = to_dev(a, dev, "F")
    LU = to_dev(a, dev, "F")
    P = linalg.lu_decompose(LU)
    Ainv = linalg.lu_inverse(LU, P)
    eye = torch.eye(n, dtype=torch.float64, device=dev)
    r = torch.linalg.norm(A @ Ainv - eye).item()
    assert r <= 1e-12 * np.sqrt(n), r
    ata = linalg.lu_inverse_ata(LU)
    ref = Ainv @ Ainv.t()
    assert (torch.linalg.norm(ata - ref) / torch.linalg.norm(ref)).item() <= 1e-12
    assert (torch.linalg.norm(ata - ata.t()) / torch.linalg.norm(ata)).item() <= 1e-13


def test_matrix_surface_inverse(dev):
    # the tmv::Matrix mirror: m.inverse(), m.makeInverseATA(), m.isSingular()
    from helpers import tmv_square4
    from tmv_gb300.matrix import LU, Matrix

    m4, _ = tmv_square4()
    m = Matrix(m4, device=dev)
    m.divideUsing(LU)
    m.saveDiv()
    inv = m.inverse().numpy()
    assert np.abs(m4 @ inv - np.eye(4)).max() < 1e-14
    assert abs(m.det() - 28800.0) < 1e-9
    assert not m.isSingular()
    ata = m.makeInverseATA().numpy()
    assert rel_frob(ata, np.linalg.inv(m4.T @ m4)) <= 1e-12
