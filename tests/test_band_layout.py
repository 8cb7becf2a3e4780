"""Host-side band helpers on the CPU: the packed layout of a band batch
(TMV's column-major band storage: hu = min(lo+hi, n-1), ldab = lo + hu,
n (ldab + 1) slots per system), the algorithmic work the benchmark reports,
and the test helpers' pack / unpack round trip."""
import numpy as np

from tests.helpers import band_hu, band_matrix, band_pack, band_unpack
from tmv_gb300.band import band_layout, band_lu_solve_count


def test_packed_layout():
    lay = band_layout(1024, 2, 2)
    assert (lay.hu, lay.ldab, lay.stride_ab) == (4, 6, 1024 * 7)
    assert lay.slots == 1023 * 7 + 1
    tri = band_layout(1024, 1, 1)
    assert (tri.hu, tri.ldab, tri.stride_ab) == (2, 3, 4096)
    # hu is capped by n - 1; a diagonal band still has one slot per column
    small = band_layout(3, 2, 2)
    assert (small.hu, small.ldab) == (2, 4)
    diag = band_layout(5, 0, 0)
    assert (diag.hu, diag.ldab, diag.stride_ab) == (0, 1, 10)
    assert band_layout(8, 1, 1, ldab=7, stride_ab=100).stride_ab == 100


def test_solve_count_matches_enumeration():
    for n, lo, hi in [(9, 1, 1), (20, 2, 3), (5, 4, 4)]:
        lay = band_layout(n, lo, hi)
        w = band_lu_solve_count(3, lay, 2)
        hu = lay.hu
        slots = sum(1 for j in range(n) for i in range(n) if j - hu <= i <= j + lo)
        assert w["bytes"] == 3 * (8 * 2 * slots + 8 * n + 8 * 2 * n * 2)
        assert w["flops"] == 3 * (n * (1 + lo + 2 * lo * hu) + 2 * n * (2 * (lo + hu) + 1))


def test_pack_unpack_round_trip():
    rng = np.random.default_rng(3)
    for n, lo, hi in [(1, 0, 0), (6, 1, 1), (12, 3, 2), (12, 0, 4)]:
        a = band_matrix(rng, n, lo, hi)
        hu = band_hu(n, lo, hi)
        ab = band_pack(a, lo, hi, lo + hu if lo + hu > 0 else 1)
        back = band_unpack(ab, n, lo, hu, lo + hu if lo + hu > 0 else 1)
        # the fill diagonals hi+1..hu hold the packing's fill value (0)
        assert np.array_equal(back, a)
