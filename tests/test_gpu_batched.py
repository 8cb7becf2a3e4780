"""Batched uneven LU solves (one persistent launch) against TMV and the oracle."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def make_batch(rng, count, nmin, nmax, rmin, rmax, shift=2.0):
    n = rng.integers(nmin, nmax + 1, size=count).astype(np.int64)
    r = rng.integers(rmin, rmax + 1, size=count).astype(np.int64)
    a_off = np.concatenate([[0], np.cumsum(n * n)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(n * r)[:-1]]).astype(np.int64)
    A = np.zeros(int((n * n).sum()))
    B = np.zeros(int((n * r).sum()))
    for s in range(count):
        a = rng.standard_normal((n[s], n[s])) + shift * np.sqrt(n[s]) * np.eye(n[s])
        A[a_off[s]:a_off[s] + n[s] * n[s]] = a.ravel(order="F")
        B[b_off[s]:b_off[s] + n[s] * r[s]] = rng.standard_normal(n[s] * r[s])
    return n, r, a_off, b_off, A, B


def run(dev, n, r, A, B, tiles=None, tune=False):
    import torch

    from tmv_gb300.batched import BatchPlan

    plan = BatchPlan(n, r, tune=tune)
    if tiles is not None:
        plan.set_tiles(tiles)
    dA = torch.from_numpy(A.copy()).to(dev)
    dB = torch.from_numpy(B.copy()).to(dev)
    P, st = plan.solve(dA, dB)
    torch.cuda.synchronize()
    out = dA.cpu().numpy(), dB.cpu().numpy(), P.cpu().numpy(), st.cpu().numpy(), plan
    plan.close()
    return out


def test_golden_batch_matches_tmv(dev):
    g = np.load(GOLD / "batched_small.npz")
    LU, X, P, st, _ = run(dev, g["n"], g["nrhs"], g["A"], g["B"])
    assert not st.any()
    assert np.abs(X - g["X"]).max() <= 1e-12 * np.abs(g["X"]).max()


@pytest.mark.parametrize("tiles", [(8, 8, 8, 8), (16, 16, 16, 16), (8, 16, 8, 16)])
def test_random_batch_vs_oracle(dev, orc, tiles):
    rng = np.random.default_rng(10)
    n, r, a_off, b_off, A, B = make_batch(rng, 120, 1, 256, 0, 16, shift=0.0)
    LU, X, P, st, plan = run(dev, n, r, A, B, tiles=tiles)
    p_off = np.concatenate([[0], np.cumsum(n)[:-1]])
    for s in range(len(n)):
        ns, rs = int(n[s]), int(r[s])
        a = A[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F")
        lu_o = np.asfortranarray(a.copy())
        p_o = orc.lu_decompose(lu_o)
        assert np.array_equal(P[p_off[s]:p_off[s] + ns], p_o), s
        lu_g = LU[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F")
        assert np.abs(lu_g - lu_o).max() <= 1e-11 * max(np.abs(lu_o).max(), 1.0), s
        if rs:
            x_o = np.asfortranarray(B[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F"))
            orc.ldiveq(lu_o, p_o, x_o)
            x_g = X[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
            assert np.abs(x_g - x_o).max() <= 1e-10 * max(np.abs(x_o).max(), 1.0), s
    assert not st.any()


def test_singular_member_flags_only_itself(dev):
    rng = np.random.default_rng(11)
    n, r, a_off, b_off, A, B = make_batch(rng, 30, 8, 40, 1, 3)
    s = 7
    ns = int(n[s])
    blk = A[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F")
    blk[:, 3] = 0.0  # zero column: U(3,3) = 0, solve divides a nonzero by it
    A[a_off[s]:a_off[s] + ns * ns] = blk.ravel(order="F")
    LU, X, P, st, _ = run(dev, n, r, A, B)
    assert st[s] == 1 and st.sum() == 1


def test_autotuned_plan_and_workload_properties(dev, orc):
    # the batched workload's distribution (n in [8,256], nrhs in [1,16],
    # N(0,1) + 2 sqrt(n) I) at reduced count, with the autotuner on
    rng = np.random.default_rng(12)
    n, r, a_off, b_off, A, B = make_batch(rng, 600, 8, 256, 1, 16)
    LU, X, P, st, plan = run(dev, n, r, A, B, tune=True)
    assert set(plan.panel_widths) <= {8, 16}
    assert not st.any()
    # backward error of every system
    worst = 0.0
    for s in range(len(n)):
        ns, rs = int(n[s]), int(r[s])
        a = A[a_off[s]:a_off[s] + ns * ns].reshape(ns, ns, order="F")
        b = B[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
        x = X[b_off[s]:b_off[s] + ns * rs].reshape(ns, rs, order="F")
        res = np.abs(b - a @ x).max()
        worst = max(worst, res / (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max()))
    assert worst <= 1e-15
    # X matches TMV's per-system solve (oracle batch)
    Xo = B.copy()
    assert not orc.batched_divide(n, r, a_off, b_off, A.copy(), Xo).any()
    assert np.abs(X - Xo).max() <= 1e-12 * np.abs(Xo).max()


def test_tuned_widths_persist_per_device(dev, tmp_path, monkeypatch):
    """The tuner writes its widths to the table named by TMVG_TUNE_CACHE
    (keyed by SM count, size class and device name) and a later plan on the
    same device takes them from there without timing."""
    from tmv_gb300.batched import BatchPlan

    table = tmp_path / "tune.txt"
    monkeypatch.setenv("TMVG_TUNE_CACHE", str(table))
    n = np.array([20, 40, 100, 200] * 8)
    r = np.ones_like(n)
    plan = BatchPlan(n, r, tune=True)
    widths = plan.panel_widths
    plan.close()
    lines = [l.split() for l in table.read_text().splitlines() if l.strip()]
    assert len(lines) == 4  # one entry per size class present
    for l in lines:
        assert int(l[2]) in (8, 16) and int(l[2]) == widths[int(l[1])]
    # rewrite the table: the next plan must take these widths, untimed
    forced = [(l[0], l[1], "8" if l[2] == "16" else "16", l[3], " ".join(l[4:])) for l in lines]
    table.write_text("".join(" ".join(f) + "\n" for f in forced))
    plan = BatchPlan(n, r, tune=True)
    assert plan.panel_widths == [int(f[2]) for f in sorted(forced, key=lambda f: int(f[1]))]
    plan.close()
    monkeypatch.setenv("TMVG_TUNE_CACHE", "off")
