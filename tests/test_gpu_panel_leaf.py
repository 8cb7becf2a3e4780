"""The leaf register panel (lu_panel_leaf_kernel) against the column-by-column
register panel (lu_panel_cluster_reg2_kernel): bitwise the same factors,
pivots and solutions.

The leaf panel factors eight columns at a time with rank-1 updates inside the
leaf and one rank-8 update of the columns after it, keeps rows in place and
tracks their positions; every entry still receives TMV's subtractions in
TMV's order, so nothing may differ.  TMVG_PANEL_REG2=1 (read when a handle is
created) selects the column-by-column kernel.  Each run is a fresh process
over the same inputs: the FP64 factorisation of random matrices of sizes that
run in one CTA and on the 16-CTA cluster, of matrices whose pivot decisions
meet TMV's special rules (zero and underflowing columns, ties, NaNs, a
rank-deficient matrix of TMV's tests), and the mixed solve, whose FP32
factorisation uses the same panel.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

RUN = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
from tmv_gb300 import linalg
from helpers import to_dev, to_host, tmv_decomp_matrix
out = {}
dev = torch.device("cuda:0")
def lu(name, a):
    A = to_dev(a, dev, "F")
    P = linalg.lu_decompose(A)
    torch.cuda.synchronize()
    out["lu_" + name], out["p_" + name] = to_host(A), to_host(P)
rng = np.random.default_rng(11)
for n in (100, 512, 513, 700, 1000, 2049, 4096):
    lu(f"rand{n}", rng.standard_normal((n, n)))
n = 1100
a = rng.standard_normal((n, n)); a[:, 9] = 0.0; a[:, 70] = 0.0; a[40] = a[12]
lu("zerocols", a)
a = rng.standard_normal((n, n)); a[:, 5] = 1e-310 * rng.standard_normal(n); a[:, 77] = 1e-310 * rng.standard_normal(n)
lu("underflow", a)
a = rng.standard_normal((n, n)); a[:, 0] = 0.5; a[[7, 20, 33], 0] = [-3.0, 3.0, -3.0]; a[:, 13] = 0.25
lu("ties", a)
for where in [(0, 0), (3, 0), (1, 1), (6, 1), (40, 35), (100, 100), (700, 3)]:
    a = rng.standard_normal((n, n)); a[where] = np.nan
    lu(f"nan_{where[0]}_{where[1]}", a)
lu("decomp3", tmv_decomp_matrix(3, 600))
lu("int", (np.arange(n)[:, None] * 7 % 13 - np.arange(n)[None, :] * 5 % 11).astype(np.float64))
for n in (1000, 4096):
    q1, _ = np.linalg.qr(rng.standard_normal((n, n)))
    q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    a = (q1 * np.logspace(0, -6, n)) @ q2.T
    b = rng.standard_normal((n, 2))
    X, info = linalg.solve_mixed(to_dev(a, dev, "F"), to_dev(b, dev, "F"))
    out[f"x_mixed{n}"] = to_host(X)
    out[f"it_mixed{n}"] = np.array([info.iterations, info.converged])
np.savez(sys.argv[2], **out)
"""


def run(tmp_path, reg2):
    out = tmp_path / f"panel_{int(reg2)}.npz"
    env = dict(os.environ, TMVG_PANEL_REG2="1" if reg2 else "0")
    subprocess.run([sys.executable, "-c", RUN, str(ROOT), str(out)], check=True, env=env, timeout=900)
    return np.load(out)


def test_leaf_panel_is_bitwise_the_column_panel(tmp_path, dev):
    leaf = run(tmp_path, reg2=False)
    col = run(tmp_path, reg2=True)
    assert sorted(leaf.files) == sorted(col.files)
    for name in leaf.files:
        assert np.array_equal(leaf[name], col[name], equal_nan=True), name
    assert leaf["it_mixed4096"][1] == 1
