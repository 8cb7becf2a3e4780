"""The LU look-ahead (panel k+1 on a side stream while step k's update runs)
gives bitwise the same results under an extreme interleaving of the streams.

TMVG_SERIALIZE_LOOKAHEAD=1 makes every side-stream panel finish before the
main stream issues its next launch.  Every kernel of the factorisation is
deterministic, so any cross-stream dependency the library missed shows up as
a bitwise difference from the ordinary (overlapped) run, or as a failed
refinement.
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
sys.path.insert(0, sys.argv[1])
from tmv_gb300 import linalg
n, out = int(sys.argv[2]), sys.argv[3]
rng = np.random.default_rng(5)
a = rng.standard_normal((n, n))
b = rng.standard_normal((n, 1))
dev = torch.device("cuda:0")
A = torch.from_numpy(np.asfortranarray(a)).to(dev).t().contiguous().t()
LU = A.clone()
P = linalg.lu_decompose(LU)
a2 = a + 2.0 * np.sqrt(n) * np.eye(n)
A2 = torch.from_numpy(np.asfortranarray(a2)).to(dev).t().contiguous().t()
B = torch.from_numpy(b).to(dev)
X, info = linalg.solve_mixed(A2, B, max_iter=10, tol=1e-12)
torch.cuda.synchronize()
np.savez(out, lu=LU.cpu().numpy(), p=P.cpu().numpy(), x=X.cpu().numpy(),
         conv=np.array([info.converged, info.iterations]))
"""


def run(tmp_path, n, serialize):
    out = tmp_path / f"la_{n}_{int(serialize)}.npz"
    env = dict(os.environ)
    env["TMVG_SERIALIZE_LOOKAHEAD"] = "1" if serialize else "0"
    subprocess.run([sys.executable, "-c", RUN, str(ROOT), str(n), str(out)], check=True, env=env,
                   timeout=600)
    return np.load(out)


@pytest.mark.parametrize("n", [1000, 4096])
def test_serialized_lookahead_is_bitwise_identical(tmp_path, dev, orc, n):
    ref = run(tmp_path, n, serialize=False)
    ser = run(tmp_path, n, serialize=True)
    assert np.array_equal(ref["p"], ser["p"])
    assert np.array_equal(ref["lu"], ser["lu"])
    assert np.array_equal(ref["x"], ser["x"])
    assert ref["conv"][0] == 1 and ser["conv"][0] == 1
    if n <= 1000:
        # and both are TMV's factorisation
        rng = np.random.default_rng(5)
        a = rng.standard_normal((n, n))
        lu_o = np.asfortranarray(a.copy())
        p_o = orc.lu_decompose(lu_o)
        assert np.array_equal(ref["p"], p_o)
        assert np.abs(ref["lu"] - lu_o).max() <= 1e-11 * np.abs(lu_o).max()
