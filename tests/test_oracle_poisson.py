"""The reference's Gaussian test (-eq Poisson), a known answer on the same
FAS path: the oracle's solve under the reference's stop rule runs the
reference's cycles and reprints its u.X, u.Y, u.Z digit for digit
(tests/golden/poisson, from the reference's Olliptic.x)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "poisson", "*.npz")))


def cut(g, name, N):
    text, vals = g[f"{name}_{N}__text"], g[f"{name}_{N}__vals"]
    rows = [i for i in range(len(text)) if text[i]]
    pts = np.zeros((len(rows), 3))
    pts[:, "XYZ".index(name[-1])] = [float(text[i]) for i in rows]
    return pts, vals[rows]


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reprints_the_reference_gaussian_test(path):
    g = np.load(path)
    N = int(g["resolutions"][0])
    P = problem(g["args"].item().decode() + f" -N {N}")
    orc = oracle_mod.Oracle(P.oracle_dict())
    cycles, _ = orc.solve()
    assert cycles == int(g[f"cycles_{N}"])
    for name in ("u.X", "u.Y", "u.Z"):
        pts, want = cut(g, name, N)
        assert np.array_equal(orc.interpolate(pts, P.order + 1), want), name
