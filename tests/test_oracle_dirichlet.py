"""The Dirichlet boundary (the reference's default without -B) in the
oracle, pinned against the reference: its solve runs the reference's cycles
and reprints the reference's u.X, u.Y, u.Z digit for digit
(tests/golden/dirichlet, from its Olliptic.x)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem
from tests.test_oracle_approx import cut_points

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "dirichlet", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reprints_the_reference_dirichlet_runs(path):
    g = np.load(path)
    P = problem(g["args"].item().decode())
    assert P.boundary == "Dirichlet"
    orc = oracle_mod.Oracle(P.oracle_dict())
    cycles, _ = orc.solve()
    assert cycles == int(g["cycles"])
    for name in ("u.X", "u.Y", "u.Z"):
        pts, want = cut_points(g, name)
        assert np.array_equal(orc.interpolate(pts, P.order + 1), want), name
