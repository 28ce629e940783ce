"""The oracle's printed-cut interpolation (orc_interpolate) pinned against the
reference itself: the oracle solves the golden runs' problems with the
reference's algorithm and stop rule (its iterates are the reference's bit for
bit), and its values at the points of the reference's u.X, u.Y, u.Z and u.XY
are the ones the reference printed, to all 18 printed digits."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = [p for p in sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "output", "*.npz")))
          if "u.X__text" in np.load(p).files]


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reprints_the_reference_cuts(path):
    g = np.load(path)
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.solve()
    for name, axis in (("u.X", 0), ("u.Y", 1), ("u.Z", 2), ("u.XY", None)):
        text, vals = g[name + "__text"], g[name + "__vals"]
        rows = [i for i in range(len(text)) if text[i]]
        pts = np.zeros((len(rows), 3))
        for q, i in enumerate(rows):
            c = [float(t) for t in text[i].decode().split("\t")]
            if axis is None:
                pts[q, 0], pts[q, 1] = c
            else:
                pts[q, axis] = c[0]
        got = orc.interpolate(pts, P.order + 1)
        assert not np.isnan(got).any()
        assert np.array_equal(got, vals[rows]), name


@pytest.mark.parametrize("case", ["o2_spin_l4", "o4_spin_l4"])
def test_oracle_reprints_the_reference_convergence_run(case):
    """The coarsest run of the convergence study (N = 25): the oracle's
    solve under the reference's stop rule and its u.X cut are the
    reference's, digit for digit."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "convergence", case + ".npz"))
    P = problem(g["args"].item().decode() + " -N 25")
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.solve()
    x = g["x_25"]
    got = orc.interpolate(np.stack([x, 0 * x, 0 * x], axis=1), P.order + 1)
    assert np.array_equal(got, g["u_25"])
