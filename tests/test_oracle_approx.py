"""The oracle's analytic puncture approximation (elliptic::ApproximateID)
pinned against the reference itself: on the same hierarchy, its u at the
points of the reference's printed u.X, u.Y, u.Z and u.XY is the value the
reference printed, to all 18 digits."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "approx", "*.npz")))


def cut_points(g, name):
    text = g[name + "__text"]
    rows = [i for i in range(len(text)) if text[i]]
    pts = np.zeros((len(rows), 3))
    for q, i in enumerate(rows):
        c = [float(t) for t in text[i].decode().split("\t")]
        if name == "u.XY":
            pts[q, :2] = c
        else:
            pts[q, "XYZ".index(name[-1])] = c[0]
    return pts, g[name + "__vals"][rows]


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reprints_the_reference_approximation(path):
    g = np.load(path)
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.approximate_id()
    for name in ("u.X", "u.Y", "u.Z", "u.XY"):
        pts, want = cut_points(g, name)
        got = orc.interpolate(pts, P.order + 1, first_level=orc.mgrid_levels)
        assert np.array_equal(got, want), name
