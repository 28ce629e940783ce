"""Convergence order across resolutions, the reference's utils/run_conv.sh
study: one spinning puncture solved at N = 25, 49, 97 on the GPU (plain FP64
and mixed precision), u read at the points of the reference's u.X, and the
self-convergence order p of |u_h - u_h/2| ~ h^p away from the puncture
compared with the order of the reference's own runs
(tests/golden/convergence/*.npz, from its Olliptic.x)."""
import glob
import os

import numpy as np
import pytest

from ollipticid_gb300 import _abi
from tests.cases import problem
from tests.golden.make_convergence_golden import orders

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "convergence", "*.npz")))

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_convergence_order_matches_the_reference(path, mixed):
    import ollipticid_gb300 as og
    g = np.load(path)
    args = g["args"].item().decode()
    x = g["x_25"]
    pts = np.stack([x, np.zeros_like(x), np.zeros_like(x)], axis=1)
    cuts = []
    for N in g["resolutions"]:
        with og.Elliptic(problem(args + f" -N {int(N)}")) as E:
            E.set_precision(mixed)
            rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=300, tol=1e-11)
            assert rep.final_res <= 1e-11
            u = E.interpolate(pts)
        # the reference stops by its own rule at a residual near 1e-7, about
        # 3e-7 in u from the discrete solution the GPU converges to
        assert np.max(np.abs(u - g[f"u_{int(N)}"])) <= 2e-6
        cuts.append(u)
    p_inf, p_l2 = orders(x, *cuts)
    assert abs(p_inf - float(g["p_inf"])) <= 0.02, (p_inf, float(g["p_inf"]))
    assert abs(p_l2 - float(g["p_l2"])) <= 0.02, (p_l2, float(g["p_l2"]))
