"""The W-cycle (elliptic::Wcycle, src/elliptic.cc:1348-1380: FASN with every
level repeated until its norm meets the tolerance) in the oracle, pinned
against the reference's own runs (tests/golden/wcycle, from its Olliptic.x
with -m Wcycle): the same sequence of level iterations with the same cycle
numbers and bit-identical norms (Loo.gp), the same cycle tables
(stdout0.out) and u.X, u.Y, u.Z digit for digit; the V-cycle's calls are
pinned the same way (tests/golden/vcycle)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem
from tests.test_oracle_approx import cut_points
from tests.wcycle_log import render_cycle_tables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "wcycle", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_wcycle_reprints_the_reference(path):
    g = np.load(path)
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    cycles, res = orc.solve_wcycle()
    assert cycles == 1 and res <= P.tol      # the top level's own loop met the tolerance
    ev = orc.events()
    pre = [(c, v) for _, post, c, v in ev if not post]
    assert [c for c, _ in pre] == list(g["loo_cycle"])
    assert np.array_equal(np.array([v for _, v in pre]), g["loo_norm"])
    text = render_cycle_tables(ev, orc.levels, P.tol)
    assert text == g["stdout_cycles"].item().decode()
    for name in ("u.X", "u.Y", "u.Z"):
        pts, want = cut_points(g, name)
        assert np.array_equal(orc.interpolate(pts, P.order + 1), want), name


def test_wcycle_and_vcycle_share_the_fixed_point(oracle_mod):
    """Both cycles solve the same discrete equations: solved far below the
    truncation error they agree on every solution level."""
    g = np.load(GOLDEN[0])
    P = problem(g["args"].item().decode())
    P.tol = 1e-13
    ow = oracle_mod.Oracle(P.oracle_dict())
    ow.solve_wcycle()
    ov = oracle_mod.Oracle(P.oracle_dict())
    ov.solve()
    for g_ in range(ow.nboxes):
        if ow.boxes[g_].level >= ow.mgrid_levels:
            assert np.max(np.abs(ow.field(g_, "u") - ov.field(g_, "u"))) < 1e-11


def test_wcycle_call_checker_accepts_the_reference_and_rejects_a_v_cycle(oracle_mod):
    """The call checker the GPU tests use, on the oracle's (reference-pinned)
    W-cycle calls, and on a V-cycle's, which it must reject."""
    from tests.wcycle_log import check_wcycle_calls
    g = np.load(GOLDEN[0])
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.solve_wcycle()
    iters = check_wcycle_calls(orc.events(), orc.levels, P.tol)
    assert iters[-1] == g["stdout_cycles"].item().decode().count("Cycle:")
    ov = oracle_mod.Oracle(P.oracle_dict())
    ov.solve()
    with pytest.raises(AssertionError):
        check_wcycle_calls(ov.events(), ov.levels, P.tol)


def test_oracle_vcycle_calls_reprint_the_reference(oracle_mod):
    """The V-cycle's print calls (pre-smoothing from the top down, the
    coarsest solve, post-smoothing back up, all with the cycle's number), the
    order the library logs for its V-cycles, give the reference's own Loo.gp
    and stdout0.out tables bit for bit (tests/golden/vcycle)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "vcycle", "o2_single.npz"))
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.solve()
    ev = orc.events()
    top = orc.levels - 1
    assert [(e[0], e[1]) for e in ev[:2 * top + 1]] == [(k, 0) for k in range(top, -1, -1)] + \
        [(k, 1) for k in range(1, top + 1)]
    pre = [(c, v) for _, post, c, v in ev if not post]
    assert [c for c, _ in pre] == list(g["loo_cycle"])
    assert np.array_equal(np.array([v for _, v in pre]), g["loo_norm"])
    assert render_cycle_tables(ev, orc.levels, P.tol) == g["stdout_cycles"].item().decode()
