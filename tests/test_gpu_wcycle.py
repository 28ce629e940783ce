"""The W-cycle (elliptic::Wcycle, src/elliptic.cc:1348-1380) on the GPU.
Through the C ABI: one top-level call whose level iterations follow the
reference's nesting (each level repeats until its own norm meets the
tolerance), the oracle's fixed point, the oracle's ADM mass; mixed precision,
olgpu_cycle_launch and olgpu_solve_many refuse it.  Through Olliptic_gpu.x
-m Wcycle: the reference's printed cuts (tests/golden/wcycle, from its
Olliptic.x), Loo.gp holding every pre-smoothing call and stdout0.out's
tables rendered from the same calls."""
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem
from tests.test_gpu_output import box_levels
from tests.test_oracle_approx import cut_points
from tests.wcycle_log import check_wcycle_calls, render_cycle_tables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "wcycle", "*.npz")))
BANNER_END = "  Init Multigrid iteration\n"

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_wcycle_solve_through_the_abi(path):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    g = np.load(path)
    P = problem(g["args"].item().decode())
    P.method = "Wcycle"
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.solve_wcycle()
    with og.Elliptic(P) as E:
        rep = E.Solve(max_cycles=300)      # also caps each level's loop
        assert rep.status == 0 and rep.cycles == 1 and rep.final_res <= P.tol
        iters = check_wcycle_calls(E.cycle_events(), E.levels, P.tol)
        assert all(n >= 1 for n in iters[1:])
        adm = E.ADM_mass
        with pytest.raises(_abi.OlgpuError):
            E.set_precision(True)
        with pytest.raises(_abi.OlgpuError):
            E.cycle_launch()
    for a, b in zip(adm, orc.adm()):
        assert abs(a - b) <= 1e-8 * abs(b)


def test_wcycle_fixed_point_is_the_oracles():
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    g = np.load(GOLDEN[0])
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.fixed_point()
    u_fix = orc.all_u()
    P.method = "Wcycle"
    with og.Elliptic(P) as E:
        rep = E.Solve(max_cycles=200, tol=1e-12)
        assert rep.status == 0 and rep.final_res <= 1e-12
        sol = [b for b, box in enumerate(E.boxes) if box.level >= E.mgrid_levels]
        err = max(float(np.max(np.abs(E.get_field(b).ravel() - u_fix[b].ravel()))) for b in sol)
    assert err <= 1e-10, err


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_cli_wcycle_matches_the_reference(path, tmp_path):
    g = np.load(path)
    args = g["args"].item().decode()
    r = subprocess.run([CLI] + args.split() + ["-m", "Wcycle", "-o", "Output"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "Solved in 1 W-cycles" in r.stdout
    mg = int(re.search(r"\((\d+) multigrid\)", r.stdout).group(1))
    level_of = box_levels(args)
    for name in ("u.X", "u.Y", "u.Z"):
        ours = np.loadtxt(tmp_path / "Output" / name)
        pts, want = cut_points(g, name)
        assert np.array_equal(ours[:, 0], pts[:, "XYZ".index(name[-1])])
        tol = np.where(level_of(pts) < mg, 1e-6, 1e-8)
        assert (np.abs(ours[:, 1] - want) <= tol).all(), (name, np.max(np.abs(ours[:, 1] - want)))
    # stdout0.out's tables, parsed back into calls, follow the W nesting and
    # their pre-smoothing calls are Loo.gp's lines
    P = problem(args)
    text = (tmp_path / "Output" / "stdout0.out").read_text()
    tables = text[text.index(BANNER_END) + len(BANNER_END):]
    nl = len(tables.split("\n")[3]) // 24            # the rule: 24 "=" per level
    calls, cycle = [], None
    for line in tables.splitlines():
        m = re.match(r"Cycle: (\d+)$", line)
        if m:
            cycle = int(m.group(1))
        m = re.search(r"\|Loo\[(\d+)\] : (\S+)\|", line)
        if m:
            calls.append([int(m.group(1)), None, None, float(m.group(2))])
    loo = np.loadtxt(tmp_path / "Output" / "Loo.gp", ndmin=2)
    # the post flag and cycle of each call follow from the nesting: replay it
    seen, pre_idx = {}, 0
    for c in calls:
        k = c[0]
        c[1] = 1 if seen.get(k) == "pre" and k != 0 else 0
        seen[k] = "post" if c[1] else "pre"
        if not c[1]:
            c[2] = int(loo[pre_idx, 0])
            assert float("%.8e" % loo[pre_idx, 1]) == c[3]
            pre_idx += 1
    assert pre_idx == len(loo)
    open_cycle = {}
    for c in calls:
        if not c[1]:
            open_cycle[c[0]] = c[2]
        else:
            c[2] = open_cycle[c[0]]
    assert cycle is not None
    check_wcycle_calls([tuple(c) for c in calls], nl, float("%.8e" % P.tol))
    assert render_cycle_tables([tuple(c) for c in calls], nl, P.tol) == tables
