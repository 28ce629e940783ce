"""The Dirichlet boundary (the reference's default without -B) on the GPU:
Olliptic_gpu.x without -B prints the reference's cuts (tests/golden/
dirichlet, from its Olliptic.x) for a puncture binary and the Gaussian test;
the device solve reaches the oracle's fixed point; mixed precision, built
for the Robin boundary, is refused."""
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

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "dirichlet", "*.npz")))

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_dirichlet_runs_match_the_reference(path, tmp_path):
    g = np.load(path)
    args = g["args"].item().decode()
    r = subprocess.run([CLI] + args.split() + ["-o", "Output"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    mg = int(re.search(r"\((\d+) multigrid\)", r.stdout).group(1))
    level_of = box_levels(args)
    for name in ("u.X", "u.Y", "u.Z"):
        ours = np.loadtxt(tmp_path / "Output" / name)
        pts, want = cut_points(g, name)
        assert np.array_equal(ours[:, 0], pts[:, "XYZ".index(name[-1])])
        tol = np.where(level_of(pts) < mg, 1e-6, 1e-9)
        assert (np.abs(ours[:, 1] - want) <= tol).all(), (name, np.max(np.abs(ours[:, 1] - want)))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_dirichlet_fixed_point_is_the_oracles(path):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    g = np.load(path)
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.fixed_point()
    u_fix = orc.all_u()
    with og.Elliptic(P) as E:
        rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=400, tol=1e-13)
        assert rep.final_res <= 1e-13
        sol = [b for b, box in enumerate(E.boxes) if box.level >= E.mgrid_levels]
        err = max(float(np.max(np.abs(E.get_field(b).ravel() - u_fix[b].ravel()))) for b in sol)
        with pytest.raises(_abi.OlgpuError):
            E.set_precision(True)
    assert err <= 1e-10, err
