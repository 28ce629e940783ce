"""The analytic puncture approximation on the device (olgpu_approximate_id,
elliptic::ApproximateID): the oracle's values on every point of every box,
the reference's printed cuts through Olliptic_gpu.x -m AppPuncture, and, as
a starting guess, the same fixed point in fewer V-cycles."""
import glob
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import CASES, problem
from tests.golden.make_output_golden import parse_data_file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "approx", "*.npz")))

pytestmark = pytest.mark.gpu

# every operation is rounded as on the host except the logarithm (CUDA's
# against the C library's, within an ulp or two); near a puncture the
# formula's bracket amplifies that by about 1/R^2
TOL = 1e-12


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_device_approximation_is_the_oracles(path):
    import ollipticid_gb300 as og
    g = np.load(path)
    P = problem(g["args"].item().decode())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.approximate_id()
    with og.Elliptic(P) as E:
        E.ApproximateID(as_guess=False)
        err = max(float(np.max(np.abs(E.get_field(b).ravel() - orc.field(b, "u").ravel())))
                  for b in range(len(E.boxes)))
    assert err <= TOL, err


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_cli_prints_the_reference_approximation(path, tmp_path):
    g = np.load(path)
    r = subprocess.run([CLI] + g["args"].item().decode().split() + ["-o", "Output"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    u_p = [float(line.split(" u : ")[1]) for line in r.stdout.splitlines() if " u : " in line]
    assert np.allclose(u_p, g["u_at_punctures"], rtol=1e-7, atol=0)     # printed with 8 digits
    assert "V-cycle" not in r.stdout and "ADM mass" not in r.stdout
    for name in ("u.X", "u.Y", "u.Z", "u.XY"):
        text, vals = parse_data_file(str(tmp_path / "Output" / name))
        ref_text, ref_vals = g[name + "__text"], g[name + "__vals"]
        assert (text == ref_text).all(), name
        ok = ~np.isnan(ref_vals)
        assert np.max(np.abs(vals[ok] - ref_vals[ok])) <= TOL, name


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("case", ["o4_binary_merge", "o4_spin", "sf_binary"])
def test_approximate_start_keeps_the_fixed_point(case, mixed):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    with og.Elliptic(problem(case)) as E:
        E.set_precision(mixed)
        zero = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=400, tol=1e-13)
        u0 = [E.get_field(b) for b in range(len(E.boxes))]
        E.ApproximateID()
        appr = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=400, tol=1e-13)
        u1 = [E.get_field(b) for b in range(len(E.boxes))]
        # the multigrid coarse grids hold the last coarse-grid approximation,
        # which depends on the path (as in the reference); the solution is
        # the refinement levels
        sol = [b for b, box in enumerate(E.boxes) if box.level >= E.mgrid_levels]
    assert zero.final_res <= 1e-13 and appr.final_res <= 1e-13
    err = max(float(np.max(np.abs(u0[b] - u1[b]))) for b in sol)
    assert err <= 1e-10, err
    assert appr.cycles <= zero.cycles, (appr.cycles, zero.cycles)
