"""Olliptic_gpu.x: the reference's command line on the C ABI.  The plan and
the refusal of other equations need no GPU; the solve's printed ADM masses
equal the Python API's solve of the same command line."""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from tests.cases import CASES, CONFIG2, problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")


@pytest.fixture(scope="module")
def cli():
    from ollipticid_gb300 import build
    build.build()
    assert os.path.exists(CLI)
    return CLI


def run(cli, args, check=True, cwd=None):
    """Runs the command line in `cwd` (a fresh temporary directory when None:
    it writes its output directory where it runs)."""
    with tempfile.TemporaryDirectory() as tmp:
        r = subprocess.run([cli] + args.split(), capture_output=True, text=True, timeout=600, cwd=cwd or tmp)
    if check:
        assert r.returncode == 0, r.stderr
    return r


def test_plan_matches_the_library(cli):
    import ctypes as C
    from ollipticid_gb300 import _abi
    r = run(cli, CONFIG2 + " -plan yes")
    m = re.search(r"(\d+) levels \((\d+) multigrid\), (\d+) boxes", r.stdout)
    assert m, r.stdout
    lib = _abi.load()
    cp = problem(CONFIG2).to_c()
    out = (_abi.BoxInfo * 512)()
    nb, nl, mg = C.c_int(), C.c_int(), C.c_int()
    _abi.check(lib.olgpu_plan_boxes(C.byref(cp), out, 512, C.byref(nb), C.byref(nl), C.byref(mg)))
    assert (int(m.group(1)), int(m.group(2)), int(m.group(3))) == (nl.value, mg.value, nb.value)
    sizes = re.findall(r"box +\d+ level +\d+ +(\d+) x (\d+) x (\d+)", r.stdout)
    assert [tuple(map(int, s)) for s in sizes] == [(out[g].nx, out[g].ny, out[g].nz) for g in range(nb.value)]


def test_output_directory_is_rotated_like_the_reference(cli, tmp_path):
    """interface.cc:1470-1538: <dir> is made at start-up with <dir>.run (the
    command line); a second run moves it to <dir>_prev.  No GPU is needed:
    the directory exists before the device is touched (the run then fails
    here, or solves where a GPU is present)."""
    args = "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -N 25 -L 40 -O 2 -l 3 -o Res -p1d no -pint no -gpu-device 9999"
    run(cli, args, check=False, cwd=str(tmp_path))
    assert (tmp_path / "Res" / "Res.run").exists()
    recorded = (tmp_path / "Res" / "Res.run").read_text().split()
    assert recorded[1:] == args.split() and os.access(tmp_path / "Res" / "Res.run", os.X_OK)
    (tmp_path / "Res" / "marker").write_text("first")
    run(cli, args, check=False, cwd=str(tmp_path))
    assert (tmp_path / "Res_prev" / "marker").read_text() == "first"
    assert not (tmp_path / "Res" / "marker").exists()


def test_bam_export_needs_a_file(cli, tmp_path):
    """interface.cc:1168-1176: -iob yes without -iof is refused before any work."""
    r = run(cli, "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -N 25 -L 40 -O 2 -l 3 -iob yes", check=False,
            cwd=str(tmp_path))
    assert r.returncode == 1 and "Missing file" in r.stdout
    assert not (tmp_path / "Output").exists()


def test_other_equations_are_refused(cli):
    r = run(cli, "-eq Bowen_York -B Robin -N 33", check=False)
    assert r.returncode != 0 and "not on the puncture FAS path" in r.stderr
    for m in ("Full-Multigrid", "Gauss-Seidel"):
        r = run(cli, "-eq Punctures -B Robin -N 33 -m " + m, check=False)
        assert r.returncode != 0 and "not on the puncture FAS path" in r.stderr


@pytest.mark.parametrize("flag", ["-B Asymptotic", "-B Neumann"])
def test_boundaries_other_than_robin_and_dirichlet_are_refused(cli, flag, tmp_path):
    """Robin (what every pars/ file passes) and Dirichlet (the reference's
    default without -B) are on the GPU path; another condition is refused
    before any work rather than replaced."""
    r = run(cli, "-eq Punctures -NumBH 1 -bhmp1 0.5 -N 25 -L 40 -O 2 -l 3 " + flag, check=False, cwd=str(tmp_path))
    assert r.returncode != 0 and "is not on the GPU path" in r.stderr
    assert not (tmp_path / "Output").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["o4_binary_merge", "sf_binary"])
def test_cli_solve_matches_the_api(cli, case):
    import ollipticid_gb300 as og
    r = run(cli, CASES[case])
    adm = [float(x) for x in re.findall(r"ADM mass\[\d+\] = (\S+)", r.stdout)]
    with og.Elliptic(problem(case)) as E:
        rep = E.Solve()
        assert len(adm) == len(E.ADM_mass)
        for a, b in zip(adm, E.ADM_mass):
            assert a == b
        assert f"Solved in {rep.cycles} V-cycles" in r.stdout


@pytest.mark.parametrize("args", [
    "-eq Poisson -B Robin -L 10 -N 25 -O 4 -l 3",
    "-eq Boundary-test -L 10 -N 25 -O 4 -l 3",
    "-eq Multibox-test -B Dirichlet -NumBH 2 -bhx1 -3 -bhx2 3 -L 20 -N 25 -O 2 -l 3",
    "-eq Punctures -NumBH 1 -bhmp1 0.5 -L 40 -N 25 -O 4 -l 3 -m AppPuncture",
    "-eq Punctures -NumBH 1 -bhmp1 0.5 -L 40 -N 25 -O 4 -l 3 -m Wcycle",
    "-eq Punctures -NumBH 1 -bhmp1 0.5 -L 40 -N 25 -O 4 -l 3 -m Multigrid",   # an unknown name is Vcycle
])
def test_test_equations_methods_and_boundaries_are_accepted(cli, args):
    """The test equations, the Dirichlet default and the analytic method parse
    and plan without a GPU (the plan is the same host geometry as the solve)."""
    r = run(cli, args + " -plan yes")
    assert re.search(r"(\d+) levels \((\d+) multigrid\), (\d+) boxes", r.stdout), r.stdout
