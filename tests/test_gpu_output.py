"""Output files of Olliptic_gpu.x against the reference's own (tests/golden/
output/*.npz, written by the reference's Olliptic.x built from its sources):
the same files, the same lines and blank lines, the coordinates printed
identically (compared as text), and the values within the fixture's
tolerance of the reference's: 1e-9 where both runs stop at residual 1e-12 by
the reference's rule (from different smoother orderings), wider where that
rule stops the reference early on a non-monotone residual, and on the
multigrid coarse grids, whose u is the last coarse-grid approximation.  The
Lagrange gather itself is checked bit for bit against the oracle on the same
u."""
import re
import glob
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as oracle_mod
from tests.cases import problem
from tests.golden.make_output_golden import parse_data_file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "output", "*.npz")))

pytestmark = pytest.mark.gpu


def box_levels(args):
    """Level of the box the printed-cut rule reads each point from
    (multigrid::Print_Interpol_1D: the last box in level order whose interior
    holds the point, else the largest box), from the host-only plan."""
    import ctypes as C
    from ollipticid_gb300 import _abi
    lib = _abi.load()
    cp = problem(args).to_c()
    out = (_abi.BoxInfo * 512)()
    nb = C.c_int()
    _abi.check(lib.olgpu_plan_boxes(C.byref(cp), out, 512, C.byref(nb), None, None))
    B = [out[g] for g in range(nb.value)]
    lo = np.array([[b.xi, b.yi, b.zi] for b in B])
    hi = np.array([[b.xf, b.yf, b.zf] for b in B])
    d = np.array([[b.dx, b.dy, b.dz] for b in B])
    m = d * (np.array([b.buf for b in B])[:, None] - 0.1)
    base = 0
    for g in range(1, len(B)):
        if (lo[g] < lo[base]).all() and (hi[base] < hi[g]).all():
            base = g

    def level_of(pts):
        chosen = np.full(len(pts), base)
        for g in range(len(B)):
            inside = ((lo[g] + m[g] < pts) & (pts < hi[g] - m[g])).all(axis=1)
            chosen[inside] = g
        return np.array([B[g].level for g in chosen])
    return level_of


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_output_files_match_the_reference(path, tmp_path):
    from ollipticid_gb300 import build
    build.build()
    g = np.load(path)
    args = g["args"].item().decode()
    r = subprocess.run([CLI] + args.split() + ["-o", "Output"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    mg = int(re.search(r"\((\d+) multigrid\)", r.stdout).group(1))
    level_of = box_levels(args)
    out = tmp_path / "Output"
    ours = sorted(f for f in os.listdir(out) if f != "stdout0.out")   # the fixtures leave the log out
    assert ours == [f.decode() for f in g["files"]]
    for name in ours:
        p = str(out / name)
        if name.endswith(".run"):
            assert open(p).read().split()[1:] == [a.decode() for a in g["run_args"]]
            continue
        if name == "Loo.gp":
            rows = [line.split("\t") for line in open(p) if line.strip()]
            cyc = [int(c) for c, _ in rows]
            levels = int(g["loo_levels"])
            assert cyc.count(0) == levels and len(rows) % levels == 0
            assert cyc == [c for c in range(len(rows) // levels) for _ in range(levels)]
            assert all(float(v) >= 0.0 for _, v in rows)
            # stdout0.out: one block a cycle, the levels' pre-smoothing norms
            # down, the coarsest solve's, the post-smoothing norms back up
            log = (out / "stdout0.out").read_text()
            blocks = log.split("\n\nCycle: ")[1:]
            assert len(blocks) == len(rows) // levels
            for c, blk in enumerate(blocks):
                assert blk.startswith(f"{c}\n") and blk.count("|Loo[") == 2 * levels - 1
                assert "  -->  " in blk
            continue
        text, vals = parse_data_file(p)
        ref_text, ref_vals = g[name + "__text"], g[name + "__vals"]
        assert len(text) == len(ref_text), name
        assert (text == ref_text).all(), name
        blank = np.isnan(ref_vals)
        assert (np.isnan(vals) == blank).all(), name
        err = np.abs(vals - ref_vals)[~blank]
        if name.startswith("u-l"):   # one box's cut
            coarse = np.full(err.shape, int(name[3:name.index("b")]) < mg)
        else:                        # interpolated cut: the box each point is read from
            cols = [[float(t) for t in row.decode().split("\t")] for row in ref_text[~blank]]
            pts = np.zeros((len(cols), 3))
            for q, c in enumerate(cols):
                if name == "u.XY":
                    pts[q, :2] = c
                else:
                    pts[q, "XYZ".index(name[-1])] = c[0]
            coarse = level_of(pts) < mg
        tol = np.where(coarse, float(g["mg_tol"]), float(g["value_tol"]))
        assert (err <= tol).all(), (name, err.max(), int(coarse.sum()))


@pytest.mark.parametrize("case,ord", [("o4_spin", 5), ("o4_binary_merge", 5), ("o2_single", 3), ("o8_offset", 9)])
def test_interpolation_is_the_oracles_bit_for_bit(case, ord):
    """The same u in both (the oracle's, uploaded), points on and off the
    nodes, inside and outside the base box, every box and the printed-cut
    rule: the GPU gather returns the oracle's bits."""
    import ollipticid_gb300 as og
    P = problem(case)
    orc = oracle_mod.Oracle(P.oracle_dict())
    for _ in range(2):
        orc.vcycle()
    rng = np.random.default_rng(7)
    half = 0.5 * P.L
    pts = np.concatenate([
        rng.uniform(-0.6 * half, 0.6 * half, size=(600, 3)),     # mostly inside
        rng.uniform(-1.3 * half, 1.3 * half, size=(200, 3)),     # some outside the base box
        np.array([[x, 0.0, 0.0] for x in np.linspace(-half, half, 97)]),   # on-axis, many on nodes
    ])
    with og.Elliptic(P) as E:
        for b in range(len(E.boxes)):
            E.set_field(b, "u", orc.field(b, "u"))
        got = E.interpolate(pts, ord=ord)
        want = orc.interpolate(pts, ord)
        assert np.isnan(got).sum() > 0
        assert np.array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        assert np.array_equal(got[ok].view(np.int64), want[ok].view(np.int64))
        for b in range(len(E.boxes)):
            inside = pts[np.abs(pts).max(axis=1) < 0.25 * half]
            gb = E.interpolate(inside, ord=min(ord, min(E.boxes[b].n) - 1), box=b)
            wb = orc.interpolate(inside, min(ord, min(E.boxes[b].n) - 1), box=b)
            assert np.array_equal(gb.view(np.int64), wb.view(np.int64)), b


STORAGE = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "storage", "*.npz")))


@pytest.mark.parametrize("path", STORAGE, ids=lambda p: os.path.basename(p)[:-4])
def test_3d_dumps_match_the_reference(path, tmp_path):
    """Olliptic_gpu.x -p3d: every point of every box in the reference's
    storage order (the order of the printed coordinates is compared exactly)
    with u within the solve-to-solve difference (both stop at residual 1e-10;
    the fixture keeps the reference's u in float32)."""
    from tests.golden.make_storage_golden import order_of
    g = np.load(path)
    args = g["args"].item().decode()
    r = subprocess.run([CLI] + args.split() + ["-o", "Output"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    mg = int(re.search(r"\((\d+) multigrid\)", r.stdout).group(1))
    for f in g["files"]:
        name = f.decode()
        order, n, u = order_of(str(tmp_path / "Output" / name))
        assert list(n) == list(g[name + "__n"]) and np.array_equal(order, g[name + "__order"]), name
        if name + "__u" in g.files:
            tol = 1e-6 if int(name[3:name.index("b")]) < mg else 5e-9
            assert np.max(np.abs(u - g[name + "__u"].astype(np.float64))) <= tol, name
