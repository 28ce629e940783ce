"""Initial data exported for other codes (Olliptic.x -iob / -ioZ) against the
reference's own exports (tests/golden/export/*.npz, from its Olliptic.x):
Zcode files get the reference's lines (its duplicated last record included),
the coordinates printed identically and u within the solve-to-solve
tolerance; BAM files are rewritten in place in BAM's fixed-width layout with
the values the reference's exporter gives at the same points."""
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from tests.test_gpu_output import box_levels

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "export", "*.npz")))

pytestmark = pytest.mark.gpu

# both runs stop at residual 1e-12 (2nd order); points read from a multigrid
# coarse grid carry that grid's last coarse approximation
TOL, TOL_MG = 1e-9, 1e-6


def tolerances(level_of, mg, pts):
    return np.where(level_of(pts) < mg, TOL_MG, TOL)


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_exports_match_the_reference(path, tmp_path):
    from ollipticid_gb300 import build
    build.build()
    g = np.load(path)
    args = g["args"].item().decode() + " -iob yes -o Output"
    for key in g.files:
        if key.startswith("in:"):
            (tmp_path / key[3:]).write_bytes(g[key].item())
    r = subprocess.run([CLI] + args.split(), cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    mg = int(re.search(r"\((\d+) multigrid\)", r.stdout).group(1))
    level_of = box_levels(g["args"].item().decode())
    # Zcode: <file>_m beside each input
    for key in g.files:
        if not key.startswith("out:"):
            continue
        ours = (tmp_path / key[4:]).read_text().splitlines()
        ref = g[key].item().decode().splitlines()
        assert len(ours) == len(ref), key
        o = np.array([[float(v) for v in line.split()] for line in ours])
        f = np.array([[float(v) for v in line.split()] for line in ref])
        assert [line.split()[:3] for line in ours] == [line.split()[:3] for line in ref], key
        assert (np.abs(o[:, 3] - f[:, 3]) <= tolerances(level_of, mg, f[:, :3])).all(), key
    # BAM: rewritten in place; the reference's values for its points come from
    # the Zcode file that repeats them
    ref_bam = np.array([[float(v) for v in line.split()] for line in
                        g["out:grid_02-00.mgid_m"].item().decode().splitlines()])
    q = 0
    for name in ("grid_0", "grid_0a", "grid_1"):
        before = g["in:" + name].item().decode().splitlines()
        after = (tmp_path / name).read_text().splitlines()
        assert len(after) == len(before), name
        for b, a in zip(before, after):
            assert len(a) == 74 and a[:50] == b[:50], (name, a)
            x, y, z, u = (float(v) for v in a.split())
            assert [x, y, z] == list(ref_bam[q, :3])
            tol = tolerances(level_of, mg, ref_bam[q:q + 1, :3])[0]
            assert abs(u - ref_bam[q, 3]) <= tol + 1e-15 * abs(u), (name, u, ref_bam[q, 3])
            q += 1
    assert q == len(ref_bam) - 1        # the Zcode copy repeats its last record
