"""The oracle's Bowen-York momentum-constraint test against the reference's
own run of it (tests/golden/make_bowen_york_golden.py): the sources rho0..rho2
bit for bit (every point of the momentum balls included), and the four
variables V1, V2, V3, lambda at the fixed point.  The oracle solves the V
equations and then lambda one after another where the reference advances
all four together, so the iterates differ but the discrete system does not:
the fixed points agree to rounding (1e-13 here; the reference's own last
cycle still moved them by about 1e-14).  A multigrid coarse grid's ghost
layers are not fixed by the system (the coarsest solve leaves whatever its
last Robin pass wrote there) and are left out."""
import glob
import os

import numpy as np
import pytest

from ollipticid_gb300 import parse_olliptic_args

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bowen_york", "o*.npz")))
VARS = ("V1", "V2", "V3", "lambda")
FIXED_TOL = 1e-13


def fixed_mask(orc, g, idx):
    """Sampled points the discrete system fixes: all but a multigrid coarse
    grid's ghost layers."""
    b = orc.boxes[g]
    if b.level >= orc.mgrid_levels:
        return np.ones(len(idx), dtype=bool)
    k, j, i = np.unravel_index(idx, (b.nz, b.ny, b.nx))
    return (i >= b.buf) & (i < b.nx - b.buf) & (j >= b.buf) & (j < b.ny - b.buf) & (k >= b.buf) & (k < b.nz - b.buf)


@pytest.mark.parametrize("path", GOLD, ids=lambda p: os.path.basename(p)[:-4])
def test_sources_bit_exact(path, oracle_mod):
    G = np.load(path)
    P = parse_olliptic_args(str(G["args"]).split())
    for c in range(3):
        orc = oracle_mod.Oracle(dict(P.oracle_dict(), by_var=c))
        assert [[b.nx, b.ny, b.nz] for b in orc.boxes] == G["box_n"].tolist()
        for g in range(orc.nboxes):
            rho = orc.field(g, "rho").ravel()
            np.testing.assert_array_equal(rho[G[f"idx_b{g}"]], G[f"rho{c}_b{g}"])
            np.testing.assert_array_equal(rho[G[f"ball_b{g}"]], G[f"rho{c}_ball_b{g}"])
            assert np.count_nonzero(rho) <= len(G[f"ball_b{g}"])   # nothing outside the balls


@pytest.mark.parametrize("path", GOLD, ids=lambda p: os.path.basename(p)[:-4])
def test_fixed_point_matches_the_reference(path, oracle_mod):
    G = np.load(path)
    P = parse_olliptic_args(str(G["args"]).split())
    fields, deltas = oracle_mod.bowen_york_fixed_point(P.oracle_dict())
    assert max(deltas.values()) <= 1e-14
    orc = oracle_mod.Oracle(dict(P.oracle_dict(), by_var=0))
    for g in range(orc.nboxes):
        idx = G[f"idx_b{g}"]
        keep = fixed_mask(orc, g, idx)
        for v in VARS:
            got = fields[v][g].ravel()[idx]
            err = np.max(np.abs(got[keep] - G[f"{v}_b{g}"][keep]))
            assert err <= FIXED_TOL, (v, g, err)
