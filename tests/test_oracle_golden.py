"""The oracle against fixtures generated by the reference solver itself
(tests/golden/make_golden.py): geometry, coefficients, two V-cycles and, for
three cases, the fixed point.  The oracle restates the reference's
arithmetic in the same order, so everything must match bit for bit."""
import glob
import os

import numpy as np
import pytest

from ollipticid_gb300 import parse_olliptic_args

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLD, "*.npz")))


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


@pytest.mark.parametrize("name", CASES)
def test_geometry_and_coefficients(name, oracle_mod):
    G = load(name)
    P = parse_olliptic_args(str(G["args"]).split())
    orc = oracle_mod.Oracle(P.oracle_dict())
    assert orc.nboxes == len(G["box_n"])
    for g, b in enumerate(orc.boxes):
        assert [b.nx, b.ny, b.nz] == list(G["box_n"][g])
        assert b.level == G["box_level"][g] and b.buf == G["box_buf"][g]
        assert [b.xi, b.yi, b.zi] == list(G["box_origin"][g])
        assert [b.dx, b.dy, b.dz] == list(G["box_d"][g])
        assert [b.cx, b.cy, b.cz] == list(G["box_c"][g])
        idx = G[f"idx_b{g}"]
        for f in ("b", "c", "d", "e"):
            key = f"coeff_{f}_b{g}"
            if key in G:
                np.testing.assert_array_equal(orc.field(g, f).ravel()[idx], G[key], err_msg=f"{f} box {g}")


@pytest.mark.parametrize("name", CASES)
def test_two_cycles_bit_exact(name, oracle_mod):
    G = load(name)
    P = parse_olliptic_args(str(G["args"]).split())
    orc = oracle_mod.Oracle(P.oracle_dict())
    norms = [orc.vcycle() for _ in range(2)]
    np.testing.assert_array_equal(norms, G["cyc2_norms"])
    np.testing.assert_array_equal(orc.adm(), G["cyc2_adm"])
    for g in range(orc.nboxes):
        np.testing.assert_array_equal(orc.field(g).ravel()[G[f"idx_b{g}"]], G[f"cyc2_u_b{g}"],
                                      err_msg=f"u box {g}")


@pytest.mark.parametrize("name", [c for c in CASES if "fixed_norms" in load(c)])
def test_fixed_point_bit_exact(name, oracle_mod):
    G = load(name)
    P = parse_olliptic_args(str(G["args"]).split())
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.solve()
    norms = []
    prev = orc.all_u()
    for _ in range(80):
        norms.append(orc.vcycle())
        cur = orc.all_u()
        d = max(float(np.max(np.abs(a - b))) for a, b in zip(cur, prev))
        prev = cur
        if d <= 1e-14:
            break
    np.testing.assert_array_equal(norms, G["fixed_norms"])
    np.testing.assert_array_equal(orc.adm(), G["fixed_adm"])
    for g in range(orc.nboxes):
        np.testing.assert_array_equal(prev[g].ravel()[G[f"idx_b{g}"]], G[f"fixed_u_b{g}"], err_msg=f"box {g}")


def test_valid_n(oracle_mod):
    L = oracle_mod.load()
    assert [L.orc_valid_n(n) for n in (33, 65, 66, 67, 69, 70, 120, 129, 140)] == [33, 65, 65, 65, 73, 73, 113, 129, 145]
