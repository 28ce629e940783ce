"""Product geometry (libolgpu's host hierarchy builder, olgpu_plan_boxes)
against the reference's boxes recorded in tests/golden and against the
oracle for the benchmark configurations."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from ollipticid_gb300 import _abi, parse_olliptic_args
from tests.cases import CONFIG2, CONFIG3

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def plan(args):
    lib = _abi.load()
    P = parse_olliptic_args(args.split())
    cp = P.to_c()
    out = (_abi.BoxInfo * 256)()
    nb, nl, mg = C.c_int(), C.c_int(), C.c_int()
    _abi.check(lib.olgpu_plan_boxes(C.byref(cp), out, 256, C.byref(nb), C.byref(nl), C.byref(mg)))
    return [out[g] for g in range(nb.value)], nl.value, mg.value


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "*.npz"))))
def test_boxes_match_reference(path):
    G = dict(np.load(path))
    boxes, nl, mg = plan(str(G["args"]))
    assert len(boxes) == len(G["box_n"])
    for g, b in enumerate(boxes):
        assert [b.nx, b.ny, b.nz] == list(G["box_n"][g])
        assert b.level == G["box_level"][g] and b.buf == G["box_buf"][g]
        assert [b.xi, b.yi, b.zi] == list(G["box_origin"][g])      # bit-exact
        assert [b.dx, b.dy, b.dz] == list(G["box_d"][g])
        assert [b.cx, b.cy, b.cz] == list(G["box_c"][g])


@pytest.mark.parametrize("args", [CONFIG2, CONFIG3], ids=["config2", "config3"])
def test_benchmark_geometry_matches_oracle(args, oracle_mod):
    boxes, nl, mg = plan(args)
    orc = oracle_mod.Oracle(parse_olliptic_args(args.split()).oracle_dict())
    assert (nl, mg) == (orc.levels, orc.mgrid_levels)
    assert len(boxes) == orc.nboxes
    for b, o in zip(boxes, orc.boxes):
        assert (b.nx, b.ny, b.nz, b.level, b.buf) == (o.nx, o.ny, o.nz, o.level, o.buf)
        assert (b.xi, b.yi, b.zi, b.dx, b.cx, b.cy, b.cz) == (o.xi, o.yi, o.zi, o.dx, o.cx, o.cy, o.cz)


def test_config2_hierarchy_shape():
    boxes, nl, mg = plan(CONFIG2)
    assert (nl, mg) == (11, 2)
    assert [(b.nx, b.ny, b.nz) for b in boxes] == [
        (17, 17, 17), (33, 33, 33), (67, 67, 67), (67, 75, 67), (67, 75, 67), (67, 75, 67), (67, 83, 67),
        (67, 91, 67), (67, 115, 67), (67, 67, 67), (67, 67, 67), (67, 67, 67), (67, 67, 67)]


def test_parse_ignores_unknown_flags():
    P = parse_olliptic_args("-eq Punctures -B Robin -BA 0.0 -Bn 1 -NumBH 2 -bhmp1 0.4 -bhmp2 0.6 -Dp 0.05 "
                            "-o Out -pc yes -N 65 -L 100 -O 6 -l 5".split())
    assert P.mp == [0.4, 0.6] and (P.n, P.L, P.order, P.levels) == (65, 100.0, 6, 5)
    with pytest.raises(ValueError):
        parse_olliptic_args("-eq Bowen_York".split())
    assert parse_olliptic_args("-eq Poisson".split()).equation == "Poisson"   # the Gaussian test
    assert parse_olliptic_args("-m Wcycle".split()).method == "Wcycle"
    assert parse_olliptic_args("-m Multigrid".split()).method == "Vcycle"      # interface.cc: unknown = Vcycle
    with pytest.raises(ValueError):
        parse_olliptic_args("-m Gauss-Seidel".split())
