"""Host side of the Bowen-York test (no GPU): the command line maps to
OLGPU_EQ_BOWEN_YORK, and the library's host-only plan (olgpu_plan_boxes)
gives the boxes of the reference's own run of it."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import ollipticid_gb300 as og
from ollipticid_gb300 import _abi

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bowen_york", "o*.npz")))


def test_command_line_selects_bowen_york():
    P = og.parse_olliptic_args("-eq Bowen-York -B Robin -NumBH 1 -bhpx1 0.1 -N 25 -L 20 -l 3 -O 2".split())
    assert P.equation == "Bowen-York"
    assert P.to_c().equation == 5 and P.oracle_dict()["equation"] == 5
    assert og.BY_VARS == ("V1", "V2", "V3", "lambda")


@pytest.mark.parametrize("path", GOLD, ids=lambda p: os.path.basename(p)[:-4])
def test_plan_is_the_reference_geometry(path):
    G = np.load(path)
    cp = og.parse_olliptic_args(str(G["args"]).split()).to_c()
    lib = _abi.load()
    out = (_abi.BoxInfo * 64)()
    nb, nl, mg = C.c_int(), C.c_int(), C.c_int()
    _abi.check(lib.olgpu_plan_boxes(C.byref(cp), out, 64, C.byref(nb), C.byref(nl), C.byref(mg)))
    assert [[out[g].nx, out[g].ny, out[g].nz] for g in range(nb.value)] == G["box_n"].tolist()
    assert [out[g].level for g in range(nb.value)] == G["box_level"].tolist()


def test_header_and_host_agree_on_the_equation_codes():
    import re
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "olgpu.h")).read()
    codes = {m.group(1): int(m.group(2)) for m in re.finditer(r"OLGPU_EQ_(\w+)\s*=\s*(\d+)", hdr)}
    assert codes["BOWEN_YORK"] == og.EQUATIONS["Bowen-York"] == 5
    assert codes["POISSON"] == og.EQUATIONS["Poisson"]
