"""The C ABI library builds, loads and exports every entry point that
include/olgpu.h declares; argument checks and the geometry-only entry work
without a GPU."""
import ctypes as C
import os
import re

import pytest

from ollipticid_gb300 import _abi, parse_olliptic_args

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "olgpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(olgpu_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _abi.load()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_abi.SIGNATURES), set(names) - set(_abi.SIGNATURES)


def test_invalid_arguments_are_rejected_without_a_device():
    lib = _abi.load()
    p = _abi.Problem()
    lib.olgpu_problem_defaults(C.byref(p))
    p.order = 3
    h = C.c_void_p()
    assert lib.olgpu_hierarchy_create(C.byref(p), 0, C.byref(h)) == _abi.ERR_INVALID_ARG
    assert b"order" in lib.olgpu_last_error()
    p.order = 4
    p.numbh = 0
    assert lib.olgpu_hierarchy_create(C.byref(p), 0, C.byref(h)) == _abi.ERR_INVALID_ARG
    assert lib.olgpu_hierarchy_create(None, 0, C.byref(h)) == _abi.ERR_INVALID_ARG


def test_too_few_points_is_a_geometry_error():
    lib = _abi.load()
    P = parse_olliptic_args("-eq Punctures -NumBH 1 -bhmp1 0.5 -N 17 -L 10 -O 2 -l 2".split())
    cp = P.to_c()
    n = C.c_int()
    assert lib.olgpu_plan_boxes(C.byref(cp), None, 0, C.byref(n), None, None) == _abi.ERR_GEOMETRY
