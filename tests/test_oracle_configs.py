"""The oracle against the reference on the benchmark problems (no GPU).

tests/golden/configs holds, for the three benchmark command lines, the
reference's own u after two V-cycles and its fixed point at sample points
(tests/golden/make_config_golden.py).  The oracle must reproduce the two
cycles bit for bit (single puncture and TestBH binary; the 8th-order binary
on 129^3 boxes takes minutes a cycle on a CPU, so its two cycles were checked
on every point when its fixture was made) and the single puncture's fixed
point; every geometry must be the library's box plan.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.cases import CONFIG1, CONFIG2, CONFIG3

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "configs")
CONFIGS = {"config1": CONFIG1, "config2": CONFIG2, "config3": CONFIG3}


def fixture(name):
    path = os.path.join(GOLDEN, f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"{name} fixture not generated")
    return np.load(path)


def oracle(name):
    import ollipticid_gb300 as og
    from oracle import oracle as O
    return O.Oracle(og.parse_olliptic_args(CONFIGS[name].split()).oracle_dict())


@pytest.mark.parametrize("name", ["config1", "config2", "config3"])
def test_fixture_geometry_is_the_library_plan(name):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    g = fixture(name)
    lib = _abi.load()
    cp = og.parse_olliptic_args(CONFIGS[name].split()).to_c()
    out = (_abi.BoxInfo * 64)()
    nb = C.c_int()
    assert lib.olgpu_plan_boxes(C.byref(cp), out, 64, C.byref(nb), None, None) == _abi.OK
    assert nb.value == len(g["box_n"])
    for b in range(nb.value):
        o = out[b]
        assert (o.nx, o.ny, o.nz) == tuple(int(v) for v in g["box_n"][b])
        assert o.level == int(g["box_level"][b]) and o.buf == int(g["box_buf"][b])
        assert (o.xi, o.yi, o.zi) == tuple(float(v) for v in g["box_origin"][b])
        assert (o.dx, o.dy, o.dz) == tuple(float(v) for v in g["box_d"][b])


@pytest.mark.parametrize("name", ["config1", "config2"])
def test_two_cycles_bit_for_bit(name):
    g = fixture(name)
    orc = oracle(name)
    norms = [orc.vcycle() for _ in range(2)]
    assert norms == list(g["cyc2_norms"])
    assert orc.adm() == list(g["cyc2_adm"])
    for b in range(orc.nboxes):
        u = orc.field(b).ravel()
        assert np.array_equal(u[g[f"idx_b{b}"].astype(np.int64)], g[f"cyc2_u_b{b}"]), f"box {b}"


def test_config1_fixed_point():
    g = fixture("config1")
    assert str(g["fixed_source"]) == "reference"
    orc = oracle("config1")
    orc.fixed_point(tol=1e-14)
    for b in range(orc.nboxes):
        u = orc.field(b).ravel()[g[f"idx_b{b}"].astype(np.int64)]
        assert np.max(np.abs(u - g[f"fixed_u_b{b}"])) <= 1e-14, f"box {b}"
    assert np.allclose(orc.adm(), g["fixed_adm"], rtol=0, atol=1e-14)


def test_fixed_points_are_converged():
    """The fixtures' fixed points: a last cycle change of at most 1e-13 (the
    reference's own cycles), or, for the 8th-order problem on 129^3 boxes,
    whose cycle has a rounding floor near 1e-11, at most 1e-11 from the
    oracle's Anderson-mixed cycles."""
    bound = {"config1": 1e-13, "config2": 1e-13, "config3": 1e-11}
    for name in CONFIGS:
        path = os.path.join(GOLDEN, f"{name}.npz")
        if os.path.exists(path):
            assert np.load(path)["fixed_deltas"][-1] <= bound[name], name
