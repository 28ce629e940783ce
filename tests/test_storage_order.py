"""olgpu_storage_order (domain::Fix_Points: corners, edges, faces, interior)
against the point order of the reference's own 3-D dumps
(tests/golden/storage, from its Olliptic.x -p3d), ghost bands 1 and 2; host
only, no GPU."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from ollipticid_gb300 import _abi
from tests.cases import problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "storage", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_storage_order_is_the_references(path):
    lib = _abi.load()
    g = np.load(path)
    cp = problem(g["args"].item().decode()).to_c()
    boxes = (_abi.BoxInfo * 64)()
    nb, nl = C.c_int(), C.c_int()
    _abi.check(lib.olgpu_plan_boxes(C.byref(cp), boxes, 64, C.byref(nb), C.byref(nl), None))
    seen = 0
    for level in range(nl.value):
        for ib, gbox in enumerate([b for b in range(nb.value) if boxes[b].level == level]):
            name = f"u-l{level}b{ib}-0.xyz"
            B = boxes[gbox]
            assert list(g[name + "__n"]) == [B.nx, B.ny, B.nz]
            out = np.empty(B.nx * B.ny * B.nz, dtype=np.int64)
            _abi.check(lib.olgpu_storage_order(C.byref(B), out.ctypes.data_as(C.c_void_p)))
            assert np.array_equal(out, g[name + "__order"]), name
            assert np.array_equal(np.sort(out), np.arange(out.size))   # a permutation
            seen += 1
    assert seen == len(g["files"])
