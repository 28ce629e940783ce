"""Sweep-schedule autotuner: shape keys, the JSON cache (CPU) and a tuning
run whose choice solves to the same tolerance (GPU)."""
import json

import numpy as np
import pytest

from tests.cases import problem


def test_shape_key_and_cache(tmp_path):
    from ollipticid_gb300 import autotune
    P = problem("o4_binary_merge")
    k = autotune.shape_key(P, 8)
    assert k == f"eq{P.equation}_O{P.order}_N{P.n}_l{P.levels}_bh{P.numbh}_c8"
    assert autotune.shape_key(P, 4) != k
    path = tmp_path / "tuned.json"
    assert autotune.cached(P, 8, str(path)) is None
    path.write_text(json.dumps({k: {"nu1": 2, "nu2": 6, "solves_per_s": 1.0, "cycles": 9, "table": []}}))
    c = autotune.cached(P, 8, str(path))
    assert (c.nu1, c.nu2, c.blocks, c.cycles) == (2, 6, 16, 9)


@pytest.mark.gpu
def test_tuned_schedule_solves_to_tolerance(tmp_path, oracle_mod):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi, autotune
    P = problem("o4_binary_merge")
    path = str(tmp_path / "tuned.json")
    choice = autotune.tune(P, concurrency=2, candidates=((3, 20, 16), (2, 4, 0)), tol=1e-11, cache_path=path)
    assert (choice.nu1, choice.nu2, choice.blocks) in ((3, 20, 16), (2, 4, 0))
    assert len(choice.table) == 2 and all(r["reached_tol"] for r in choice.table)
    assert autotune.cached(P, 2, path).nu2 == choice.nu2
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.fixed_point(tol=1e-14)
    with og.Elliptic(P) as E:
        E.set_precision(True)
        choice.apply(E)
        rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=200, tol=1e-11)
        assert rep.final_res <= 1e-11
        for g, (a, b) in enumerate(zip([E.get_field(g) for g in range(len(E.boxes))], orc.all_u())):
            box = E.boxes[g]
            if box.level < E.mgrid_levels:
                w = box.buf
                a, b = a[w:-w, w:-w, w:-w], b[w:-w, w:-w, w:-w]
            assert float(np.max(np.abs(a - b))) <= 1e-10, g
