"""Mixed precision (FP32 correction cycles around an FP64 state) converges to
the same FP64 fixed point as the reference: max |u - u_oracle| <= 1e-10 on
the points the discrete system fixes, ADM masses within 1e-9, and its
per-cycle convergence keeps pace with the FP64 cycle."""
import numpy as np
import pytest

from tests.cases import CASES, problem

U_TOL = 1e-10
ADM_TOL = 1e-9


def settle(E, tol=1e-14, max_cycles=300):
    prev = [E.get_field(g) for g in range(len(E.boxes))]
    d = np.inf
    for _ in range(max_cycles):
        E.FASN()
        cur = [E.get_field(g) for g in range(len(E.boxes))]
        d = max(float(np.max(np.abs(a - b))) for a, b in zip(cur, prev))
        prev = cur
        if d <= tol:
            break
    return prev, d


@pytest.mark.gpu
@pytest.mark.parametrize("coarse", ["cluster", "one_block"])
@pytest.mark.parametrize("case", ["o2_single", "o4_binary_merge", "o8_offset", "sf_binary"])
def test_mixed_fixed_point_matches_oracle(case, coarse, oracle_mod, monkeypatch):
    """coarse: the coarsest FP32 correction on a cluster of 8 blocks (the
    default) or in one block (k_coarse32, which takes the boxes the cluster
    kernel does not)."""
    import ollipticid_gb300 as og
    if coarse == "one_block":
        monkeypatch.setenv("OLGPU_COARSE32_ONE_BLOCK", "1")
    P = problem(case)
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.fixed_point(tol=1e-14)
    with og.Elliptic(P) as E:
        E.set_precision(True)
        ug, d = settle(E)
        assert d < 1e-12, f"mixed solve did not settle: last change {d:.3e}"
        for g, (a, b) in enumerate(zip(ug, orc.all_u())):
            box = E.boxes[g]
            if box.level < E.mgrid_levels:
                w = box.buf
                a, b = a[w:-w, w:-w, w:-w], b[w:-w, w:-w, w:-w]
            err = float(np.max(np.abs(a - b)))
            assert err <= U_TOL, f"box {g} (level {box.level}): max|du| = {err:.3e}"
        for a, b in zip(E.ADM_mass, orc.adm()):
            assert abs(a - b) <= ADM_TOL


@pytest.mark.gpu
def test_mixed_stop_rule_bounds_the_error(oracle_mod):
    """Stopped by its own rule at tol 1e-11 (norm = max of the finest FP64
    defect and the last correction), a mixed solve is within 1e-10 of the
    oracle's fixed point on every pinned point."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    P = problem("o4_binary_merge")
    P.tol = 1e-11
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.fixed_point(tol=1e-14)
    with og.Elliptic(P) as E:
        E.set_precision(True)
        rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=200)
        assert rep.final_res <= 1e-11 and rep.cycles < 60
        for g, (a, b) in enumerate(zip([E.get_field(g) for g in range(len(E.boxes))], orc.all_u())):
            box = E.boxes[g]
            if box.level < E.mgrid_levels:
                w = box.buf
                a, b = a[w:-w, w:-w, w:-w], b[w:-w, w:-w, w:-w]
            assert float(np.max(np.abs(a - b))) <= U_TOL, g


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["o4_binary_merge", "o8_offset", "sf_binary"])
def test_cluster_smoother_equals_colour_launches(case, monkeypatch):
    """The FP32 smoother with e resident in a thread-block cluster's shared
    memory (every sweep of a level in one launch) gives the per-colour
    launches' result bit for bit."""
    import ollipticid_gb300 as og
    P = problem(case)
    out = {}
    for mode in ("cluster", "launches"):
        if mode == "launches":
            monkeypatch.setenv("OLGPU_SMOOTH32_LAUNCHES", "1")
        with og.Elliptic(P) as E:
            E.set_precision(True)
            for _ in range(3):
                E.FASN()
            out[mode] = ([E.get_field(g) for g in range(len(E.boxes))], E.kernels_per_cycle)
    (u_cl, k_cl), (u_la, k_la) = out["cluster"], out["launches"]
    assert k_cl < k_la, "no level took the cluster smoother"
    for g, (a, b) in enumerate(zip(u_cl, u_la)):
        assert np.array_equal(a, b), f"box {g}: max diff {float(np.max(np.abs(a - b))):.3e}"


@pytest.mark.gpu
def test_inner_sweeps_keep_the_fixed_point(oracle_mod):
    """A lighter FP32 inner schedule changes the work per cycle, not the
    solution: stopped at 1e-11 it is within 1e-10 of the oracle's fixed point."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    P = problem("o4_binary_merge")
    orc = oracle_mod.Oracle(P.oracle_dict())
    orc.fixed_point(tol=1e-14)
    with og.Elliptic(P) as E:
        E.set_precision(True)
        E.set_inner_sweeps(2, 4)
        rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=200, tol=1e-11)
        assert rep.final_res <= 1e-11
        for g, (a, b) in enumerate(zip([E.get_field(g) for g in range(len(E.boxes))], orc.all_u())):
            box = E.boxes[g]
            if box.level < E.mgrid_levels:
                w = box.buf
                a, b = a[w:-w, w:-w, w:-w], b[w:-w, w:-w, w:-w]
            assert float(np.max(np.abs(a - b))) <= U_TOL, g
        with pytest.raises(og.OlgpuError):
            E.set_inner_sweeps(0, 0)
