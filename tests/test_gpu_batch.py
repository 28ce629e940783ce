"""Batches of uneven solves (olgpu_batch_*) against the same problems solved alone.

A batch groups its problems into unions (same equation, order, boundary,
sweep counts and refinement depth) whose levels are aligned from the finest,
and runs every FASN step of a level as one launch over all the union's
solves; a solve that meets its stop rule is skipped by every later launch.
Each result must be the problem's solo result bit for bit -- the same u on
every point, the same cycle count and ADM masses -- in FP64 and in mixed
precision, and a failing solve (a NaN puncture mass) must leave the others
untouched.
"""
import math

import numpy as np
import pytest

from tests.cases import problem

RULE = None


def rule():
    from ollipticid_gb300 import _abi
    return dict(stop=_abi.STOP_ERROR, max_cycles=200, tol=1e-10, du_tol=5e-11)


def uneven_problems():
    """Single punctures and binaries of different sizes and depths at two
    orders (so that the batch has several unions, and unions whose members
    reach their coarsest level at different union levels)."""
    out = []
    for name, n, lev in [("o4_spin", 25, 3), ("o4_spin", 33, 3), ("o4_binary_merge", 25, 4),
                         ("o4_binary_merge", 33, 4), ("o4_spin", 49, 3), ("o2_single", 33, 4),
                         ("o2_single", 25, 4)]:
        P = problem(name)
        P.n, P.levels = n, lev
        out.append(P)
    return out


def solo(P, mixed):
    import ollipticid_gb300 as og
    with og.Elliptic(P) as E:
        E.set_precision(mixed)
        rep = E.Solve(**rule())
        return [E.get_field(g) for g in range(len(E.boxes))], rep


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_batch_results_are_the_solo_results(mixed):
    import ollipticid_gb300 as og

    probs = uneven_problems()
    with og.Batch(probs, mixed=mixed) as B:
        assert B.unions >= 2
        reps = B.solve(**rule())
        for i, P in enumerate(probs):
            want, wrep = solo(P, mixed)
            got = B.all_u(i)
            assert reps[i].status == 0
            assert reps[i].cycles == wrep.cycles, (i, reps[i].cycles, wrep.cycles)
            assert reps[i].final_res == wrep.final_res and reps[i].final_du == wrep.final_du
            assert [reps[i].adm[j] for j in range(P.numbh)] == [wrep.adm[j] for j in range(P.numbh)]
            assert all(np.array_equal(a, b) for a, b in zip(got, want)), f"problem {i}"
        # a second solve of the same batch from u = 0 repeats the first
        B.reset()
        again = B.solve(**rule())
        assert [r.cycles for r in again] == [r.cycles for r in reps]
        assert all(np.array_equal(a, b) for a, b in zip(B.all_u(0), solo(probs[0], mixed)[0]))


@pytest.mark.gpu
def test_batch_shares_launches():
    """A union of several solves launches each step once, where the solves
    alone launch it once each."""
    import ollipticid_gb300 as og

    probs = [problem("o4_binary_merge") for _ in range(4)]
    for i, P in enumerate(probs):
        P.mp = [0.45 + 0.01 * i, 0.48]
    with og.Batch(probs, mixed=True) as B:
        assert B.unions == 1
        batched = B.kernels_per_cycle
    with og.Elliptic(probs[0]) as E:
        E.set_precision(True)
        alone = E.kernels_per_cycle
    # per-solve tail kernels (Anderson, ADM, change of u, coarsest solve)
    # stay one per solve; everything else is shared
    assert batched < 2 * alone, (batched, alone)


@pytest.mark.gpu
def test_seeded_binaries_batched_equal_alone():
    """The first eight seeded binaries of the batched workload (N 33-97,
    6-10 levels, 4th order), mixed precision."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import workloads

    probs = workloads.batched_binaries(256)[:8]
    with og.Batch(probs, mixed=True, inner_sweeps=(4, 6)) as B:
        reps = B.solve(**rule())
        for i in (0, 3, 7):
            with og.Elliptic(probs[i]) as E:
                E.set_inner_sweeps(4, 6)
                E.set_precision(True)
                wrep = E.Solve(**rule())
                want = [E.get_field(g) for g in range(len(E.boxes))]
            assert reps[i].cycles == wrep.cycles
            assert all(np.array_equal(a, b) for a, b in zip(B.all_u(i), want)), f"binary {i}"


@pytest.mark.gpu
def test_batch_isolates_a_failing_solve():
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi

    probs = [problem("o4_spin"), problem("o4_spin"), problem("o4_spin")]
    probs[0].mp = [0.45]
    probs[1].mp = [math.nan]
    probs[2].mp = [0.55]
    with og.Batch(probs, mixed=True) as B:
        reps = B.solve(raise_on_error=False, **rule())
        assert [r.status for r in reps] == [_abi.OK, _abi.ERR_NAN, _abi.OK]
        for i in (0, 2):
            want, wrep = solo(probs[i], True)
            assert reps[i].cycles == wrep.cycles
            assert all(np.array_equal(a, b) for a, b in zip(B.all_u(i), want))


@pytest.mark.gpu
def test_batch_autotuner_times_every_candidate():
    """autotune.tune_batch solves the batch once per candidate layout and
    returns the fastest of those that all reached the stop rule."""
    from ollipticid_gb300 import autotune
    cands = ((2, 3, 16), (2, 3, 0))
    choice = autotune.tune_batch(uneven_problems(), candidates=cands, tol=1e-9, max_cycles=80)
    assert [(r["nu1"], r["nu2"], r["blocks"]) for r in choice.table] == list(cands)
    assert all(r["reached_tol"] and r["solves_per_s"] > 0 for r in choice.table)
    assert (choice.nu1, choice.nu2, choice.blocks) in cands
    assert choice.solves_per_s == max(r["solves_per_s"] for r in choice.table)
