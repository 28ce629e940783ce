"""Concurrent solves: problems stepped together (each on its own stream,
overlapping on the GPU) give the same result as solved alone -- bit for bit,
since every kernel's arithmetic is independent of scheduling (multicolour
sweeps, max reductions, Anderson sums added in block order)."""
import numpy as np
import pytest

from tests.cases import problem

NAMES = ["o2_single", "o4_binary_merge", "sf_binary"]


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_same_alone_and_in_the_mix(mixed):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    alone = []
    for name in NAMES:
        with og.Elliptic(problem(name)) as E:
            E.set_precision(mixed)
            rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=80, tol=1e-11)
            alone.append((rep.cycles, [E.get_field(g) for g in range(len(E.boxes))], E.ADM_mass))
    solvers = [og.Elliptic(problem(n)) for n in NAMES]
    try:
        for E in solvers:
            E.set_precision(mixed)
        reps = og.solve_many(solvers, stop=_abi.STOP_TOLERANCE, max_cycles=80, tol=1e-11)
        for (cyc, u, adm), E, rep in zip(alone, solvers, reps):
            got = [E.get_field(g) for g in range(len(E.boxes))]
            err = max(float(np.max(np.abs(a - b))) for a, b in zip(u, got))
            assert err == 0.0 and rep.cycles == cyc
            assert list(adm) == list(E.ADM_mass)
    finally:
        for E in solvers:
            E.close()
