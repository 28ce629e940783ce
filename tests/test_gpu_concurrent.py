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


@pytest.mark.gpu
def test_device_pool_reuses_freed_memory():
    """Hierarchies allocate from one stream-ordered pool per device and free
    into it without a device-wide wait: made and destroyed over and over
    beside a live one (as a server does), they reuse the same memory -- the
    pool does not grow -- and the pool gives everything back after the last
    hierarchy is destroyed."""
    import gc
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    gc.collect()                                            # hierarchies other tests left to the collector
    r0, u0 = og.device_pool_bytes(0)
    keep = og.Elliptic(problem("o4_binary_merge"))
    try:
        seen = []
        for i in range(8):
            for mixed in (False, True):
                with og.Elliptic(problem("sf_binary" if i % 2 else "o2_single")) as E:
                    E.set_precision(mixed)
                    E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=2, tol=1e-30)
            seen.append(og.device_pool_bytes(0))
        reserved = [r for r, _ in seen]
        used = [u for _, u in seen]
        assert used[-1] == used[0] and used[0] > 0          # only the live hierarchy's memory is in use
        assert reserved[-1] <= reserved[1], reserved       # freed memory is reused, not added to
    finally:
        keep.close()
    r, u = og.device_pool_bytes(0)
    assert u == u0, (u, u0)
    if u0 == 0:                                             # no hierarchy left: the pool gave its memory back
        assert r == 0, r
