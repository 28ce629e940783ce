"""The continuous-batching server: requests that arrive while others are on
the GPU are admitted as slots free up, run concurrently, and each result is
the same as the same request solved alone (bit for bit: no kernel's
arithmetic depends on scheduling); memory admission refuses a request that
can never fit."""
import numpy as np
import pytest

from tests.cases import problem

NAMES = ["o2_single", "o4_spin", "o4_binary_merge", "sf_binary", "o6_boost_y"]


@pytest.mark.gpu
def test_served_results_match_solo_solves():
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    from ollipticid_gb300.serve import Server
    probs = [problem(n) for n in NAMES]
    stream = [(0.002 * i, p) for i, p in enumerate(probs)]
    rep = Server(max_active=3, keep_u=True, tol=1e-11).run(stream)
    assert rep["completed"] == len(probs)
    assert rep["peak_concurrent_solves"] >= 2          # the work overlapped
    for p, r in zip(probs, rep["results"]):
        with og.Elliptic(p) as E:
            E.set_precision(True)
            solo = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=200, tol=1e-11)
            u = [E.get_field(g) for g in range(len(E.boxes))]
        assert r.status == 0 and r.cycles == solo.cycles
        err = max(float(np.max(np.abs(a - b))) for a, b in zip(u, r.u))
        assert err == 0.0, err


@pytest.mark.gpu
def test_request_larger_than_the_budget_is_refused():
    from ollipticid_gb300 import _abi
    from ollipticid_gb300.serve import Server
    rep = Server(mem_budget=1 << 20).run([(0.0, problem("o4_spin"))])
    assert rep["results"][0].status == _abi.ERR_OOM


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [True, False], ids=["mixed", "fp64"])
def test_native_server_results_match_solo_solves(mixed):
    """The C++ server behind the C ABI (olgpu_server_*): uneven requests
    overlap on the GPU and each result is the solo solve's bit for bit."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    from ollipticid_gb300.serve import NativeServer
    probs = [problem(n) for n in NAMES]
    stream = [(0.002 * i, p) for i, p in enumerate(probs)]
    with NativeServer(max_active=3, keep_u=True, tol=1e-11, mixed=mixed) as S:
        rep = S.run(stream)
    assert rep["completed"] == len(probs)
    assert rep["peak_concurrent_solves"] >= 2
    for p, r in zip(probs, rep["results"]):
        with og.Elliptic(p) as E:
            E.set_precision(mixed)
            solo = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=200, tol=1e-11)
            u = [E.get_field(g) for g in range(len(E.boxes))]
            adm = E.ADM_mass
        assert r.status == 0 and r.cycles == solo.cycles and r.final_res == solo.final_res
        assert r.adm == adm
        err = max(float(np.max(np.abs(a - b))) for a, b in zip(u, r.u))
        assert err == 0.0, err


@pytest.mark.gpu
def test_native_server_admits_by_memory():
    """A budget that holds one solve at a time runs them one after another."""
    from ollipticid_gb300.serve import NativeServer, footprint
    probs = [problem("o4_spin") for _ in range(3)]
    with NativeServer(mem_budget=footprint(probs[0]) + 1024, max_active=8, tol=1e-10) as S:
        rep = S.run([(0.0, p) for p in probs])
    assert [r.status for r in rep["results"]] == [0, 0, 0]
    assert rep["peak_concurrent_solves"] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [True, False], ids=["mixed", "fp64"])
def test_native_server_batching_matches_solo_solves(mixed):
    """The C++ server with batching (batch_max >= 2): requests admitted
    together are solved as one batch; every result (status, cycles, final
    norms, ADM masses) is the solo solve's bit for bit, and a request with a
    NaN mass fails alone."""
    import math
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    from ollipticid_gb300.serve import NativeServer
    probs = [problem(n) for n in NAMES]
    bad = problem("o4_spin")
    bad.mp = [math.nan]
    stream = [(0.0, p) for p in probs[:3]] + [(0.0, bad)] + [(0.01, p) for p in probs[3:]]
    rule = dict(stop=_abi.STOP_ERROR, max_cycles=100, tol=1e-10)
    with NativeServer(max_active=16, mixed=mixed, batch_max=4, batch_window=0.005, **rule) as S:
        rep = S.run(stream)
    res = rep["results"]
    assert res[3].status == _abi.ERR_NAN
    for i, p in enumerate(probs):
        r = res[i if i < 3 else i + 1]
        with og.Elliptic(p) as E:
            E.set_precision(mixed)
            solo = E.Solve(**rule)
        assert r.status == _abi.OK and r.cycles == solo.cycles, (i, r.cycles, solo.cycles)
        assert r.final_res == solo.final_res and r.final_du == solo.final_du
        assert list(r.adm) == list(solo.adm[:p.numbh])
