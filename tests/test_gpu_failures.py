"""Failure paths, with every fault made on the host (no GPU fault).

* A NaN in u (uploaded into one interior point) makes the smoother report
  OLGPU_ERR_NAN, where the reference calls exit(0) (src/elliptic.cc:1194-1207);
  the hierarchy stays usable: after a reset the same problem solves.
* In a set solved together (olgpu_solve_many) and in both servers, the one
  request that fails (a NaN in its u, or a NaN puncture mass) ends with
  OLGPU_ERR_NAN and every other result is its solo result bit for bit.
* A W-cycle level that cannot meet its tolerance within the per-level cap
  ends the solve with OLGPU_ERR_DIVERGED instead of looping forever (the
  reference has no cap, src/elliptic.cc:1956).
"""
import math

import numpy as np
import pytest

from tests.cases import problem


def poison(E, level=None):
    """A NaN at the centre of the first box of `level` (default: the finest)."""
    level = E.levels - 1 if level is None else level
    g = E.box_index(level, 0)
    u = E.get_field(g)
    nz, ny, nx = u.shape
    u[nz // 2, ny // 2, nx // 2] = np.nan
    E.set_field(g, "u", u)


def solo(P, mixed, rule):
    import ollipticid_gb300 as og
    with og.Elliptic(P) as E:
        E.set_precision(mixed)
        rep = E.Solve(**rule)
        return [E.get_field(g) for g in range(len(E.boxes))], rep.cycles


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_nan_in_u_is_reported_and_the_hierarchy_recovers(mixed):
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi

    P = problem("o4_spin")
    rule = dict(stop=_abi.STOP_ERROR, max_cycles=100, tol=1e-10)
    with og.Elliptic(P) as E:
        E.set_precision(mixed)
        poison(E)
        with pytest.raises(og.OlgpuError) as exc:
            E.Solve(**rule)
        assert exc.value.status == _abi.ERR_NAN
        assert E.last_report.status == _abi.ERR_NAN and E.last_report.cycles == 1
        E.reset()
        rep = E.Solve(**rule)
        assert rep.status == _abi.OK and rep.final_res <= 1e-10
        u = [E.get_field(g) for g in range(len(E.boxes))]
    want, _ = solo(P, mixed, rule)
    assert all(np.array_equal(a, b) for a, b in zip(u, want))


@pytest.mark.gpu
def test_one_failed_solve_leaves_the_others_untouched():
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi

    names = ["o4_spin", "o2_single", "sf_binary"]
    rule = dict(stop=_abi.STOP_ERROR, max_cycles=100, tol=1e-10)
    sol = [og.Elliptic(problem(n)) for n in names]
    try:
        for E in sol:
            E.set_precision(True)
        poison(sol[1])
        reps = og.solve_many(sol, raise_on_error=False, **rule)
        assert [r.status for r in reps] == [_abi.OK, _abi.ERR_NAN, _abi.OK]
        for i in (0, 2):
            want, cycles = solo(problem(names[i]), True, rule)
            got = [sol[i].get_field(g) for g in range(len(sol[i].boxes))]
            assert reps[i].cycles == cycles
            assert all(np.array_equal(a, b) for a, b in zip(got, want)), names[i]
    finally:
        for E in sol:
            E.close()


@pytest.mark.gpu
@pytest.mark.parametrize("native", [False, True])
def test_server_isolates_a_failing_request(native):
    from ollipticid_gb300 import _abi
    from ollipticid_gb300.serve import NativeServer, Server

    good = [problem("o4_spin"), problem("o2_single")]
    bad = problem("o4_spin")
    bad.mp = [math.nan]
    stream = [(0.0, good[0]), (0.0, bad), (0.0, good[1])]
    kw = dict(mem_budget=8 << 30, max_active=4, tol=1e-10, max_cycles=100, keep_u=True,
              stop=_abi.STOP_ERROR)
    if native:
        with NativeServer(**kw) as S:
            rep = S.run(stream)
    else:
        rep = Server(**kw).run(stream)
    res = rep["results"]
    assert [r.status for r in res] == [_abi.OK, _abi.ERR_NAN, _abi.OK]
    for r, P in ((res[0], good[0]), (res[2], good[1])):
        want, cycles = solo(P, True, dict(stop=_abi.STOP_ERROR, max_cycles=100, tol=1e-10))
        assert r.cycles == cycles
        assert all(np.array_equal(a, b) for a, b in zip(r.u, want))


@pytest.mark.gpu
def test_wcycle_level_cap_reports_divergence():
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi

    P = problem("o2_single")
    P.method = "Wcycle"
    with og.Elliptic(P) as E:
        with pytest.raises(og.OlgpuError) as exc:
            E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=2, tol=1e-14)
        assert exc.value.status == _abi.ERR_DIVERGED
        assert "did not reach the tolerance" in str(exc.value)
        # the hierarchy is still usable: the same problem solves afterwards
        E.reset()
        rep = E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=100, tol=1e-9)
        assert rep.status == _abi.OK and rep.final_res <= 1e-9
