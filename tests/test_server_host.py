"""The C++ server's host side without a GPU: its threads start and stop, a
request that can never fit is refused at once with OLGPU_ERR_OOM, a request
whose build fails reports the failure as its status (no fallback), a
W-cycle request (the scheduler steps V-cycles) is refused at submission, and
a result can be collected once."""
import ctypes as C

import pytest

from ollipticid_gb300 import _abi
from tests.cases import problem


def test_server_refuses_and_reports_without_a_device():
    lib = _abi.load()
    cfg = _abi.ServerConfig()
    lib.olgpu_server_config_defaults(C.byref(cfg))
    assert cfg.max_active > 0 and cfg.builders > 0 and cfg.blocks == -1
    cfg.device = 9999                      # no such device here or on a one-GPU machine
    cfg.mem_budget = 256 << 20
    s = C.c_void_p()
    assert lib.olgpu_server_create(C.byref(cfg), C.byref(s)) == _abi.OK
    try:
        big = problem("-eq Punctures -NumBH 1 -bhmp1 0.5 -N 129 -L 40 -O 4 -l 6").to_c()
        small = problem("o4_spin").to_c()
        ids = []
        for p in (big, small):
            rid = C.c_longlong()
            assert lib.olgpu_server_submit(s, C.byref(p), C.byref(rid)) == _abi.OK
            ids.append(rid.value)
        out = _abi.ServerResult()
        done = C.c_int()
        assert lib.olgpu_server_poll(s, ids[0], 1, C.byref(done), C.byref(out)) == _abi.OK
        assert done.value == 1 and out.status == _abi.ERR_OOM and out.id == ids[0]
        assert lib.olgpu_server_poll(s, ids[1], 1, C.byref(done), C.byref(out)) == _abi.OK
        assert done.value == 1 and out.status not in (_abi.OK, _abi.ERR_OOM) and not out.h
        assert lib.olgpu_server_poll(s, ids[1], 0, C.byref(done), C.byref(out)) == _abi.OK and done.value == 0
        assert lib.olgpu_server_poll(s, 12345, 0, C.byref(done), C.byref(out)) == _abi.ERR_INVALID_ARG
        w = problem("o4_spin")
        w.method = "Wcycle"
        wp, rid = w.to_c(), C.c_longlong()
        assert lib.olgpu_server_submit(s, C.byref(wp), C.byref(rid)) == _abi.ERR_INVALID_ARG
        v = [C.c_int() for _ in range(4)]
        assert lib.olgpu_server_stats(s, *(C.byref(x) for x in v)) == _abi.OK
        assert [x.value for x in v[:3]] == [0, 0, 0]
    finally:
        assert lib.olgpu_server_destroy(s) == _abi.OK


def test_server_config_is_checked():
    lib = _abi.load()
    cfg = _abi.ServerConfig()
    lib.olgpu_server_config_defaults(C.byref(cfg))
    cfg.max_active = 0
    s = C.c_void_p()
    assert lib.olgpu_server_create(C.byref(cfg), C.byref(s)) == _abi.ERR_INVALID_ARG


def test_server_batching_config_and_a_failed_batch():
    """Batching (batch_max >= 2) refuses keep_solutions (a batch's
    hierarchies are not handed out); without a device, a group's batch
    cannot be made and every request of it fails with its own status."""
    lib = _abi.load()
    cfg = _abi.ServerConfig()
    lib.olgpu_server_config_defaults(C.byref(cfg))
    assert cfg.batch_max == 0 and cfg.batch_window > 0
    cfg.batch_max, cfg.keep_solutions = 4, 1
    s = C.c_void_p()
    assert lib.olgpu_server_create(C.byref(cfg), C.byref(s)) == _abi.ERR_INVALID_ARG
    cfg.keep_solutions, cfg.device, cfg.batch_window = 0, 9999, 0.0
    assert lib.olgpu_server_create(C.byref(cfg), C.byref(s)) == _abi.OK
    try:
        ids = []
        for name in ("o4_spin", "o2_single"):
            p, rid = problem(name).to_c(), C.c_longlong()
            assert lib.olgpu_server_submit(s, C.byref(p), C.byref(rid)) == _abi.OK
            ids.append(rid.value)
        out, done = _abi.ServerResult(), C.c_int()
        for rid in ids:
            assert lib.olgpu_server_poll(s, rid, 1, C.byref(done), C.byref(out)) == _abi.OK
            assert done.value == 1 and out.id == rid and out.status != _abi.OK and not out.h
    finally:
        assert lib.olgpu_server_destroy(s) == _abi.OK


def test_python_scheduler_refuses_a_wcycle_request():
    """The Python scheduler steps V-cycles too: a W-cycle request is refused
    on arrival, before any device work."""
    from ollipticid_gb300.serve import Server
    w = problem("o4_spin")
    w.method = "Wcycle"
    S = Server(device=9999)
    rep = S.run([(0.0, w)])
    assert rep["completed"] == 1 and rep["results"][0].status == _abi.ERR_INVALID_ARG
