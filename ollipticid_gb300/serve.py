"""Continuous-batching server for puncture solves.

Requests arrive over time.  A request is admitted as soon as a slot and its
device-memory footprint are free; its hierarchy is built on a worker thread
(host geometry, plans, device allocation, coefficients, graph capture) while
the main loop keeps stepping the solves already on the GPU.  Every active
solve owns a CUDA stream; each round the loop enqueues the next V-cycle of
every solve whose previous cycle finished (olgpu_cycle_launch /
olgpu_cycle_poll), so the work of different requests overlaps on the device.
A solve leaves when its stop rule is met; its memory is released at once and
the next waiting request takes its place.

Latency is measured from a request's arrival to the end of its last cycle;
the report gives p50 / p99 latency and throughput (completed solves over the
makespan).
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import Elliptic, Problem, _abi
from ._abi import check

# device bytes per point: 12 FP64 fields and one mask byte (the points the
# discrete system fixes); mixed precision adds 11 FP32 fields, the
# colour-packed (A, 1/(c+u)) pairs and 9 FP32 Anderson vectors
BYTES_PER_POINT_MIXED = 12 * 8 + 11 * 4 + 2 * 4 + 9 * 4 + 1
BYTES_PER_POINT_FP64 = 12 * 8 + 1


def footprint(problem: Problem, mixed: bool = True) -> int:
    """Device bytes a solve of `problem` needs (from the host-only plan)."""
    lib = _abi.load()
    cp = problem.to_c()
    out = (_abi.BoxInfo * 512)()
    nb = C.c_int()
    check(lib.olgpu_plan_boxes(C.byref(cp), out, 512, C.byref(nb), None, None))
    pts = sum(out[g].nx * out[g].ny * out[g].nz for g in range(nb.value))
    return pts * (BYTES_PER_POINT_MIXED if mixed else BYTES_PER_POINT_FP64) + (64 << 20)


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float = 0.0
    started: float = 0.0
    finished: float = 0.0
    cycles: int = 0
    final_res: float = 0.0
    final_du: float = 0.0
    status: int = 0
    adm: List[float] = field(default_factory=list)
    u: Optional[list] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class _Track:
    """The stop rule of olgpu_solve: STOP_TOLERANCE (the cycle norm <= tol)
    or STOP_ERROR (its residual part <= tol and its largest change of u <=
    du_tol)."""

    def __init__(self, tol: float, max_cycles: int, stop: int = _abi.STOP_TOLERANCE, du_tol: float = 0.0):
        self.tol, self.max_cycles, self.stop = tol, max_cycles, stop
        self.du_tol = du_tol if du_tol > 0 else tol
        self.cycles = 0
        self.res = 1e12
        self.du = 0.0

    def step(self, res: float, part: float = None, du: float = 0.0) -> bool:
        self.cycles += 1
        self.res, self.du = res, du
        if self.cycles >= self.max_cycles:
            return True
        if self.stop == _abi.STOP_ERROR:
            return (res if part is None else part) <= self.tol and du <= self.du_tol
        return not (res > self.tol)


class Server:
    def __init__(self, device: int = 0, mem_budget: int = 64 << 30, max_active: int = 32, mixed: bool = True,
                 tol: Optional[float] = None, max_cycles: int = 200, builders: int = 2, keep_u: bool = False,
                 inner_sweeps: Optional[Tuple[int, ...]] = None, busy: int = 4, stop: int = _abi.STOP_TOLERANCE,
                 du_tol: float = 0.0):
        """stop: STOP_TOLERANCE or STOP_ERROR (with du_tol, 0: the
        tolerance), the rule of every solve.  inner_sweeps: (nu1, nu2[, smoother cluster blocks]) of every mixed
        solve's FP32 cycle (for example an autotune choice); None keeps each
        problem's own nu1/nu2 and the default smoother layout.  Without a
        layout in inner_sweeps the layout follows the load when a request is
        admitted: per-colour launches while fewer than `busy` solves are on
        the GPU (a solve alone is bound by its chain of launches), the
        cluster-resident smoother beyond (it holds fewer SMs per solve).  The
        two layouts give the same result bit for bit."""
        self.device, self.mem_budget, self.max_active = device, mem_budget, max_active
        self.mixed, self.tol, self.max_cycles, self.keep_u = mixed, tol, max_cycles, keep_u
        self.inner_sweeps, self.busy = inner_sweeps, busy
        self.stop, self.du_tol = stop, du_tol
        self.pool = ThreadPoolExecutor(max_workers=builders)

    def _build(self, problem: Problem, blocks: int) -> Elliptic:
        E = Elliptic(problem, device=self.device)
        if self.mixed:
            # the schedule first: set before the mixed cycle is captured, once
            E.set_smoother_blocks(blocks)
            if self.inner_sweeps:
                E.set_inner_sweeps(*self.inner_sweeps[:2])
        E.set_precision(self.mixed)
        return E

    def run(self, stream: Sequence[Tuple[float, Problem]]) -> dict:
        """Replays (arrival time, problem) pairs in real time; returns the report."""
        reqs = sorted(enumerate(stream), key=lambda r: r[1][0])
        pending = deque(reqs)
        waiting: deque = deque()
        building = []          # (future, rid, problem, bytes)
        active = []            # dicts
        results = {}
        used = 0
        peak_active = 0
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        while pending or waiting or building or active:
            t = now()
            while pending and pending[0][1][0] <= t:
                rid, (arr, prob) = pending.popleft()
                results[rid] = Result(rid, arr)
                if prob.method != "Vcycle":           # the scheduler steps V-cycles
                    results[rid].status = _abi.ERR_INVALID_ARG
                    results[rid].finished = now()
                    continue
                nbytes = footprint(prob, self.mixed)
                if nbytes > self.mem_budget:          # can never fit: refuse now
                    results[rid].status = _abi.ERR_OOM
                    results[rid].finished = now()
                    continue
                waiting.append((rid, arr, prob, nbytes))
            # admission: by slots and device-memory footprint, in arrival order
            while waiting and len(active) + len(building) < self.max_active and used + waiting[0][3] <= self.mem_budget:
                rid, arr, prob, nbytes = waiting.popleft()
                used += nbytes
                results[rid].admitted = now()
                if self.inner_sweeps and len(self.inner_sweeps) > 2:
                    blocks = self.inner_sweeps[2]
                else:
                    blocks = 0 if len(active) + len(building) < self.busy else 16
                building.append((self.pool.submit(self._build, prob, blocks), rid, prob, nbytes))
            for item in list(building):
                fut, rid, prob, nbytes = item
                if fut.done():
                    building.remove(item)
                    try:
                        E = fut.result()
                    except Exception as exc:            # e.g. out of device memory
                        results[rid].status = getattr(exc, "status", _abi.ERR_CUDA)
                        results[rid].finished = now()
                        used -= nbytes
                        continue
                    tol = self.tol if self.tol is not None else prob.tol
                    E.cycle_launch()
                    results[rid].started = now()
                    active.append({"rid": rid, "E": E, "bytes": nbytes,
                                   "track": _Track(tol, self.max_cycles, self.stop, self.du_tol)})
            peak_active = max(peak_active, len(active))
            progressed = False
            for a in list(active):
                status = _abi.OK
                try:
                    done, res = a["E"].cycle_poll(False)
                except _abi.OlgpuError as exc:      # e.g. NaN: this request ends, the others go on
                    done, res, status = True, float("nan"), exc.status
                if not done:
                    continue
                progressed = True
                part, du = a["E"].last_cycle()
                if status != _abi.OK or a["track"].step(res, part, du):
                    r = results[a["rid"]]
                    r.finished = now()
                    r.status = status
                    r.cycles, r.final_res, r.final_du = a["track"].cycles + (status != _abi.OK), res, du
                    r.adm = a["E"].ADM_mass
                    if self.keep_u and status == _abi.OK:
                        r.u = [a["E"].get_field(g) for g in range(len(a["E"].boxes))]
                    a["E"].close()
                    used -= a["bytes"]
                    active.remove(a)
                else:
                    a["E"].cycle_launch()
            if not progressed:
                time.sleep(20e-6)
        makespan = max(r.finished for r in results.values()) - min(r.arrival for r in results.values())
        lat = np.array([results[i].latency for i in sorted(results)])
        return {
            "completed": len(results),
            "makespan_s": makespan,
            "throughput_solves_per_s": len(results) / makespan if makespan > 0 else float("nan"),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()),
            "cycles_mean": float(np.mean([r.cycles for r in results.values()])),
            "peak_concurrent_solves": peak_active,
            "results": [results[i] for i in sorted(results)],
        }


class NativeServer:
    """The library's own continuous-batching server (olgpu_server_*, server.cpp):
    C++ builder threads make the hierarchies and a C++ scheduler thread admits
    requests and keeps their cycles queued; Python only submits and polls.
    Same admission rule, smoother layout policy and stop rule as `Server`."""

    def __init__(self, device: int = 0, mem_budget: int = 64 << 30, max_active: int = 32, mixed: bool = True,
                 tol: Optional[float] = None, max_cycles: int = 200, builders: int = 2, keep_u: bool = False,
                 inner_sweeps: Optional[Tuple[int, ...]] = None, busy: int = 4, stop: int = _abi.STOP_TOLERANCE,
                 du_tol: float = 0.0, keep_only=None, batch_max: int = 0, batch_window: float = 0.02):
        """keep_u: hand every result's u back; keep_only (a set of indices
        into the stream given to run(), with keep_u) limits that to those
        requests.  batch_max >= 2: requests admitted together (up to
        batch_max, after at most batch_window seconds of waiting) are solved
        as one batch (no keep_u then)."""
        self.lib = _abi.load()
        self.keep_only = keep_only
        self._keep_rids = None
        c = _abi.ServerConfig()
        self.lib.olgpu_server_config_defaults(C.byref(c))
        c.device, c.mem_budget, c.max_active = device, mem_budget, max_active
        c.precision = _abi.PREC_MIXED if mixed else _abi.PREC_FP64
        c.stop, c.max_cycles, c.tol, c.builders, c.busy = stop, max_cycles, tol or 0.0, builders, busy
        if inner_sweeps:
            c.nu1, c.nu2 = inner_sweeps[0], inner_sweeps[1]
            c.blocks = inner_sweeps[2] if len(inner_sweeps) > 2 else -1
        c.keep_solutions = 1 if keep_u else 0
        c.du_tol = du_tol
        c.batch_max, c.batch_window = batch_max, batch_window
        self.keep_u = keep_u
        s = C.c_void_p()
        check(self.lib.olgpu_server_create(C.byref(c), C.byref(s)))
        self._s = s
        self._problems = {}

    def submit(self, problem: Problem) -> int:
        cp = problem.to_c()
        rid = C.c_longlong()
        check(self.lib.olgpu_server_submit(self._s, C.byref(cp), C.byref(rid)))
        self._problems[rid.value] = problem
        return rid.value

    def poll(self, rid: int, wait: bool = True) -> Optional[Result]:
        out = _abi.ServerResult()
        done = C.c_int()
        check(self.lib.olgpu_server_poll(self._s, rid, 1 if wait else 0, C.byref(done), C.byref(out)))
        if not done.value:
            return None
        r = Result(rid, 0.0, cycles=out.cycles, final_res=out.final_res, final_du=out.final_du, status=out.status)
        r.admitted = out.queue_s
        r.finished = out.latency_s          # relative to arrival
        nbh = self._problems.pop(rid).numbh
        r.adm = [out.adm[i] for i in range(nbh)]
        if out.h:
            h = C.c_void_p(out.h)
            if self.keep_u and (self._keep_rids is None or rid in self._keep_rids):
                r.u = []
                for g in range(self.lib.olgpu_num_boxes(h)):
                    bi = _abi.BoxInfo()
                    check(self.lib.olgpu_box(h, g, C.byref(bi)))
                    a = np.empty((bi.nz, bi.ny, bi.nx))
                    check(self.lib.olgpu_download(h, g, b"u", a.ctypes.data_as(C.c_void_p)))
                    r.u.append(a)
            self.lib.olgpu_hierarchy_destroy(h)
        return r

    def stats(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        check(self.lib.olgpu_server_stats(self._s, *(C.byref(x) for x in v)))
        return dict(zip(("active", "building", "waiting", "peak_active"), (x.value for x in v)))

    def run(self, stream: Sequence[Tuple[float, Problem]]) -> dict:
        """Submits (arrival time, problem) pairs in real time from a thread
        while this one collects the results as they finish (so that a
        finished solve's memory is released at once); the report has the
        keys of `Server.run`."""
        import threading
        reqs = sorted(enumerate(stream), key=lambda r: r[1][0])
        t0 = time.perf_counter()
        ids = {}
        lock = threading.Lock()
        if self.keep_only is not None:
            self._keep_rids = set()

        def submitter():
            for i, (arr, prob) in reqs:
                delay = arr - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                with lock:
                    rid = self.submit(prob)
                    ids[i] = (rid, time.perf_counter() - t0)
                    if self.keep_only is not None and i in self.keep_only:
                        self._keep_rids.add(rid)

        th = threading.Thread(target=submitter)
        th.start()
        results = {}
        while len(results) < len(reqs):
            with lock:
                pending = [(i, v) for i, v in ids.items() if i not in results]
            got = False
            for i, (rid, arrival) in pending:
                with lock:
                    r = self.poll(rid, wait=False)
                if r is None:
                    continue
                got = True
                r.rid, r.arrival = i, arrival
                r.admitted += arrival
                r.finished += arrival
                results[i] = r
            if not got:
                time.sleep(0.002)
        th.join()
        makespan = max(r.finished for r in results.values()) - min(r.arrival for r in results.values())
        lat = np.array([results[i].latency for i in sorted(results)])
        return {
            "completed": len(results),
            "makespan_s": makespan,
            "throughput_solves_per_s": len(results) / makespan if makespan > 0 else float("nan"),
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_max_s": float(lat.max()),
            "cycles_mean": float(np.mean([r.cycles for r in results.values()])),
            "peak_concurrent_solves": self.stats()["peak_active"],
            "results": [results[i] for i in sorted(results)],
        }

    def close(self):
        if getattr(self, "_s", None):
            self.lib.olgpu_server_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
