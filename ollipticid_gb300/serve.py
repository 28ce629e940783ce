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

# device bytes per point: 11 FP64 fields, 11 FP32 fields, 9 FP32 Anderson
# vectors, one mask byte (mixed precision); 11 FP64 fields in plain FP64
BYTES_PER_POINT_MIXED = 11 * 8 + 11 * 4 + 9 * 4 + 1
BYTES_PER_POINT_FP64 = 11 * 8


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
    status: int = 0
    adm: List[float] = field(default_factory=list)
    u: Optional[list] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class _Track:
    """The stop rule of olgpu_solve (tolerance on the cycle norm)."""

    def __init__(self, tol: float, max_cycles: int):
        self.tol, self.max_cycles = tol, max_cycles
        self.cycles = 0
        self.res = 1e12

    def step(self, res: float) -> bool:
        self.cycles += 1
        self.res = res
        return not (res > self.tol) or self.cycles >= self.max_cycles


class Server:
    def __init__(self, device: int = 0, mem_budget: int = 64 << 30, max_active: int = 32, mixed: bool = True,
                 tol: Optional[float] = None, max_cycles: int = 200, builders: int = 2, keep_u: bool = False,
                 inner_sweeps: Optional[Tuple[int, ...]] = None, busy: int = 4):
        """inner_sweeps: (nu1, nu2[, smoother cluster blocks]) of every mixed
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
                    active.append({"rid": rid, "E": E, "track": _Track(tol, self.max_cycles), "bytes": nbytes})
            peak_active = max(peak_active, len(active))
            progressed = False
            for a in list(active):
                done, res = a["E"].cycle_poll(False)
                if not done:
                    continue
                progressed = True
                if a["track"].step(res):
                    r = results[a["rid"]]
                    r.finished = now()
                    r.cycles, r.final_res = a["track"].cycles, res
                    r.adm = a["E"].ADM_mass
                    if self.keep_u:
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
