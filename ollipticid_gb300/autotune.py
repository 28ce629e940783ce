"""Sweep-schedule and smoother-layout autotuner for the mixed-precision solve.

The FP32 correction cycle of a mixed-precision solve may use any number of
pre- and post-smoothing sweeps: the FP64 defect that drives it fixes the
solution, so the schedule changes only the work per outer cycle and the
number of outer cycles (`olgpu_set_inner_sweeps`).  Which schedule is fastest
depends on the problem's shape and on how many solves share the GPU (with
many concurrent solves the GPU is full and fewer sweeps per cycle win; a
solve alone is bound by launch latency).  `tune` measures a small set of
candidates on the problem itself, `concurrency` copies at a time through
`solve_many`, each to the same stop rule, and returns the fastest.  The
candidates also choose the FP32 smoother's layout (`olgpu_set_smoother_blocks`):
a thread-block cluster per box keeping the correction in shared memory for
every sweep (blocks = 16), or one launch per colour and sweep (blocks = 0),
which wins for a solve alone.  Results
are cached per problem shape (equation, order, N, levels, punctures) and
concurrency, in memory and optionally in a JSON file.  `tune_batch` makes
the same choice for a batch of uneven problems (`olgpu_batch_*`) by timing
one batch solve per candidate on the problems themselves.
"""
from __future__ import annotations

import json
import os
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

from . import Elliptic, Problem, _abi, solve_many

# (nu1, nu2, smoother cluster blocks) candidates: the reference's own (3, 20)
# and lighter schedules (more pre- than post-smoothing pays: fewer outer
# cycles), cluster-resident or per-colour smoothing
CANDIDATES: Tuple[Tuple[int, int, int], ...] = ((3, 20, 16), (3, 8, 16), (4, 6, 16), (4, 4, 16), (5, 4, 16),
                                                (5, 6, 16), (6, 4, 16), (4, 6, 0), (3, 8, 0), (2, 4, 0))

# candidates for batches: the schedules that win for many solves at once
# (lighter ones win on the batched binaries: (3, 3) and (4, 3) ahead of
# (4, 4) and (4, 6)), cluster-resident or per-colour smoothing
BATCH_CANDIDATES: Tuple[Tuple[int, int, int], ...] = ((4, 6, 16), (4, 4, 16), (4, 4, 0), (4, 3, 0), (3, 3, 16),
                                                      (3, 3, 0))

_lock = threading.Lock()
_memo: Dict[str, "Choice"] = {}


@dataclass
class Choice:
    nu1: int
    nu2: int
    blocks: int
    solves_per_s: float
    cycles: int
    table: List[dict] = field(default_factory=list)   # every candidate's measurement

    def to_dict(self) -> dict:
        return {"nu1": self.nu1, "nu2": self.nu2, "blocks": self.blocks, "solves_per_s": self.solves_per_s,
                "cycles": self.cycles, "table": self.table}

    @staticmethod
    def from_dict(d: dict) -> "Choice":
        return Choice(d["nu1"], d["nu2"], d.get("blocks", 16), d["solves_per_s"], d["cycles"], d.get("table", []))

    def apply(self, E: Elliptic) -> None:
        """Sets this choice on a mixed-precision solver."""
        E.set_smoother_blocks(self.blocks)
        E.set_inner_sweeps(self.nu1, self.nu2)


def shape_key(p: Problem, concurrency: int) -> str:
    """Problems with the same key have the same hierarchy shape and stencil."""
    return f"eq{p.equation}_O{p.order}_N{p.n}_l{p.levels}_bh{p.numbh}_c{concurrency}"


def _load(path: Optional[str]) -> dict:
    if path and os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def tune(p: Problem, concurrency: int = 8, candidates: Sequence[Tuple[int, int, int]] = CANDIDATES,
         tol: Optional[float] = None, max_cycles: int = 200, cache_path: Optional[str] = None,
         device: int = 0, repeats: int = 1) -> Choice:
    """Fastest inner schedule for `concurrency` concurrent mixed solves of p."""
    key = shape_key(p, concurrency)
    with _lock:
        if key in _memo:
            return _memo[key]
        disk = _load(cache_path)
        if key in disk:
            _memo[key] = Choice.from_dict(disk[key])
            return _memo[key]
    tol = p.tol if tol is None else tol
    sol = [Elliptic(p, device=device) for _ in range(concurrency)]
    table = []
    try:
        for E in sol:
            E.set_precision(True)
        for nu1, nu2, blocks in candidates:
            for E in sol:
                E.set_smoother_blocks(blocks)
                E.set_inner_sweeps(nu1, nu2)
            for E in sol:                      # warm-up (first launches of the new graph)
                E.reset()
            solve_many(sol, stop=_abi.STOP_TOLERANCE, max_cycles=max_cycles, tol=tol)
            best = None
            for _ in range(repeats):
                for E in sol:
                    E.reset()
                t = time.perf_counter()
                reps = solve_many(sol, stop=_abi.STOP_TOLERANCE, max_cycles=max_cycles, tol=tol)
                dt = time.perf_counter() - t
                ok = all(r.final_res <= tol for r in reps)
                rate = concurrency / dt if ok else 0.0
                best = rate if best is None else max(best, rate)
            table.append({"nu1": nu1, "nu2": nu2, "blocks": blocks, "solves_per_s": best, "cycles": int(reps[0].cycles),
                          "reached_tol": ok})
    finally:
        for E in sol:
            E.close()
    top = max(table, key=lambda r: r["solves_per_s"])
    choice = Choice(top["nu1"], top["nu2"], top["blocks"], top["solves_per_s"], top["cycles"], table)
    with _lock:
        _memo[key] = choice
        if cache_path:
            disk = _load(cache_path)
            disk[key] = choice.to_dict()
            tmp = cache_path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(disk, f, indent=1)
            os.replace(tmp, cache_path)
    return choice


def cached(p: Problem, concurrency: int = 8, cache_path: Optional[str] = None) -> Optional[Choice]:
    """The cached choice for p's shape, or None (never measures)."""
    key = shape_key(p, concurrency)
    with _lock:
        if key in _memo:
            return _memo[key]
    d = _load(cache_path).get(key)
    return Choice.from_dict(d) if d else None


def tune_batch(problems: Sequence[Problem], candidates: Sequence[Tuple[int, int, int]] = BATCH_CANDIDATES,
               tol: float = 1e-10, du_tol: float = 0.0, max_cycles: int = 300) -> Choice:
    """Fastest (nu1, nu2, blocks) for solving `problems` as one mixed-precision
    batch: each candidate's batch is built, solved once to warm up and once
    timed (host wall clock of olgpu_batch_solve), every solve under the same
    stop rule (OLGPU_STOP_ERROR with tol and du_tol, or the residual alone
    when du_tol is 0).  Not cached: a batch is a set of problems, not a
    shape."""
    from . import Batch
    rule = dict(stop=_abi.STOP_ERROR if du_tol > 0 else _abi.STOP_TOLERANCE, max_cycles=max_cycles, tol=tol,
                du_tol=du_tol)
    table = []
    for nu1, nu2, blocks in candidates:
        with Batch(problems, mixed=True, inner_sweeps=(nu1, nu2), blocks=blocks) as B:
            B.solve(**rule)
            B.reset()
            reps = B.solve(**rule)
            ok = all(r.status == _abi.OK and (r.final_part <= tol and r.final_du <= du_tol if du_tol > 0
                                              else r.final_res <= tol) for r in reps)
            rate = len(problems) / (B.last_ms / 1000.0) if ok else 0.0
        table.append({"nu1": nu1, "nu2": nu2, "blocks": blocks, "solves_per_s": rate,
                      "cycles": int(max(r.cycles for r in reps)), "reached_tol": ok})
    top = max(table, key=lambda r: r["solves_per_s"])
    return Choice(top["nu1"], top["nu2"], top["blocks"], top["solves_per_s"], top["cycles"], table)
