"""Benchmark: puncture FAS solves/s on one GB300, plain FP64.

Workload (one step = one full solve): the equal-mass binary of the reference's
pars/Punctures/TestBH.run at 4th order -- two punctures m=0.487209 at
y=+-5.5 with momenta (-+0.0901099, -+0.000703975, 0), Robin boundary, N=65,
9 refinement levels, L=1000, 20 post-smoothing sweeps, solved from u = 0
until the top-level residual is <= 1e-11 and the cycle's largest change of u
is <= 5e-11 (so that u ends within 1e-10 of the fixed point on every level,
which the accuracy keys check against the reference's own fixed point).
Inputs are synthetic (the reference ships no data set; the problem is
defined by its command line).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

--impl reference times complete solves of the same workload on the host CPU
cores by the oracle port (a bit-exact restatement of the reference's CPU
solver) under the reference's own stop rule.  With torchrun (N > 1) every rank solves its own copies of the
workload on its own GPU (replicas: one solve never spans GPUs) and rank 0
prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD_ARGS = ("-eq Punctures -B Robin -BA 0.0 -Bn 1 -NumBH 2 -bhmp1 0.487209 -bhy1 5.5 -bhpx1 -0.0901099 "
                 "-bhpy1 -0.000703975 -bhmp2 0.487209 -bhy2 -5.5 -bhpx2 0.0901099 -bhpy2 0.000703975 "
                 "-L 1000 -N 65 -O 4 -l 9 -s 1e-11 -Dp 0.05 -nu2 20")
WORKLOAD_NAME = "binary_O4_N65_l9_L1000_tol1e-11"
METRIC = "puncture solves/s to 1e-10 (served FP32/FP64 vs plain FP64); p99 latency; GB/s"
UNIT = "solves/s"
# The timed stop (OLGPU_STOP_ERROR): top-level residual <= the problem's
# tolerance (1e-11) and the cycle's largest change of u on every fixed point
# <= half the metric's 1e-10 accuracy bar, so that u ends within 1e-10 of the
# fixed point on every level (the reference's own rule, residual only, ends
# this workload 1e-9 away).
DU_TOL = 5e-11
CONCURRENT_SOLVES = 16   # solves sharing the GPU in the concurrent and smoother-rate measurements
SERVED_SLOTS = 16        # the C++ server's slots for the served binaries (24 and 32 measured no faster)
ACCEL = 4   # Anderson depth of the plain FP64 iteration (FP64 history and sums)
SMOOTH_BYTES_PER_POINT = 40          # read u, b, c, S; write u (FP64)
# DRAM bytes (read + write), FP64-pipe occupancy and FP64 instructions per
# point-update of one finest-level launch of k_smooth_color<4,0> on this
# workload, from an ncu capture (dram__bytes_read.sum + dram__bytes_write.sum;
# sm__inst_executed_pipe_fp64.avg.pct_of_peak_sustained_active; that
# occupancy x sm__cycles_active.avg x 2 per clock x 152 SMs / point-updates)
SMOOTH_TRAFFIC_PER_LAUNCH = 17_598_208
SMOOTH_FP64_PIPE_PCT = 64.6
SMOOTH_FP64_INST_PER_POINT = 28.0
GOLDEN = os.path.join(ROOT, "tests", "golden", "configs")


def bench_config():
    """The workload as both arms name it (static: no measured values)."""
    return {"workload": WORKLOAD_NAME, "args": WORKLOAD_ARGS,
            "stop": f"top-level residual <= 1e-11 and the cycle's largest change of u <= {DU_TOL:g}",
            "l2": "256 MiB buffer written before every timed solve (the 370 MB arena also exceeds L2)",
            "boxes": 13, "points": 3852011}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------
# CPU side (oracle port of the reference solver): complete solves
# ----------------------------------------------------------------------------
def _cpu_solver(args):
    """One process: `n` complete solves of the workload by the oracle port
    under the reference's own stop rule (src/elliptic.cc:1330), each timed
    from u = 0 to the stop; the hierarchy is built once, outside the timing
    (the GPU arm's hierarchy is also resident)."""
    n, q = args
    from oracle import oracle as O
    import ollipticid_gb300 as og
    P = og.parse_olliptic_args(WORKLOAD_ARGS.split())
    out = []
    for _ in range(n):
        orc = O.Oracle(P.oracle_dict())
        t0 = time.perf_counter()
        cycles, res = orc.solve()
        out.append((time.perf_counter() - t0, cycles, res))
        orc.close()
    q.put(out)


def cpu_solves(total: int, procs: int):
    """`total` complete CPU solves spread over `procs` single-threaded
    processes (spawned); returns (aggregate solves/s of the busy processes,
    wall seconds, per-solve records)."""
    from oracle import oracle as O
    O.build()
    procs = max(1, min(procs, total))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    share = [total // procs + (1 if i < total % procs else 0) for i in range(procs)]
    ps = [ctx.Process(target=_cpu_solver, args=((n, q),)) for n in share]
    t0 = time.perf_counter()
    for p in ps:
        p.start()
    recs = [q.get() for _ in ps]
    wall = time.perf_counter() - t0
    for p in ps:
        p.join()
    rate = sum(len(r) / sum(t for t, _, _ in r) for r in recs)
    return rate, wall, [x for r in recs for x in r]


class CpuBaseline:
    """One complete single-core solve, run in a spawned process beside the
    GPU work (one host core of the GPU machine's 16)."""

    def __init__(self):
        from oracle import oracle as O
        O.build()
        ctx = mp.get_context("spawn")
        self.q = ctx.Queue()
        self.p = ctx.Process(target=_cpu_solver, args=((1, self.q),))
        self.p.start()

    def result(self):
        (t, cycles, res), = self.q.get()
        self.p.join()
        return {"value": 1.0 / t, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": f"one complete single-threaded solve of this workload by the oracle port under the "
                          f"reference's stop rule: {cycles} V-cycles to residual {res:.3g} in {t:.1f} s"}


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    procs = min(os.cpu_count() or 1, max(1, args.steps))
    rate, wall, recs = cpu_solves(args.steps, procs)
    cyc = sorted({c for _, c, _ in recs})
    line = {
        "impl": "reference",
        "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{args.steps} complete solves of the workload (the reference's stop rule, "
                                   f"{'/'.join(map(str, cyc))} V-cycles each) by the oracle port in {procs} "
                                   f"single-threaded processes; value = the sum of the processes' solve rates, "
                                   f"ms_per_step = wall / steps ({wall:.1f} s); the hierarchy is built before each "
                                   f"solve's timing; no warm-up (a CPU solve has nothing to warm)"},
        "solves": [{"s": t, "cycles": c, "final_res": r} for t, c, r in recs],
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nme, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nme)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _flush_l2(dev):
    import torch
    buf = getattr(_flush_l2, "buf", None)
    if buf is None:
        buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
        _flush_l2.buf = buf
    buf.fill_(1.0)
    torch.cuda.synchronize(dev)


def pinned_max_diff(E, a, b):
    """max |a - b| over the points the discrete system fixes (all points of
    the base and refinement levels, the interior of coarser multigrid levels)."""
    worst = 0.0
    for g, box in enumerate(E.boxes):
        x, y = a[g], b[g]
        if box.level < E.mgrid_levels:
            w = box.buf
            x, y = x[w:-w, w:-w, w:-w], y[w:-w, w:-w, w:-w]
        worst = max(worst, float(abs(x - y).max()))
    return worst


def load_fixture(name):
    """The reference's fixed point of a benchmark problem, sampled
    (tests/golden/configs, made by tests/golden/make_config_golden.py)."""
    import numpy as np
    path = os.path.join(GOLDEN, f"{name}.npz")
    return np.load(path) if os.path.exists(path) else None


def reference_error(E, fx, u=None, adm=None):
    """max |u - u_reference| at the fixture's sample points the discrete
    system fixes, and the ADM masses' differences; u: per-box arrays (default:
    the hierarchy's current u)."""
    import numpy as np
    if fx is None:
        return None
    worst, count = 0.0, 0
    for g, box in enumerate(E.boxes):
        x = (E.get_field(g) if u is None else u[g]).ravel()
        idx = fx[f"idx_b{g}"].astype(np.int64)
        want = fx[f"fixed_u_b{g}"]
        if box.level < E.mgrid_levels:
            nx, ny, nz = box.n
            k, rem = np.divmod(idx, nx * ny)
            j, i = np.divmod(rem, nx)
            w = box.buf
            keep = (i >= w) & (i < nx - w) & (j >= w) & (j < ny - w) & (k >= w) & (k < nz - w)
            idx, want = idx[keep], want[keep]
        worst = max(worst, float(np.max(np.abs(x[idx] - want))))
        count += len(idx)
    adm = E.ADM_mass if adm is None else adm
    return {"max_abs_u_minus_reference": worst,
            "adm_minus_reference": [float(a - b) for a, b in zip(adm, fx["fixed_adm"])],
            "reference_points": count, "reference_source": str(fx["fixed_source"])}


def fixed_point(E, du_tol=1e-13, max_cycles=300):
    """The GPU's own FP64 fixed point (untimed): cycles until the largest
    change of u is <= du_tol; returns u per box."""
    from ollipticid_gb300 import _abi
    E.set_precision(False)
    E.reset()
    E.Solve(stop=_abi.STOP_ERROR, max_cycles=max_cycles, tol=E.problem.tol, du_tol=du_tol)
    return [E.get_field(g) for g in range(len(E.boxes))]


def timed_solves(E, steps, dev, tol, du_tol=DU_TOL):
    """`steps` solves from u = 0 under the timed stop, L2 flushed before each;
    (device ms, reports)."""
    from ollipticid_gb300 import _abi
    ms, reps = 0.0, []
    for _ in range(steps):
        _flush_l2(dev)
        E.reset()
        rep = E.Solve(stop=_abi.STOP_ERROR, max_cycles=300, tol=tol, du_tol=du_tol)
        if not (rep.final_part <= tol and rep.final_du <= du_tol):
            raise RuntimeError(f"solve stopped at residual {rep.final_part:.3g}, change {rep.final_du:.3g}")
        ms += E.last_device_ms
        reps.append(rep)
    return ms, reps


def run_mixed(E, P, args, dev, u_fix, fx):
    """Solves/s of the mixed-precision cycle on the same workload under the
    same stop (finest FP64 defect <= tol, change of u <= DU_TOL), with its
    deviation from the reference's fixed point and from the GPU's FP64 one."""
    E.set_precision(True)
    timed_solves(E, args.warmup, dev, P.tol)
    ms, reps = timed_solves(E, args.steps, dev, P.tol)
    u = [E.get_field(g) for g in range(len(E.boxes))]
    ref = reference_error(E, fx, u, reps[-1].adm[:2])
    # the same solve alone with the schedule the autotuner picks for one solve
    from ollipticid_gb300 import autotune
    choice = autotune.tune(P, concurrency=1)
    choice.apply(E)
    tms, treps = timed_solves(E, args.steps, dev, P.tol)
    tu = [E.get_field(g) for g in range(len(E.boxes))]
    tuned = {"value": args.steps / (tms / 1000.0), "ms_per_step": tms / args.steps,
             "inner_sweeps": [choice.nu1, choice.nu2], "smoother_blocks": choice.blocks,
             "cycles_per_solve": sum(r.cycles for r in treps) / args.steps, "final_fp64_defect": treps[-1].final_res,
             "final_du": treps[-1].final_du, "accuracy": reference_error(E, fx, tu, treps[-1].adm[:2]),
             "max_abs_u_minus_gpu_fp64_fixed_point": pinned_max_diff(E, tu, u_fix)}
    E.set_smoother_blocks(16)
    E.set_inner_sweeps(P.nu1, P.nu2)
    out = {"value": args.steps / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / args.steps,
           "cycles_per_solve": sum(r.cycles for r in reps) / args.steps, "final_fp64_defect": reps[-1].final_res,
           "final_du": reps[-1].final_du, "accuracy": ref,
           "max_abs_u_minus_gpu_fp64_fixed_point": pinned_max_diff(E, u, u_fix),
           "kernels_per_cycle": E.kernels_per_cycle, "tuned_alone": tuned,
           "dtype": "FP32 inner V-cycle (smoothing, Robin, transfers, coarse solve) on a correction; "
                    "FP64 defect, singular terms, update and norm"}
    E.set_precision(False)
    return out


def run_concurrent(E_ref, P, fx, plain_value, n: int = 16):
    """n copies of the workload solved at once (solve_many), mixed precision,
    inner sweep schedule chosen by the autotuner at this concurrency, every
    copy under the timed stop and checked against the reference's fixed
    point."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi, autotune
    choice = autotune.tune(P, concurrency=n)
    sol = [og.Elliptic(P) for _ in range(n)]
    try:
        for E in sol:
            E.set_precision(True)
            choice.apply(E)
        for E in sol:
            E.reset()
        og.solve_many(sol, stop=_abi.STOP_ERROR, max_cycles=300, du_tol=DU_TOL)           # warm-up
        best = None
        for _ in range(3):
            for E in sol:
                E.reset()
            t = time.perf_counter()
            reps = og.solve_many(sol, stop=_abi.STOP_ERROR, max_cycles=300, du_tol=DU_TOL)
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        errs = [reference_error(E, fx) for E in sol]
        value = n / best
        return {"workload": f"{n} copies of {WORKLOAD_NAME} at once (solve_many), mixed precision",
                "concurrent_solves": n, "value": value, "unit": UNIT,
                "inner_sweeps": [choice.nu1, choice.nu2], "smoother_blocks": choice.blocks,
                "autotune_table": choice.table,
                "cycles_per_solve": reps[0].cycles, "final_fp64_defect": max(r.final_res for r in reps),
                "final_du": max(r.final_du for r in reps),
                "max_abs_u_minus_reference": max(e["max_abs_u_minus_reference"] for e in errs) if fx else None,
                "max_abs_adm_minus_reference": max(abs(a) for e in errs for a in e["adm_minus_reference"]) if fx
                else None,
                "vs_plain_fp64": value / plain_value,
                "timing": "host wall clock around solve_many (best of 3), inputs resident in HBM"}
    finally:
        for E in sol:
            E.close()


CONFIG3_ARGS = WORKLOAD_ARGS.replace("-N 65", "-N 129").replace("-O 4", "-O 8").replace("-s 1e-11", "-s 1e-10")


def run_config3():
    """The same binary at 8th order on boxes of 129^3 points: plain FP64 and
    mixed precision, each solved from u = 0 under the timed stop (residual
    <= 1e-10, change of u <= DU_TOL), against the reference's fixed point."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    P = og.parse_olliptic_args(CONFIG3_ARGS.split())
    fx = load_fixture("config3")
    E = og.Elliptic(P)
    try:
        out = {"workload": "binary O8 N129 l9 L1000, tol 1e-10", "boxes": len(E.boxes),
               "points": sum(b.n[0] * b.n[1] * b.n[2] for b in E.boxes)}
        for mixed, key in ((False, "plain_fp64"), (True, "mixed")):
            E.set_precision(mixed)
            best = None
            for _ in range(2):
                E.reset()
                rep = E.Solve(stop=_abi.STOP_ERROR, max_cycles=300, tol=1e-10, du_tol=DU_TOL)
                best = E.last_device_ms if best is None else min(best, E.last_device_ms)
            out[key] = {"solves_per_s": 1000.0 / best, "ms_per_solve": best, "cycles": rep.cycles,
                        "final_res": rep.final_res, "final_du": rep.final_du,
                        "accuracy": reference_error(E, fx, None, rep.adm[:2])}
        E.set_precision(False)
        return out
    finally:
        E.close()


def run_convergence():
    """The reference's self-convergence study (utils/run_conv.sh): one
    spinning puncture at N = 25, 49, 97 (4th order, 4 levels, L = 100),
    solved on the GPU in FP64 and in mixed precision to 1e-11, u read on the
    reference's u.X points; the order p of |u_h - u_h/2| ~ h^p away from the
    puncture beside the order of the reference's own runs (the committed
    fixture made by its Olliptic.x)."""
    import numpy as np
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "convergence",
                        "o4_spin_l4.npz")
    g = np.load(path)
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from tests.golden.make_convergence_golden import orders
    args = g["args"].item().decode()
    x = g["x_25"]
    pts = np.stack([x, np.zeros_like(x), np.zeros_like(x)], axis=1)
    out = {"workload": "run_conv.sh study: " + args + ", N = 25/49/97",
           "reference": {"p_inf": float(g["p_inf"]), "p_l2": float(g["p_l2"])}}
    for mixed, key in ((False, "plain_fp64"), (True, "mixed")):
        cuts, dev = [], []
        for N in g["resolutions"]:
            with og.Elliptic(og.parse_olliptic_args((args + f" -N {int(N)}").split())) as E:
                E.set_precision(mixed)
                E.Solve(stop=_abi.STOP_TOLERANCE, max_cycles=300, tol=1e-11)
                cuts.append(E.interpolate(pts))
                dev.append(float(np.max(np.abs(cuts[-1] - g[f"u_{int(N)}"]))))
        p_inf, p_l2 = orders(x, *cuts)
        out[key] = {"p_inf": p_inf, "p_l2": p_l2, "max_abs_u_minus_reference_cut": dev}
    return out


def run_approx_start():
    """The benchmark binary solved from the reference's analytic puncture
    approximation (elliptic::ApproximateID, olgpu_approximate_id) instead of
    u = 0, plain FP64 and mixed precision, each under the timed stop; cycles
    and solves/s beside the zero start."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    P = og.parse_olliptic_args(WORKLOAD_ARGS.split())
    out = {"workload": "binary_O4_N65_l9_L1000_tol1e-11, FP64 and mixed, zero and approximate start"}
    with og.Elliptic(P) as E:
        for mixed, key in ((False, "plain_fp64"), (True, "mixed")):
            E.set_precision(mixed)
            row = {}
            for start in ("zero", "approx"):
                best = None
                for _ in range(3):
                    if start == "approx":
                        E.ApproximateID()
                    else:
                        E.reset()
                    rep = E.Solve(stop=_abi.STOP_ERROR, max_cycles=300, tol=P.tol, du_tol=DU_TOL)
                    best = E.last_device_ms if best is None else min(best, E.last_device_ms)
                row[start] = {"cycles": rep.cycles, "final_res": rep.final_res, "ms_per_solve": best,
                              "solves_per_s": 1000.0 / best}
            out[key] = row
    return out


def run_bowen_york():
    """The Bowen-York momentum-constraint test (four unknowns V1, V2, V3,
    lambda) of tests/golden/bowen_york/o4.npz (two punctures with momenta,
    N = 25, 3 levels, O4, Robin with falloff 2): GPU solves/s from zero
    (FP64 cycles with FP64 Anderson mixing as in the headline solve, each
    variable to the problem's residual 1e-10 and a change of at most 1e-11;
    device time, five solves after a warm-up), the largest distance from the
    reference's own fixed point over the fixture's samples, and as the CPU
    baseline the oracle restatement's single-threaded solve of the same case
    under the reference's stop rule."""
    import numpy as np
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi
    path = os.path.join(ROOT, "tests", "golden", "bowen_york", "o4.npz")
    G = np.load(path)
    P = og.parse_olliptic_args(str(G["args"]).split())
    rule = dict(stop=_abi.STOP_ERROR, max_cycles=400, tol=P.tol, du_tol=0.1 * P.tol)
    with og.Elliptic(P) as E:
        E.set_fp64_acceleration(ACCEL)
        E.Solve(**rule)
        ms, cycles = 0.0, 0
        for _ in range(5):
            E.reset()
            rep = E.Solve(**rule)
            ms += E.last_device_ms
            cycles += rep.cycles
        err = 0.0
        for g, b in enumerate(E.boxes):
            idx = G[f"idx_b{g}"]
            nx, ny, nz = b.n
            k, j, i = np.unravel_index(idx, (nz, ny, nx))
            keep = np.ones(len(idx), dtype=bool)
            if b.level < E.mgrid_levels:   # a multigrid grid's ghost layers are not fixed by the system
                keep = (i >= b.buf) & (i < nx - b.buf) & (j >= b.buf) & (j < ny - b.buf) & (k >= b.buf) & (
                    k < nz - b.buf)
            for v in og.BY_VARS:
                got = E.get_field(g, v).ravel()[idx]
                err = max(err, float(np.max(np.abs(got[keep] - G[f"{v}_b{g}"][keep]))))
    from oracle import oracle as oracle_mod
    t = time.perf_counter()
    solved, ocycles = [], []
    for v in range(4):
        o = oracle_mod.Oracle(dict(P.oracle_dict(), equation=oracle_mod.BOWEN_YORK, by_var=v))
        if v == 3:
            o.L.orc_set_divergence_source(o._s, *(s._s for s in solved))
        ocycles.append(o.solve()[0])
        solved.append(o)
    cpu_s = time.perf_counter() - t
    return {"workload": "Bowen-York momentum-constraint test, 2 punctures with momenta, N = 25, 3 levels, O4, "
                        "Robin falloff 2 (tests/golden/bowen_york/o4.npz)",
            "value": 5 / (ms / 1000.0), "unit": UNIT, "ms_per_solve": ms / 5, "cycles_per_solve": cycles / 5,
            "max_abs_minus_reference_fixed_point": err,
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"one solve by the oracle restatement under the reference's stop rule "
                                       f"({sum(ocycles)} V-cycles over the four variables) in {cpu_s:.1f} s"},
            "iteration": f"each variable: FP64 V-cycles with FP64 Anderson mixing of depth {ACCEL}",
            "timing": "device time of olgpu_solve (CUDA events), five solves from zero after a warm-up"}


def fp32_smoother_roofline(peak: float, peak_kind: str):
    """The mixed cycle's dominant kernel, the cluster-resident FP32 smoother
    (k_smooth32_cluster), on the finest level of the benchmark binary, 20
    algorithmic bytes per interior point and sweep (read S, A, 1/(c+u) and e,
    write e): 12 sweeps of CONCURRENT_SOLVES solves at once, each on its own
    stream, timed with CUDA events from the common start to the last end
    (olgpu_time_smoother_many) -- the rate when many solves share the GPU,
    as in the served and batched forms; beside it one solve alone
    (olgpu_time_smoother), whose two 16-block clusters hold 32 SMs."""
    import ollipticid_gb300 as og
    P = og.parse_olliptic_args(WORKLOAD_ARGS.split())
    sols = [og.Elliptic(P) for _ in range(CONCURRENT_SOLVES)]
    try:
        for E in sols:
            E.set_smoother_blocks(16)
            E.set_inner_sweeps(4, 6)
            E.set_precision(True)
        E = sols[0]
        top = E.levels - 1
        pts = E.interior_points(top)
        boxes = sum(1 for b in E.boxes if b.level == top)
        E.time_smoother(top, 3)                               # warm
        sweeps = 12
        ms, nl = E.time_smoother(top, sweeps)
        og.time_smoother_many(sols, top, 3)                   # warm
        ms_all = og.time_smoother_many(sols, top, sweeps)
    finally:
        for x in sols:
            x.close()
    achieved = 20.0 * pts * sweeps / (ms / 1e3) / 1e9
    achieved_all = 20.0 * pts * sweeps * len(sols) / (ms_all / 1e3) / 1e9
    sms = 16 * boxes
    return {"bound": "hbm", "kernel": f"k_smooth32_cluster<{P.order},0>: {sweeps} sweeps of the finest level "
                                      f"({pts} interior points, {boxes} boxes, one 16-block cluster each)",
            "achieved": achieved_all, "peak": peak, "unit": "GB/s", "frac": achieved_all / peak,
            "peak_kind": peak_kind, "concurrent_solves": len(sols), "ms": ms_all,
            "how": f"the level's sweeps of {len(sols)} solves at once, each on its own stream "
                   f"(olgpu_time_smoother_many), CUDA events from the common start to the last end",
            "one_solve": {"achieved": achieved, "frac": achieved / peak, "sms": sms, "ms": ms, "launches": nl},
            "note": "the level stays in shared and L2 memory through the sweeps; alone, one solve's clusters "
                    "hold 16 SMs per box"}


def batched_fixture_error(B, i, inst, fx):
    """max |u - u_oracle| of batch member i (workload instance inst) at the
    fixture's sample points, and its ADM masses' largest difference."""
    import numpy as np
    worst = 0.0
    boxes = B.boxes(i)
    u = B.all_u(i)
    for g, bi in enumerate(boxes):
        idx = fx[f"inst{inst}_idx_b{g}"].astype(np.int64)
        want = fx[f"inst{inst}_fixed_u_b{g}"]
        x = u[g].ravel()
        if bi.level < B.mgrid_levels(i):
            nx, ny, nz = bi.nx, bi.ny, bi.nz
            k, rem = np.divmod(idx, nx * ny)
            j, ii = np.divmod(rem, nx)
            w = bi.buf
            keep = (ii >= w) & (ii < nx - w) & (j >= w) & (j < ny - w) & (k >= w) & (k < nz - w)
            idx, want = idx[keep], want[keep]
        worst = max(worst, float(np.max(np.abs(x[idx] - want))))
    adm = max(abs(a - b) for a, b in zip(B.ADM_mass(i), fx[f"inst{inst}_adm"]))
    return worst, adm


def run_batched(args, tuned=None, count: int = 256, chunk: int = 64, plain_rate=None):
    """The batched workload: all `count` seeded binaries (N in {33, 49, 65,
    97}, 6-10 levels, 4th order), mixed precision, residual <= 1e-10 and
    change of u <= DU_TOL, solved as batches of `chunk` (olgpu_batch: unions
    of solves share one launch per FASN step).  Host wall clock around each
    batch's solve, hierarchies resident; each result with an oracle fixture
    (tests/golden/configs/batched.npz) is checked against it.  For
    comparison, the first 16 also through solve_many (one stream and its own
    launches per solve)."""
    import numpy as np
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi, workloads
    probs = workloads.batched_binaries(256)[:count]
    path = os.path.join(GOLDEN, "batched.npz")
    fx = np.load(path) if os.path.exists(path) else None
    with_fx = set(int(i) for i in fx["instances"]) if fx is not None else set()
    rule = dict(stop=_abi.STOP_ERROR, max_cycles=300, tol=1e-10, du_tol=DU_TOL)
    inner = (tuned.nu1, tuned.nu2) if tuned is not None else None
    blocks = tuned.blocks if tuned is not None else -1
    solve_s, cycles, errs, unions, kpc, build_s = 0.0, [], [], 0, 0, 0.0
    for g0 in range(0, count, chunk):
        t = time.perf_counter()
        B = og.Batch(probs[g0:g0 + chunk], mixed=True, inner_sweeps=inner, blocks=blocks)
        build_s += time.perf_counter() - t
        try:
            B.solve(**rule)                               # warm-up
            B.reset()
            reps = B.solve(**rule)
            solve_s += B.last_ms / 1000.0
            cycles += [r.cycles for r in reps]
            unions += B.unions
            kpc += B.kernels_per_cycle
            for q in range(len(reps)):
                if g0 + q in with_fx:
                    errs.append(batched_fixture_error(B, q, g0 + q, fx))
        finally:
            B.close()
    # the first 16 as separate solves on streams (olgpu_solve_many), same rule
    sol = [og.Elliptic(p) for p in probs[:16]]
    try:
        for E in sol:
            if tuned is not None:
                tuned.apply(E)
            E.set_precision(True)
        og.solve_many(sol, **rule)
        for E in sol:
            E.reset()
        t = time.perf_counter()
        og.solve_many(sol, **rule)
        streams = 16 / (time.perf_counter() - t)
    finally:
        for E in sol:
            E.close()
    return {"workload": f"{count} seeded binaries (N in {{33,49,65,97}}, 6-10 levels, O4), mixed precision, "
                        f"residual <= 1e-10 and change of u <= {DU_TOL:g}, batches of {chunk}",
            "value": count / solve_s, "unit": UNIT, "solve_s": solve_s, "build_s": build_s,
            "unions": unions, "kernels_per_cycle_all_unions": kpc,
            "inner_sweeps": None if tuned is None else [tuned.nu1, tuned.nu2, tuned.blocks],
            "autotune_table": None if tuned is None else tuned.table,
            "cycles_mean": sum(cycles) / len(cycles), "cycles_max": max(cycles),
            "oracle_checked_instances": len(errs),
            "max_abs_u_minus_oracle": max((e for e, _ in errs), default=None),
            "max_abs_adm_minus_oracle": max((a for _, a in errs), default=None),
            "first16_as_separate_streams": streams,
            "plain_fp64_same_binaries_solves_per_s": plain_rate,
            "vs_plain_fp64": (count / solve_s) / plain_rate if plain_rate else None,
            "timing": "host wall clock around olgpu_batch_solve (u = 0 to the stop; hierarchies resident)"}


def run_served(rates=(4.0, 16.0, 64.0), count: int = 24, inner_sweeps=None, native: bool = False):
    """Poisson request streams (NumBH 1-4, N 33-129, orders 2-8, 6-10
    levels, 10% scalar field) served with memory admission, by the Python
    loop (serve.Server) or by the library's C++ server (native)."""
    from ollipticid_gb300 import workloads
    from ollipticid_gb300.serve import NativeServer, Server
    out = []
    for rate in rates:
        if native:
            with NativeServer(mem_budget=120 << 30, max_active=16, inner_sweeps=inner_sweeps) as S:
                rep = S.run(workloads.served_stream(count, rate))
        else:
            rep = Server(mem_budget=120 << 30, max_active=16, inner_sweeps=inner_sweeps).run(
                workloads.served_stream(count, rate))
        out.append({"rate_hz": rate, "requests": count, "inner_sweeps": inner_sweeps,
                    "server": "C++ (olgpu_server_*)" if native else "Python loop",
                    **{k: rep[k] for k in ("throughput_solves_per_s", "latency_p50_s", "latency_p99_s",
                                           "latency_max_s", "cycles_mean", "peak_concurrent_solves", "makespan_s")}})
    return out


def served_binary_error(u, P, inst, fx):
    """max |u - u_oracle| of a served result of workload instance inst at the
    fixture's sample points (multigrid coarse ghosts excluded)."""
    import ctypes as C
    import numpy as np
    from ollipticid_gb300 import _abi
    lib = _abi.load()
    cp = P.to_c()
    out = (_abi.BoxInfo * 256)()
    nb, mg = C.c_int(), C.c_int()
    lib.olgpu_plan_boxes(C.byref(cp), out, 256, C.byref(nb), None, C.byref(mg))
    worst = 0.0
    for g in range(nb.value):
        bi = out[g]
        idx = fx[f"inst{inst}_idx_b{g}"].astype(np.int64)
        want = fx[f"inst{inst}_fixed_u_b{g}"]
        if bi.level < mg.value:
            k, rem = np.divmod(idx, bi.nx * bi.ny)
            j, i = np.divmod(rem, bi.nx)
            w = bi.buf
            keep = (i >= w) & (i < bi.nx - w) & (j >= w) & (j < bi.ny - w) & (k >= w) & (k < bi.nz - w)
            idx, want = idx[keep], want[keep]
        worst = max(worst, float(np.max(np.abs(u[g].ravel()[idx] - want))))
    return worst


def plain_binaries_rate(sample: int = 8):
    """The plain FP64 solver (FP64 cycles with FP64 mixing, the timed stop)
    on the first `sample` binaries of the batched workload, one at a time:
    solves/s from device time, after one untimed solve each."""
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi, workloads
    ms = []
    for P in workloads.batched_binaries(sample):
        with og.Elliptic(P) as E:
            E.set_fp64_acceleration(ACCEL)
            E.Solve(stop=_abi.STOP_ERROR, max_cycles=300, tol=1e-10, du_tol=DU_TOL)
            E.reset()
            E.Solve(stop=_abi.STOP_ERROR, max_cycles=300, tol=1e-10, du_tol=DU_TOL)
            ms.append(E.last_device_ms)
    return len(ms) / (sum(ms) / 1000.0)


def run_served_binaries(count: int = 256, rate: float = 400.0, inner_sweeps=None, plain_rate=None,
                        plain_sample: int = 8):
    """The batched workload's binaries as a Poisson request stream at a
    saturating rate through the library's C++ server (continuous batching:
    requests admitted as slots and memory free up, each on its own stream,
    their cycles overlapping on the GPU), mixed precision, residual <= 1e-10
    and change of u <= DU_TOL.  Throughput, p50/p99 latency, the results of
    the instances with oracle fixtures against them, and the plain FP64
    solver's rate on the same binaries (a sample solved one at a time)."""
    import numpy as np
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi, workloads
    from ollipticid_gb300.serve import NativeServer
    path = os.path.join(GOLDEN, "batched.npz")
    fx = np.load(path) if os.path.exists(path) else None
    with_fx = set(int(i) for i in fx["instances"]) if fx is not None else set()
    stream = workloads.served_binaries(count, rate)
    with NativeServer(mem_budget=200 << 30, max_active=SERVED_SLOTS, builders=8, inner_sweeps=inner_sweeps,
                      stop=_abi.STOP_ERROR, tol=1e-10, du_tol=DU_TOL, keep_u=True, keep_only=with_fx,
                      max_cycles=300) as S:
        rep = S.run(stream)
    errs = [served_binary_error(r.u, stream[i][1], i, fx) for i, r in enumerate(rep["results"])
            if i in with_fx and r.u is not None]
    if plain_rate is None:
        plain_rate = plain_binaries_rate(plain_sample)
    statuses = [r.status for r in rep["results"]]
    return {"workload": f"{count} seeded binaries of the batched workload as a Poisson stream at {rate:g} "
                        f"requests/s, C++ server (olgpu_server_*), mixed precision, residual <= 1e-10 and change "
                        f"of u <= {DU_TOL:g}",
            **{k: rep[k] for k in ("throughput_solves_per_s", "latency_p50_s", "latency_p99_s", "latency_max_s",
                                   "cycles_mean", "peak_concurrent_solves", "makespan_s")},
            "failed": sum(1 for x in statuses if x != 0),
            "oracle_checked_results": len(errs), "max_abs_u_minus_oracle": max(errs) if errs else None,
            "plain_fp64_same_binaries_solves_per_s": plain_rate,
            "plain_fp64_sample": f"the first {plain_sample} binaries solved alone by the plain FP64 solver, "
                                 f"device time",
            "vs_plain_fp64": rep["throughput_solves_per_s"] / plain_rate}


def run_served_binaries_batching(count: int = 256, rate: float = 400.0, inner_sweeps=None, plain_rate=None,
                                 batch_max: int = 16, batch_window: float = 0.02, max_active: int = 64):
    """The same Poisson stream of the batched workload's binaries through the
    C++ server with batching: requests admitted together (up to batch_max,
    after at most batch_window seconds) are solved as one batch
    (olgpu_batch_*) on a builder thread, several batches at once.  The
    results carry no u (a batch's hierarchies are not handed out), so each
    result with an oracle fixture is checked by its ADM masses, and its
    cycles are reported."""
    import numpy as np
    from ollipticid_gb300 import _abi, workloads
    from ollipticid_gb300.serve import NativeServer
    path = os.path.join(GOLDEN, "batched.npz")
    fx = np.load(path) if os.path.exists(path) else None
    stream = workloads.served_binaries(count, rate)
    with NativeServer(mem_budget=200 << 30, max_active=max_active, builders=8, inner_sweeps=inner_sweeps,
                      stop=_abi.STOP_ERROR, tol=1e-10, du_tol=DU_TOL, max_cycles=300, batch_max=batch_max,
                      batch_window=batch_window) as S:
        rep = S.run(stream)
    adm_err = []
    if fx is not None:
        for inst in (int(i) for i in fx["instances"]):
            r = rep["results"][inst]
            want = fx[f"inst{inst}_adm"]
            adm_err.append(max(abs(a - b) for a, b in zip(r.adm, want)))
    statuses = [r.status for r in rep["results"]]
    out = {"workload": f"{count} seeded binaries of the batched workload as a Poisson stream at {rate:g} "
                       f"requests/s, C++ server batching up to {batch_max} admitted requests (window "
                       f"{batch_window:g} s, {max_active} slots), mixed precision, residual <= 1e-10 and change of "
                       f"u <= {DU_TOL:g}",
           **{k: rep[k] for k in ("throughput_solves_per_s", "latency_p50_s", "latency_p99_s", "latency_max_s",
                                  "cycles_mean", "peak_concurrent_solves", "makespan_s")},
           "failed": sum(1 for x in statuses if x != 0),
           "oracle_checked_results": len(adm_err), "max_abs_adm_minus_oracle": max(adm_err) if adm_err else None,
           "inner_sweeps": list(inner_sweeps) if inner_sweeps else None}
    if plain_rate:
        out["plain_fp64_same_binaries_solves_per_s"] = plain_rate
        out["vs_plain_fp64"] = rep["throughput_solves_per_s"] / plain_rate
    return out


def slowest_rank_ms(ms: float, world: int, device) -> float:
    """The timed region's length: the maximum over ranks (replicas run the
    same work; the job is done when the slowest one is)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def replica_throughput(steps: int, slowest_ms: float, world: int) -> float:
    """Whole-job solves/s: every rank solves `steps` problems of its own."""
    return world * steps / (slowest_ms / 1000.0)


def run_gpu(args, rank: int, world: int, local: int):
    import numpy as np
    import torch
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi

    # the single-core CPU solve runs in a spawned process beside the GPU work
    cpu_job = CpuBaseline() if rank == 0 and world == 1 and not args.no_cpu_baseline else None
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    P = og.parse_olliptic_args(WORKLOAD_ARGS.split())
    E = og.Elliptic(P, device=local)
    nboxes = len(E.boxes)
    total_pts = sum(b.n[0] * b.n[1] * b.n[2] for b in E.boxes)
    fx = load_fixture("config2")
    # the plain FP64 solver: FP64 FAS V-cycles with FP64 Anderson mixing of
    # depth 4 (the same fixed point, fewer cycles than the reference's
    # iteration, which is timed below beside it)
    E.set_fp64_acceleration(ACCEL)

    timed_solves(E, args.warmup, dev, P.tol)
    # ---- timed region: K solves (device time from CUDA events on the solver's stream)
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    t_wall0 = time.perf_counter()
    dev_ms, reps = timed_solves(E, args.steps, dev, P.tol)
    cycles = sum(r.cycles for r in reps)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t_wall0
    dev_ms = slowest_rank_ms(dev_ms, world, dev)
    clk = clocks.stop()
    ms_per_step = dev_ms / args.steps
    value = replica_throughput(args.steps, dev_ms, world)
    launches = E.kernels_per_cycle * cycles
    u_stop = [E.get_field(g) for g in range(nboxes)]
    accuracy = reference_error(E, fx, u_stop, reps[-1].adm[:2]) or {"reference": "fixture missing"}
    # the reference's iteration (no mixing) under the same stop, for comparison
    E.set_fp64_acceleration(0)
    timed_solves(E, 1, dev, P.tol)
    ums, ureps = timed_solves(E, args.steps, dev, P.tol)
    unaccelerated = {"value": args.steps / (ums / 1000.0), "unit": UNIT, "ms_per_step": ums / args.steps,
                     "cycles_per_solve": sum(r.cycles for r in ureps) / args.steps,
                     "accuracy": reference_error(E, fx, None, ureps[-1].adm[:2]),
                     "iteration": "FP64 FAS V-cycles without mixing (the reference's iteration, multicolour)"}
    E.set_fp64_acceleration(ACCEL)

    # ---- end to end through the C ABI with host buffers (pinned host memory)
    def pinned_like(x):
        return torch.empty(x.shape, dtype=torch.float64, pin_memory=True).numpy()

    hb, hc, hu0, hu = [], [], [], []
    for g in range(nboxes):
        b_, c_ = E.get_field(g, "b"), E.get_field(g, "c")
        for lst, src in ((hb, b_), (hc, c_), (hu0, None), (hu, None)):
            buf = pinned_like(b_)
            buf[...] = 0.0 if src is None else src
            lst.append(buf)
    e2e_steps = max(1, min(args.steps, 5))

    def e2e_step():
        for g in range(nboxes):
            E.set_field(g, "b", hb[g])
            E.set_field(g, "c", hc[g])
        E.reset()
        for g in range(nboxes):
            E.set_field(g, "u", hu0[g])
        E.Solve(stop=_abi.STOP_ERROR, max_cycles=300, tol=P.tol, du_tol=DU_TOL)
        for g in range(nboxes):
            E.get_field(g, "u", out=hu[g])

    e2e_step()                    # untimed: the first transfers of the pinned buffers
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    # the hierarchy's set-up, outside the steps above (a resident solver
    # reuses it): host plan, device arena from the pool, tables, coefficients
    # and the captured cycle, timed on the host for a fresh hierarchy
    t1 = time.perf_counter()
    E_setup = og.Elliptic(P, device=local)
    E_setup.set_fp64_acceleration(ACCEL)
    torch.cuda.synchronize(dev)
    setup_s = time.perf_counter() - t1
    E_setup.close()
    e2e = {"value": world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 3 * 8 * total_pts,
           "d2h_bytes_per_step": 8 * total_pts, "host_buffers": "pinned",
           "setup_ms": 1000.0 * setup_s, "value_with_setup": world / (e2e_s + setup_s),
           "setup_note": "each step reuses a resident hierarchy; setup_ms is one fresh hierarchy's set-up "
                         "(plan, device memory, tables, coefficients, captured cycle), value_with_setup counts "
                         "it in every step"}

    # ---- the GPU's own FP64 fixed point (every point, beside the reference's samples)
    u_fix = fixed_point(E)
    accuracy["max_abs_u_minus_gpu_fp64_fixed_point"] = pinned_max_diff(E, u_stop, u_fix)
    accuracy["gpu_fp64_fixed_point_vs_reference"] = reference_error(E, fx, u_fix)

    # ---- the same workload with the mixed-precision cycle
    mixed = run_mixed(E, P, args, dev, u_fix, fx)

    concurrent = batched = served = served_binaries = served_binaries_batching = None
    config3 = convergence = approx_start = bowen_york = None
    if rank == 0 and world == 1 and not args.no_extra:
        from ollipticid_gb300 import autotune
        concurrent = run_concurrent(E, P, fx, value / world)
        plain_bin = plain_binaries_rate(8)
        # the batched workload's schedule and smoother layout, tuned on its first 64 binaries
        from ollipticid_gb300 import workloads
        tuned_batch = autotune.tune_batch(workloads.batched_binaries(256)[:64], du_tol=DU_TOL)
        batched = run_batched(args, tuned=tuned_batch, plain_rate=plain_bin)
        config3 = run_config3()
        convergence = run_convergence()
        approx_start = run_approx_start()
        bowen_york = run_bowen_york()
        served = run_served(inner_sweeps=tuple(concurrent["inner_sweeps"]))   # layout follows the load
        served += run_served(inner_sweeps=tuple(concurrent["inner_sweeps"]), native=True)
        served_binaries = run_served_binaries(
            inner_sweeps=(tuned_batch.nu1, tuned_batch.nu2, tuned_batch.blocks), plain_rate=plain_bin)
        served_binaries_batching = run_served_binaries_batching(
            inner_sweeps=(tuned_batch.nu1, tuned_batch.nu2, tuned_batch.blocks), plain_rate=plain_bin)

    # ---- roofline of the dominant kernel: one colour pass of the FP64
    # multicolour smoother (k_smooth_color) on the finest level, timed with
    # CUDA events on the solver's stream over 10 sweeps of that level
    peak, peak_kind = _peaks()
    top = E.levels - 1
    colours = P.order // 2 + 1
    E.time_smoother(top, 2)                               # warm
    ms, nl = E.time_smoother(top, 10)
    pts = E.interior_points(top)
    launch_s = ms / 1000.0 / nl
    bytes_per_launch = SMOOTH_BYTES_PER_POINT * pts / colours
    achieved = bytes_per_launch / launch_s / 1e9
    # FMA issue rates of this GPU (the stencils' instruction roofline)
    fma = {"fp64_tflops": og.fma_peak(True), "fp32_tflops": og.fma_peak(False),
           "how": "olgpu_fma_peak: 8 blocks of 256 threads per SM, 8 independent FMA chains a thread, CUDA events, "
                  "best of 3 after a warm-up launch; 2 flops per FMA"}
    fp64_rate = SMOOTH_FP64_INST_PER_POINT * (pts / colours) / launch_s / 1e9   # G FP64 instructions/s
    fp64_peak = fma["fp64_tflops"] * 1e3 / 2.0                                   # G FP64 FMA/s, measured
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind, "traffic": SMOOTH_TRAFFIC_PER_LAUNCH,
            "kernel": f"k_smooth_color<{P.order},0>: one colour pass of the finest level "
                      f"({pts} interior points, {colours} colours)",
            "algorithmic_bytes_per_launch": bytes_per_launch, "launch_us": launch_s * 1e6, "launches_timed": nl,
            "fp64_pipe_active_pct": SMOOTH_FP64_PIPE_PCT,
            "fp64_issue": {"instructions_per_point": SMOOTH_FP64_INST_PER_POINT, "achieved_ginst_s": fp64_rate,
                           "peak_ginst_s": fp64_peak, "frac": fp64_rate / fp64_peak,
                           "peak_kind": "measured (olgpu_fma_peak, this run)"},
            "note": "FP64-issue bound on GB300 (fp64_fma_peak_tflops, measured in this run): the HBM fraction is "
                    "low by design; traffic and FP64 pipe occupancy are from one ncu capture of this launch (ncu "
                    "flushes L2 first, so traffic is the level's fields read once; in the timed sweeps they stay "
                    "in L2)"}

    roof32 = fp32_smoother_roofline(peak, peak_kind) if rank == 0 and world == 1 and not args.no_extra else None
    roof["fp64_fma_peak_tflops"] = fma["fp64_tflops"]

    cpu = cpu_job.result() if cpu_job is not None else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(),
            "solve": {"precision": "plain FP64",
                      "iteration": f"FP64 FAS V-cycles with FP64 Anderson mixing of depth {ACCEL}",
                      "cycles_per_solve": cycles / args.steps,
                      "final_res": reps[-1].final_res, "final_du": reps[-1].final_du,
                      "adm": [reps[-1].adm[0], reps[-1].adm[1]], "wall_s": wall},
            "accuracy": accuracy, "plain_fp64_unaccelerated": unaccelerated,
            "mixed": mixed, "concurrent": concurrent, "batched": batched, "served": served,
            "served_binaries": served_binaries, "served_binaries_batching": served_binaries_batching,
            "config3": config3,
            "convergence": convergence, "approx_start": approx_start, "bowen_york": bowen_york,
            "roofline": roof, "roofline_fp32_smoother": roof32, "fma_peaks": fma, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    E.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and served sub-results")
    ap.add_argument("--profile-cycle", action="store_true",
                    help="run two V-cycles of the workload and exit (for the ncu launch list)")
    ap.add_argument("--mixed", action="store_true", help="with --profile-cycle: the mixed-precision cycle")
    ap.add_argument("--inner", default=None,
                    help="with --profile-cycle --mixed: inner schedule nu1,nu2,blocks (e.g. 4,6,16)")
    ap.add_argument("--profile-batch", type=int, default=0, metavar="N",
                    help="run two cycles of one batch of the first N seeded binaries of the batched workload "
                         "(mixed precision, schedule 4,6,16) and exit (for the ncu launch list)")
    args = ap.parse_args()
    if args.profile_batch:
        import ollipticid_gb300 as og
        from ollipticid_gb300 import _abi, workloads
        with og.Batch(workloads.batched_binaries(256)[:args.profile_batch], mixed=True, inner_sweeps=(4, 6),
                      blocks=16) as B:
            reps = B.solve(stop=_abi.STOP_ERROR, max_cycles=2, tol=1e-10, du_tol=DU_TOL)
            print(json.dumps({"profile_batch": args.profile_batch, "cycles": [r.cycles for r in reps],
                              "unions": B.unions, "kernels_per_cycle": B.kernels_per_cycle}))
        return
    if args.profile_cycle:
        import ollipticid_gb300 as og
        E = og.Elliptic(og.parse_olliptic_args(WORKLOAD_ARGS.split()))
        if args.inner:
            nu1, nu2, blocks = (int(v) for v in args.inner.split(","))
            E.set_inner_sweeps(nu1, nu2)
            E.set_smoother_blocks(blocks)
        E.set_precision(args.mixed)
        if not args.mixed:
            E.set_fp64_acceleration(ACCEL)   # the timed plain FP64 cycle
        r = [E.FASN() for _ in range(2)]
        print(json.dumps({"profile_cycles": 2, "res": r, "kernels_per_cycle": E.kernels_per_cycle}))
        E.close()
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    run_gpu(args, rank, world, local)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
