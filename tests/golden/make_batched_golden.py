"""Regenerates tests/golden/configs/batched.npz: the fixed points of the
seeded binaries of the batched workload that a CPU reaches in minutes.

The batched workload is ollipticid_gb300.workloads.batched_binaries (256
seeded equal-order binaries, N from {33, 49, 65, 97}, 6-10 levels); among its
first sixteen, the N = 33 instances are solved here by the oracle to their
fixed point (the reference's stop rule, then V-cycles until max |du| <=
1e-14), after its first two cycles were checked against the UNMODIFIED
reference's (oracle/_ref/ref_harness, the instance written as an Olliptic.x
command line) on every point, bit for bit.  Stored per instance: its index in
the workload, the sample indices of each box (the same sampling as
make_config_golden.py) and u there, and the ADM masses.

Needs the reference sources; run in the build container only:

    make -C oracle ref && python tests/golden/make_batched_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden.make_config_golden import HARNESS, WORK, sample_index  # noqa: E402

FIRST = 16
FIXED_TOL, FIXED_MAX = 1e-14, 150


def command_line(P):
    """The problem as an Olliptic.x command line (shortest round-trip floats)."""
    a = [f"-eq {P.equation} -B {P.boundary} -NumBH {P.numbh}"]
    for i in range(P.numbh):
        for name, flag in (("mp", "bhmp"), ("x", "bhx"), ("y", "bhy"), ("z", "bhz"), ("px", "bhpx"),
                           ("py", "bhpy"), ("pz", "bhpz"), ("sx", "bhsx"), ("sy", "bhsy"), ("sz", "bhsz")):
            a.append(f"-{flag}{i + 1} {repr(float(getattr(P, name)[i]))}")
    a.append(f"-L {repr(float(P.L))} -N {P.n} -O {P.order} -l {P.levels} -s {repr(float(P.tol))} "
             f"-nu1 {P.nu1} -nu2 {P.nu2}")
    return " ".join(a)


def main():
    import ollipticid_gb300 as og
    from ollipticid_gb300 import workloads
    from oracle import oracle as O
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: make -C oracle ref")
    probs = workloads.batched_binaries(256)[:FIRST]
    rec = {}
    chosen = [i for i, P in enumerate(probs) if P.n == 33]
    for i in chosen:
        P = probs[i]
        args = command_line(P)
        assert og.parse_olliptic_args(args.split()) == P, "command line does not round-trip"
        out = os.path.join(WORK, f"batched{i}_cyc2")
        if not os.path.exists(os.path.join(out, "meta.txt")):
            os.makedirs(WORK, exist_ok=True)
            subprocess.run([HARNESS, "cycles:2", out, "--"] + args.split() + ["-o", out + "_run"], check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd=WORK)
        orc = O.Oracle(P.oracle_dict())
        for _ in range(2):
            orc.vcycle()
        for g in range(orc.nboxes):
            ref = np.fromfile(os.path.join(out, f"b{g}_u.f64"))
            if not np.array_equal(orc.field(g).ravel(), ref):
                raise SystemExit(f"instance {i}: oracle differs from the reference after two cycles on box {g}")
        orc.solve()
        prev = orc.all_u()
        d = np.inf
        for _ in range(FIXED_MAX):
            orc.vcycle()
            cur = orc.all_u()
            d = max(float(np.max(np.abs(a - b))) for a, b in zip(cur, prev))
            prev = cur
            if d <= FIXED_TOL:
                break
        pts = [(P.x[j], P.y[j], P.z[j]) for j in range(P.numbh)]
        rec[f"inst{i}_args"] = np.array(args)
        rec[f"inst{i}_adm"] = np.array(orc.adm())
        rec[f"inst{i}_last_du"] = np.array(d)
        for g, b in enumerate(orc.boxes):
            idx = sample_index(b.level, (b.nx, b.ny, b.nz), (b.xi, b.yi, b.zi), (b.dx, b.dy, b.dz), pts, 3000 + g)
            rec[f"inst{i}_idx_b{g}"] = idx
            rec[f"inst{i}_fixed_u_b{g}"] = prev[g].ravel()[idx]
        print("instance", i, "boxes", orc.nboxes, "last |du|", d, flush=True)
    rec["instances"] = np.array(chosen)
    np.savez_compressed(os.path.join(HERE, "configs", "batched.npz"), **rec)


if __name__ == "__main__":
    main()
