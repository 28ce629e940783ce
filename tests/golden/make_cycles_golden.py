"""Regenerates tests/golden/wcycle/*.npz and tests/golden/vcycle/*.npz: runs
of the REFERENCE's own Olliptic.x (oracle/_ref, `make -C oracle ref`) with
`-m Wcycle` (elliptic::Wcycle, src/elliptic.cc:1348-1380: every level of
FASN repeats until its own norm meets the tolerance) and with its default
V-cycles.

    make -C oracle ref && python tests/golden/make_cycles_golden.py

Each fixture holds the printed u.X, u.Y, u.Z (first column as text, values as
floats, as tests/golden/output), every Loo.gp line (the cycle number and the
norm of each Print_Pre_Cycle call) and the cycle tables of stdout0.out (the
text after the banner).
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from tests.golden.make_output_golden import parse_data_file  # noqa: E402

REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")
WCYCLE_CASES = {
    "o2_single": "-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpx1 0.1 -L 40 -N 25 -O 2 -l 4 -s 1e-10 -Dp 0.5 -p1d no",
    "o4_binary": ("-eq Punctures -B Robin -NumBH 2 -bhmp1 0.487209 -bhy1 3 -bhpx1 -0.09 -bhmp2 0.487209 -bhy2 -3 "
                  "-bhpx2 0.09 -L 40 -N 25 -O 4 -l 3 -nu2 5 -s 1e-10 -Dp 0.5 -p1d no"),
}
VCYCLE_CASES = {"o2_single": WCYCLE_CASES["o2_single"]}
BANNER_END = "  Init Multigrid iteration\n"


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    runs = [("wcycle", n, a, ["-m", "Wcycle"]) for n, a in WCYCLE_CASES.items()]
    runs += [("vcycle", n, a, []) for n, a in VCYCLE_CASES.items()]
    for kind, name, args, extra in runs:
        os.makedirs(os.path.join(HERE, kind), exist_ok=True)
        run = os.path.join(ROOT, "oracle", "_ref", kind + "_" + name)
        shutil.rmtree(run, ignore_errors=True)
        os.makedirs(run)
        subprocess.run([REF_CLI] + args.split() + extra + ["-o", "Output"], cwd=run, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        out = os.path.join(run, "Output")
        rec = {"args": np.array(args.encode())}
        for f in ("u.X", "u.Y", "u.Z"):
            rec[f + "__text"], rec[f + "__vals"] = parse_data_file(os.path.join(out, f))
        loo = [line.split() for line in open(os.path.join(out, "Loo.gp")) if line.strip()]
        rec["loo_cycle"] = np.array([int(c) for c, _ in loo])
        rec["loo_norm"] = np.array([float(v) for _, v in loo])
        text = open(os.path.join(out, "stdout0.out")).read()
        rec["stdout_cycles"] = np.array(text[text.index(BANNER_END) + len(BANNER_END):].encode())
        np.savez_compressed(os.path.join(HERE, kind, name + ".npz"), **rec)
        print(kind, name, len(loo), "Loo.gp lines", text.count("Cycle:"), "top-level cycles")


if __name__ == "__main__":
    main()
