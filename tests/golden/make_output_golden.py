"""Regenerates tests/golden/output/*.npz: the output files of the REFERENCE's
own command line (Olliptic.x, built from its unmodified sources by the
oracle/Makefile `ref` target) for small puncture runs.

    make -C oracle ref && python tests/golden/make_output_golden.py

Each case runs oracle/_ref/Olliptic.x in oracle/_ref/out_<case>/ with
`-o Output` and records every file it writes there except stdout0.out (the
banner and log, which the GPU command line does not write):
  * <file>__text   the first column(s) of every line as printed (the
                   coordinates, compared as text), b"" for a blank line,
  * <file>__vals   the last numeric column as a float (NaN on blank lines),
  * run_args       the command line recorded in <dir>.run, without argv[0],
  * loo_levels     lines per cycle in Loo.gp (one per level),
  * value_tol      how far another solver's printed u may be from these:
                   1e-9 where the reference's stop rule lands at residual
                   1e-12 (the 2nd-order cases); 1e-5 for the 4th-order case,
                   where the reference stops on its non-monotone residual
                   after 5 cycles at 2e-6 (any other smoother ordering stops
                   elsewhere),
  * mg_tol         the same for the cuts of the multigrid coarse grids, whose
                   u holds the last coarse-grid approximation and so depends
                   on how exactly the coarsest problem was solved (1e-6).
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")

BIN = ("-eq Punctures -B Robin -NumBH 2 -bhmp1 0.487209 -bhy1 3 -bhpx1 -0.09 -bhmp2 0.487209 -bhy2 -3 "
       "-bhpx2 0.09 -L 40 -N 25 -O 2 -l 4 -nu2 5 -s 1e-12")
OUTPUT_CASES = {   # name: (command line, value_tol, mg_tol)
    # interpolated cuts and plane, one spinning puncture, 4th order
    "o4_spin": ("-eq Punctures -B Robin -NumBH 1 -bhmp1 0.5 -bhpx1 0.1 -bhsz1 0.1 -L 40 -N 25 -O 4 -l 3 "
                "-nu2 5 -s 1e-12 -Dp 0.5", 1e-5, 1e-5),
    # merged and off-axis boxes (cuts through a box's middle node), 2nd order
    "o2_binary": (BIN + " -Dp 0.5", 1e-9, 1e-6),
    # per-box cuts as node values, no interpolated files
    "o2_binary_nodes": (BIN + " -int no -pint no", 1e-9, 1e-6),
    # per-box planes (-p2d), interpolated through 0 where the box holds it
    "o2_binary_planes": (BIN + " -p2d yes -p1d no -pint no", 1e-9, 1e-6),
}


def parse_data_file(path):
    text, vals = [], []
    for line in open(path):
        t = line.rstrip("\n").split("\t")
        t = [x for x in t if x != ""]
        if not t:
            text.append(b"")
            vals.append(np.nan)
            continue
        text.append("\t".join(t[:-1]).encode())
        vals.append(float(t[-1]))
    return np.array(text, dtype="S64"), np.array(vals)


def collect(outdir):
    rec = {}
    names = sorted(f for f in os.listdir(outdir) if f != "stdout0.out")
    rec["files"] = np.array([n.encode() for n in names], dtype="S64")
    for n in names:
        p = os.path.join(outdir, n)
        if n.endswith(".run"):
            rec["run_args"] = np.array([a.encode() for a in open(p).read().split()[1:]], dtype="S64")
        elif n == "Loo.gp":
            cyc = [int(line.split()[0]) for line in open(p) if line.strip()]
            rec["loo_levels"] = np.array(cyc.count(0))
        else:
            rec[n + "__text"], rec[n + "__vals"] = parse_data_file(p)
    return rec


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    for name, (args, value_tol, mg_tol) in OUTPUT_CASES.items():
        run = os.path.join(ROOT, "oracle", "_ref", "out_" + name)
        shutil.rmtree(run, ignore_errors=True)
        os.makedirs(run)
        subprocess.run([REF_CLI] + args.split() + ["-o", "Output"], cwd=run, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        rec = collect(os.path.join(run, "Output"))
        rec["args"] = np.array(args.encode())
        rec["value_tol"] = np.array(value_tol)
        rec["mg_tol"] = np.array(mg_tol)
        os.makedirs(os.path.join(HERE, "output"), exist_ok=True)
        np.savez_compressed(os.path.join(HERE, "output", name + ".npz"), **rec)
        print(name, len(rec["files"]), "files")


if __name__ == "__main__":
    main()
