"""Regenerates tests/golden/bowen_york/*.npz from the REFERENCE solver itself:
its Bowen-York momentum-constraint test (-eq Bowen-York, four unknowns V1,
V2, V3, lambda: include/elliptic.h:772-803, src/operator.cc:370-398,
1320-1408, 3313-3408), run by oracle/_ref/ref_harness (built from the
unmodified sources by `make -C oracle ref`).  Build container only:

    make -C oracle ref && python tests/golden/make_bowen_york_golden.py

Each case records the box geometry, the sources rho0..rho2 (sampled, plus
every point where one is non-zero: the momenta spread over a ball of one
cell diagonal around each puncture) and the four variables at the
reference's fixed point (its own stop rule, then V-cycles until the largest
change of any variable is <= 1e-14), sampled on the three centre lines of
each box and 256 seeded points.  cli_o2.npz holds the reference's own
printout of the O2 case (Olliptic.x, -s 1e-14 so that its stop lies near the
fixed point): the interpolated cuts V1.X, V2.Y, V3.Z, lambda.X (first column
as text, values as floats) and the per-box cut lambda-l3b0-0.x.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
sys.path.insert(0, ROOT)
from tests.golden.make_golden import read_meta, sample_index  # noqa: E402
from tests.golden.make_output_golden import parse_data_file  # noqa: E402

REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")
CLI_FILES = ("V1.X", "V2.Y", "V3.Z", "lambda.X", "lambda-l3b0-0.x")

BY_ARGS = ("-eq Bowen-York -B Robin -NumBH 2 -bhx1 -1.5 -bhx2 1.5 -bhpx1 0.05 -bhpy1 0.1 -bhpy2 -0.1 "
           "-bhpz2 0.03 -L 20 -N 25 -l 3 -s 1e-10")
CASES = {"o2": BY_ARGS + " -O 2", "o4": BY_ARGS + " -O 4", "o6": BY_ARGS + " -O 6",
         "o2_dirichlet": BY_ARGS.replace("-B Robin", "-B Dirichlet") + " -O 2"}
VARS = ("V1", "V2", "V3", "lambda")


def run(mode, args, out):
    subprocess.run([HARNESS, mode, out, "--"] + args.split() + ["-o", out + "_run"], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd="/tmp")


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: make -C oracle ref")
    for name, args in CASES.items():
        tmp = f"/tmp/golden_by_{name}"
        run("coeff", args, tmp + "_coeff")
        run("fixed:1e-14:300", args, tmp + "_fixed")
        boxes, _, _ = read_meta(tmp + "_coeff")
        _, fixed_norms, _ = read_meta(tmp + "_fixed")
        rec = {"args": np.array(args), "fixed_norms": fixed_norms}
        rec["box_level"] = np.array([b[0] for b in boxes])
        rec["box_n"] = np.array([b[1] for b in boxes])
        for g, b in enumerate(boxes):
            idx = sample_index(b[1], 1000 + g)
            rho = [np.fromfile(f"{tmp}_coeff/b{g}_rho{c}.f64") for c in range(3)]
            ball = np.flatnonzero(np.any(np.stack(rho) != 0.0, axis=0))
            rec[f"idx_b{g}"] = idx
            rec[f"ball_b{g}"] = ball
            for c in range(3):
                rec[f"rho{c}_b{g}"] = rho[c][idx]
                rec[f"rho{c}_ball_b{g}"] = rho[c][ball]
            for v in VARS:
                rec[f"{v}_b{g}"] = np.fromfile(f"{tmp}_fixed/b{g}_{v}.f64")[idx]
        np.savez_compressed(os.path.join(HERE, "bowen_york", name + ".npz"), **rec)
        print(name, "boxes", len(boxes), "cycles", len(fixed_norms), "ball points",
              [len(rec[f"ball_b{g}"]) for g in range(len(boxes))])


def cli_golden():
    run = "/tmp/golden_by_cli"
    subprocess.run(["rm", "-rf", run], check=True)
    os.makedirs(run)
    args = CASES["o2"].replace("-s 1e-10", "-s 1e-14")
    subprocess.run([REF_CLI] + args.split() + ["-o", "Output"], cwd=run, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    rec = {"args": np.array(args.encode())}
    for f in CLI_FILES:
        rec[f + "__text"], rec[f + "__vals"] = parse_data_file(os.path.join(run, "Output", f))
    np.savez_compressed(os.path.join(HERE, "bowen_york", "cli_o2.npz"), **rec)
    print("cli_o2", sorted(os.listdir(os.path.join(run, "Output")))[:6], "...")


if __name__ == "__main__":
    main()
    cli_golden()
