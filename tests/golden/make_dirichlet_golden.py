"""Regenerates tests/golden/dirichlet/*.npz: runs of the REFERENCE's own
Olliptic.x (oracle/_ref, `make -C oracle ref`) without -B, i.e. with its
default Dirichlet boundary (u on the outer ghost layers fixed to the
boundary function: 0 for punctures, the Gaussian for the Gaussian test).

    make -C oracle ref && python tests/golden/make_dirichlet_golden.py

Each fixture holds the printed u.X, u.Y, u.Z (first column as text, values
as floats, as tests/golden/output) and the cycles the reference ran.
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
DIRICHLET_CASES = {
    "o2_binary": ("-eq Punctures -NumBH 2 -bhmp1 0.487209 -bhy1 3 -bhpx1 -0.09 -bhmp2 0.487209 -bhy2 -3 "
                  "-bhpx2 0.09 -L 40 -N 25 -O 2 -l 4 -nu2 5 -s 1e-12 -Dp 0.5 -p1d no"),
    "o4_gaussian": "-eq Poisson -L 10 -N 25 -O 4 -l 3 -s 1e-12 -Dp 0.1 -p1d no",
}


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "dirichlet"), exist_ok=True)
    for name, args in DIRICHLET_CASES.items():
        run = os.path.join(ROOT, "oracle", "_ref", "dirichlet_" + name)
        shutil.rmtree(run, ignore_errors=True)
        os.makedirs(run)
        subprocess.run([REF_CLI] + args.split() + ["-o", "Output"], cwd=run, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        rec = {"args": np.array(args.encode())}
        for f in ("u.X", "u.Y", "u.Z"):
            rec[f + "__text"], rec[f + "__vals"] = parse_data_file(os.path.join(run, "Output", f))
        cyc = [int(line.split()[0]) for line in open(os.path.join(run, "Output", "Loo.gp")) if line.strip()]
        rec["cycles"] = np.array(max(cyc) + 1)
        np.savez_compressed(os.path.join(HERE, "dirichlet", name + ".npz"), **rec)
        print(name, int(rec["cycles"]), "cycles")


if __name__ == "__main__":
    main()
