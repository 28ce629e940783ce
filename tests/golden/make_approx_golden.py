"""Regenerates tests/golden/approx/*.npz: the REFERENCE's analytic puncture
approximation (Olliptic.x -m AppPuncture, elliptic::ApproximateID), from its
own Olliptic.x built from its unmodified sources (`make -C oracle ref`).

    make -C oracle ref && python tests/golden/make_approx_golden.py

For each case the fixture holds the printed cuts u.X, u.Y, u.Z and u.XY
(first column(s) as text, values as floats, as tests/golden/output) and the
u the reference prints at each puncture (" u : " lines, 8 digits).
"""
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from tests.golden.make_output_golden import parse_data_file  # noqa: E402

REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")
APPROX_CASES = {
    # spin and momentum on both punctures (cross term), off-axis, unequal masses
    "binary_spin_boost": ("-eq Punctures -B Robin -NumBH 2 -bhmp1 0.5 -bhx1 0.3 -bhy1 3 -bhpx1 -0.09 -bhsz1 0.05 "
                          "-bhmp2 0.45 -bhy2 -3 -bhpx2 0.09 -bhpy2 0.02 -bhsx2 0.03 -L 40 -N 25 -O 4 -l 3 "
                          "-m AppPuncture -Dp 0.5 -p1d no"),
    # one spinning, moving puncture off the grid nodes, 2nd order (on a node
    # the formula's r -> 0 limit cancels catastrophically: r is clamped to
    # 1e-10 and u there is of order 1e10, rounding-dominated)
    "single_spin": ("-eq Punctures -B Robin -NumBH 1 -bhmp1 1.0 -bhx1 0.11 -bhy1 -0.07 -bhz1 0.03 -bhsz1 0.2 "
                    "-bhpx1 0.05 -L 100 -N 33 -O 2 -l 4 -m AppPuncture -Dp 0.5 -p1d no"),
}


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "approx"), exist_ok=True)
    for name, args in APPROX_CASES.items():
        run = os.path.join(ROOT, "oracle", "_ref", "approx_" + name)
        shutil.rmtree(run, ignore_errors=True)
        os.makedirs(run)
        r = subprocess.run([REF_CLI] + args.split() + ["-o", "Output"], cwd=run, check=True, capture_output=True,
                           text=True)
        rec = {"args": np.array(args.encode())}
        rec["u_at_punctures"] = np.array([float(v) for v in re.findall(r" u : (\S+)", r.stdout)])
        for f in ("u.X", "u.Y", "u.Z", "u.XY"):
            rec[f + "__text"], rec[f + "__vals"] = parse_data_file(os.path.join(run, "Output", f))
        np.savez_compressed(os.path.join(HERE, "approx", name + ".npz"), **rec)
        print(name, rec["u_at_punctures"])


if __name__ == "__main__":
    main()
