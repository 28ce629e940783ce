"""Regenerates tests/golden/poisson/*.npz: the reference's test equations
(Lap u + u^2 = source) from its own Olliptic.x (oracle/_ref, built from its
unmodified sources by `make -C oracle ref`): the Gaussian test (-eq Poisson,
solution u = a e^{-r^2/2}, a = 0.004) at 2nd and 4th order and
Boundary-test.

    make -C oracle ref && python tests/golden/make_poisson_golden.py

Each case (L = 10 or 20, 3 levels, Robin boundary) is run at N = 25 and 49;
the fixture holds, per N, the printed u.X, u.Y, u.Z (first column as text,
values as floats), the cycles the reference ran, and for the Gaussian test
its largest distance from the exact solution on the u.X points (NaN for the
others, whose exact solutions are not known).
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
BASE = "-eq Poisson -B Robin -L 10 -l 3 -s 1e-12 -Dp 0.1 -p1d no"
POISSON_CASES = {
    "o2": BASE + " -O 2",
    "o4": BASE + " -O 4",
    "boundary_test_o4": "-eq Boundary-test -B Robin -L 10 -l 3 -s 1e-12 -Dp 0.1 -p1d no -O 4",
}
# Multibox-test has no fixture: the reference's own runs of it (two unit
# Gaussians at x = -3, 3, L = 20, N = 25, 2nd order, Robin or Dirichlet)
# diverge on the coarsest grid (norm 1e10 in the first cycle) and did not
# finish in ten minutes; the test checks its initial state instead.
RESOLUTIONS = (25, 49)


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "poisson"), exist_ok=True)
    for name, args in POISSON_CASES.items():
        rec = {"args": np.array(args.encode()), "resolutions": np.array(RESOLUTIONS)}
        for N in RESOLUTIONS:
            run = os.path.join(ROOT, "oracle", "_ref", f"poisson_{name}_{N}")
            shutil.rmtree(run, ignore_errors=True)
            os.makedirs(run)
            subprocess.run([REF_CLI] + args.split() + ["-N", str(N), "-o", "Output"], cwd=run, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            for f in ("u.X", "u.Y", "u.Z"):
                rec[f"{f}_{N}__text"], rec[f"{f}_{N}__vals"] = parse_data_file(os.path.join(run, "Output", f))
            cyc = [int(line.split()[0]) for line in open(os.path.join(run, "Output", "Loo.gp")) if line.strip()]
            rec[f"cycles_{N}"] = np.array(max(cyc) + 1)
            a = np.loadtxt(os.path.join(run, "Output", "u.X"))
            exact = 0.004 * np.exp(-0.5 * a[:, 0] ** 2) if "-eq Poisson" in args else np.nan
            rec[f"max_error_{N}"] = np.array(np.max(np.abs(a[:, 1] - exact)))
        np.savez_compressed(os.path.join(HERE, "poisson", name + ".npz"), **rec)
        print(name, {k: float(v) for k, v in rec.items() if k.startswith(("cycles", "max_error"))})


if __name__ == "__main__":
    main()
