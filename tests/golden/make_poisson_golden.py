"""Regenerates tests/golden/poisson/*.npz: the reference's Gaussian test
(-eq Poisson: Lap u + u^2 = a e^{-r^2}(a + e^{r^2/2}(r^2 - 3)), solution
u = a e^{-r^2/2}, a = 0.004) from its own Olliptic.x (oracle/_ref, built
from its unmodified sources by `make -C oracle ref`).

    make -C oracle ref && python tests/golden/make_poisson_golden.py

Each case (2nd and 4th order, L = 10, 3 levels, Robin boundary) is run at
N = 25 and 49; the fixture holds, per N, the printed u.X, u.Y, u.Z (first
column as text, values as floats), the cycles the reference ran, and its
largest distance from the exact Gaussian on the u.X points.
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
POISSON_CASES = {"o2": BASE + " -O 2", "o4": BASE + " -O 4"}
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
            rec[f"max_error_{N}"] = np.array(np.max(np.abs(a[:, 1] - 0.004 * np.exp(-0.5 * a[:, 0] ** 2))))
        np.savez_compressed(os.path.join(HERE, "poisson", name + ".npz"), **rec)
        print(name, {k: float(v) for k, v in rec.items() if k.startswith(("cycles", "max_error"))})


if __name__ == "__main__":
    main()
