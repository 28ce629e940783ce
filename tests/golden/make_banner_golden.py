"""Regenerates tests/golden/banner/banners.npz: the head of the REFERENCE's
stdout0.out (elliptic::Print_Info: parameters and box listing, up to "Init
Multigrid iteration") for several command lines, from its own Olliptic.x
(oracle/_ref, `make -C oracle ref`).

    make -C oracle ref && python tests/golden/make_banner_golden.py
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
       "-bhpx2 0.09 -L 40 -N 25 -O 4 -l 4 -nu2 5 -s 1e-12")
BANNER_CASES = {
    "binary_o4": BIN,
    "scalar_field": ("-eq Punctures_scalar_field -B Robin -NumBH 1 -bhmp1 0.5 -L 40 -N 25 -O 2 -l 2 -s 1e-8 "
                     "-psc 2"),
    "gaussian_dirichlet": "-eq Poisson -L 10 -N 25 -O 6 -l 2 -s 1e-10",
    "boundary_test_tol": "-eq Boundary-test -B Robin -L 10 -N 25 -O 8 -l 2 -s 1e-20 -nu1 2",
    "approx": BIN + " -m AppPuncture",
    "wcycle": BIN + " -m Wcycle",
}
END = "  Init Multigrid iteration\n"


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "banner"), exist_ok=True)
    rec = {}
    for name, args in BANNER_CASES.items():
        run = os.path.join(ROOT, "oracle", "_ref", "banner_" + name)
        shutil.rmtree(run, ignore_errors=True)
        os.makedirs(run)
        # only the banner is kept: the run is cut short once it is written
        p = subprocess.Popen([REF_CLI] + args.split() + ["-o", "Output", "-p1d", "no", "-pint", "no"], cwd=run,
                             stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        try:
            p.wait(timeout=120)
        except subprocess.TimeoutExpired:
            p.kill()
            p.wait()
        text = open(os.path.join(run, "Output", "stdout0.out")).read()
        rec[name + "__args"] = np.array(args.encode())
        rec[name + "__banner"] = np.array(text[:text.index(END) + len(END)].encode())
    np.savez_compressed(os.path.join(HERE, "banner", "banners.npz"), **rec)
    print(sorted(rec))


if __name__ == "__main__":
    main()
