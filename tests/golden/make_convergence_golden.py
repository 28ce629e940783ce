"""Regenerates tests/golden/convergence/*.npz: the self-convergence study of
the reference's utils/run_conv.sh, run with the REFERENCE's own Olliptic.x
(oracle/_ref, built from its unmodified sources by `make -C oracle ref`).

    make -C oracle ref && python tests/golden/make_convergence_golden.py

run_conv.sh solves one spinning puncture (-bhmp1 1.0 -bhsz1 0.2, L = 100)
at several resolutions, joins the printed u.X cuts and fits the order p of
|u_h - u_h/2| ~ h^p.  Here each case runs N = 25, 49, 97 (h halves exactly:
24, 48, 96 intervals) with -Dp L/256, so every u.X point is the same x in all
three runs, and stores, per N, the printed x and u (18 digits, exact) and the
reference's own orders:
  p_inf, p_l2   log2 of max|u_25 - u_49| / max|u_49 - u_97| (and the RMS
                ratio) over the points with |x| > 2, away from the puncture.
The run takes about two minutes (the N = 97 solves).
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")

BASE = "-eq Punctures -B Robin -NumBH 1 -bhmp1 1.0 -bhsz1 0.2 -L 100 -l 4 -s 1e-10 -nu2 20 -Dp 0.390625 -p1d no"
CONV_CASES = {"o2_spin_l4": BASE + " -O 2", "o4_spin_l4": BASE + " -O 4"}
RESOLUTIONS = (25, 49, 97)


def orders(x, u1, u2, u3, far=2.0):
    sel = np.abs(x) > far
    d12, d23 = (u1 - u2)[sel], (u2 - u3)[sel]
    p_inf = np.log2(np.max(np.abs(d12)) / np.max(np.abs(d23)))
    p_l2 = np.log2(np.sqrt(np.mean(d12 * d12) / np.mean(d23 * d23)))
    return float(p_inf), float(p_l2)


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "convergence"), exist_ok=True)
    for name, args in CONV_CASES.items():
        rec = {"args": np.array(args.encode()), "resolutions": np.array(RESOLUTIONS)}
        cuts = []
        for N in RESOLUTIONS:
            run = os.path.join(ROOT, "oracle", "_ref", f"conv_{name}_{N}")
            shutil.rmtree(run, ignore_errors=True)
            os.makedirs(run)
            subprocess.run([REF_CLI] + args.split() + ["-N", str(N), "-o", "Output"], cwd=run, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            a = np.loadtxt(os.path.join(run, "Output", "u.X"))
            rec[f"x_{N}"], rec[f"u_{N}"] = a[:, 0], a[:, 1]
            cuts.append(a)
        assert all((c[:, 0] == cuts[0][:, 0]).all() for c in cuts)
        rec["p_inf"], rec["p_l2"] = orders(cuts[0][:, 0], *(c[:, 1] for c in cuts))
        np.savez_compressed(os.path.join(HERE, "convergence", name + ".npz"), **rec)
        print(name, "p_inf %.4f p_l2 %.4f" % (rec["p_inf"], rec["p_l2"]))


if __name__ == "__main__":
    main()
