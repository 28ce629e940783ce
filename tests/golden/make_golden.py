"""Regenerates tests/golden/*.npz from the REFERENCE solver itself.

Needs the reference sources (oracle/Makefile `ref` target builds
oracle/_ref/ref_harness from them); run in the build container only:

    make -C oracle ref && python tests/golden/make_golden.py

For every case it records, from the unmodified reference:
  * the box geometry (points, ghost width, origin, spacing, centre),
  * the coefficient fields b, c (d, e) sampled on every box,
  * u after exactly two FAS V-cycles from u = 0 (sampled),
  * the per-cycle top-level norms and the ADM masses at 17 digits,
  * for the fixed-point cases, u after the reference's own stop rule and
    further cycles until max|du| <= 1e-14 (sampled), with its ADM masses.
Samples are the three centre lines of each box plus 256 seeded points, which
keeps the fixtures small; the oracle must reproduce them bit for bit.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
sys.path.insert(0, ROOT)

from tests.cases import CASES, CONFIG1  # noqa: E402

FIXED = {"o2_single", "o4_spin", "o4_binary_merge"}


def read_meta(d):
    boxes, cyc, adm = [], [], []
    for line in open(os.path.join(d, "meta.txt")):
        t = line.split()
        if t[0] == "box":
            i = t.index("n")
            n = [int(x) for x in t[i + 1:i + 4]]
            buf = int(t[t.index("buf") + 1])
            x0 = [float(x) for x in t[t.index("x0") + 1:t.index("x0") + 4]]
            dd = [float(x) for x in t[t.index("d") + 1:t.index("d") + 4]]
            c = [float(x) for x in t[t.index("c") + 1:t.index("c") + 4]]
            lev = int(t[t.index("level") + 1])
            boxes.append((lev, n, buf, x0, dd, c))
        elif t[0] == "cycle":
            cyc.append(float(t[2]))
        elif t[0] == "adm":
            adm.append(float(t[2]))
    return boxes, np.array(cyc), np.array(adm)


def sample_index(n, seed):
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    idx = [np.ravel_multi_index((np.full(nx, nz // 2), np.full(nx, ny // 2), np.arange(nx)), (nz, ny, nx)),
           np.ravel_multi_index((np.full(ny, nz // 2), np.arange(ny), np.full(ny, nx // 2)), (nz, ny, nx)),
           np.ravel_multi_index((np.arange(nz), np.full(nz, ny // 2), np.full(nz, nx // 2)), (nz, ny, nx)),
           rng.integers(0, nx * ny * nz, 256)]
    return np.concatenate(idx)


def run(mode, args, out):
    subprocess.run([HARNESS, mode, out, "--"] + args.split() + ["-o", out + "_run"], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd="/tmp")


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: make -C oracle ref")
    cases = dict(CASES)
    cases["config1"] = CONFIG1
    for name, args in cases.items():
        rec = {"args": np.array(args)}
        tmp = f"/tmp/golden_{name}"
        run("coeff", args, tmp + "_coeff")
        boxes, _, _ = read_meta(tmp + "_coeff")
        rec["box_level"] = np.array([b[0] for b in boxes])
        rec["box_n"] = np.array([b[1] for b in boxes])
        rec["box_buf"] = np.array([b[2] for b in boxes])
        rec["box_origin"] = np.array([b[3] for b in boxes])
        rec["box_d"] = np.array([b[4] for b in boxes])
        rec["box_c"] = np.array([b[5] for b in boxes])
        modes = [("coeff", tmp + "_coeff"), ("cyc2", tmp + "_cyc2")]
        run("cycles:2", args, tmp + "_cyc2")
        if name in FIXED:
            run("fixed:1e-14:80", args, tmp + "_fixed")
            modes.append(("fixed", tmp + "_fixed"))
        for tag, d in modes:
            _, cyc, adm = read_meta(d)
            rec[f"{tag}_norms"] = cyc
            rec[f"{tag}_adm"] = adm
            for g, b in enumerate(boxes):
                idx = sample_index(b[1], 1000 + g)
                rec[f"idx_b{g}"] = idx
                fields = ["u"] if tag != "coeff" else [f for f in ("b", "c", "d", "e")
                                                     if os.path.exists(f"{d}/b{g}_{f}.f64")]
                for f in fields:
                    v = np.fromfile(f"{d}/b{g}_{f}.f64")
                    rec[f"{tag}_{f}_b{g}"] = v[idx]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, "boxes", len(boxes), "saved")


if __name__ == "__main__":
    main()
