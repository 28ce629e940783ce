"""Regenerates tests/golden/storage/*.npz: the point order of the REFERENCE's
3-D dumps (Olliptic.x -p3d, ffunction::Print_3D: every point of a box in its
storage order, domain::Fix_Points) from its own Olliptic.x (oracle/_ref,
`make -C oracle ref`).

    make -C oracle ref && python tests/golden/make_storage_golden.py

For the Gaussian test at 2nd and 4th order (ghost bands 1 and 2) the fixture
holds, per dump file, the order of its points as indices into the box's
lexicographic layout (i fastest; the node indices are the ranks of the
printed coordinates among the box's nodes), and for the 2nd-order case the
printed u as float32.
"""
import glob
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")
BASE = "-eq Poisson -B Robin -L 10 -N 25 -l 2 -s 1e-10 -p1d no -pint no -p3d yes"
STORAGE_CASES = {"o2": (BASE + " -O 2", True), "o4": (BASE + " -O 4", False)}


def order_of(path):
    a = np.loadtxt(path)
    idx = []
    for c in range(3):
        nodes = np.unique(a[:, c])
        idx.append(np.searchsorted(nodes, a[:, c]))
    n = [len(np.unique(a[:, c])) for c in range(3)]
    return ((idx[2] * n[1] + idx[1]) * n[0] + idx[0]).astype(np.int32), np.array(n), a[:, 3]


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    os.makedirs(os.path.join(HERE, "storage"), exist_ok=True)
    for name, (args, keep_u) in STORAGE_CASES.items():
        run = os.path.join(ROOT, "oracle", "_ref", "storage_" + name)
        shutil.rmtree(run, ignore_errors=True)
        os.makedirs(run)
        subprocess.run([REF_CLI] + args.split() + ["-o", "Output"], cwd=run, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        rec = {"args": np.array(args.encode())}
        files = sorted(os.path.basename(p) for p in glob.glob(os.path.join(run, "Output", "*.xyz")))
        rec["files"] = np.array([f.encode() for f in files], dtype="S64")
        for f in files:
            order, n, u = order_of(os.path.join(run, "Output", f))
            rec[f + "__order"], rec[f + "__n"] = order, n
            if keep_u:
                rec[f + "__u"] = u.astype(np.float32)
        np.savez_compressed(os.path.join(HERE, "storage", name + ".npz"), **rec)
        print(name, files)


if __name__ == "__main__":
    main()
