"""Regenerates tests/golden/export/*.npz: initial data exported for other
codes by the REFERENCE's own Olliptic.x (oracle/_ref, built from its
unmodified sources by `make -C oracle ref`).

    make -C oracle ref && python tests/golden/make_export_golden.py

The input grids are made here from a fixed seed (points inside the domain,
some on grid nodes, some near the punctures): BAM files grid_0, grid_0a,
grid_1 in BAM's fixed-width layout, Zcode files grid_00-00.mgid,
grid_00-01.mgid, grid_01-00.mgid and the shell grid_SH-xm.mgid.  The
reference runs with -ioZ only: its BAM exporter (multigrid::Print_IO_BAM)
does not end when built against a C++11 or later standard library (its read
loop ends on the end-of-file flag, which every seekg clears, so it spins on
the failed stream; a run here was stopped after ten minutes at full CPU).
So the BAM points are also written, in BAM's order, to one more Zcode file,
grid_02-00.mgid, whose reference output gives the values BAM must carry.
The fixture holds every input file and the reference's <file>_m outputs.
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "Olliptic.x")

ARGS = ("-eq Punctures -B Robin -NumBH 2 -bhmp1 0.487209 -bhy1 3 -bhpx1 -0.09 -bhmp2 0.487209 -bhy2 -3 "
        "-bhpx2 0.09 -L 40 -N 25 -O 2 -l 4 -nu2 5 -s 1e-12 -p1d no -pint no -ioZ yes -iof grid_")
BAM_FILES = {"grid_0": 40, "grid_0a": 16, "grid_1": 16}
ZCODE_FILES = {"grid_00-00.mgid": 30, "grid_00-01.mgid": 12, "grid_01-00.mgid": 12, "grid_SH-xm.mgid": 10}


def points(rng, n):
    p = rng.uniform(-15.0, 15.0, size=(n, 3))
    p[: n // 4] = np.round(p[: n // 4] / 1.25) * 1.25          # on nodes of the refinement levels
    p[n // 4: n // 2] = rng.normal(0.0, 0.6, size=(n // 2 - n // 4, 3)) + np.array([0.0, 3.0, 0.0])
    return p


def inputs():
    rng = np.random.default_rng(2024)
    files = {}
    for name, n in BAM_FILES.items():
        files[name] = "".join("%16.9e%17.9e%17.9e%24.15e\n" % (x, y, z, 0.0) for x, y, z in points(rng, n))
    for name, n in ZCODE_FILES.items():
        files[name] = "".join("%.12f %.12f %.12f %.1f\n" % (x, y, z, 0.0) for x, y, z in points(rng, n))
    # the BAM points again, as a Zcode level-2 file (the text of BAM's x, y, z)
    files["grid_02-00.mgid"] = "".join(line[:50] + " 0.0\n" for name in BAM_FILES
                                       for line in files[name].splitlines())
    return files


def main():
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference first: make -C oracle ref")
    run = os.path.join(ROOT, "oracle", "_ref", "export_run")
    shutil.rmtree(run, ignore_errors=True)
    os.makedirs(run)
    files = inputs()
    for name, text in files.items():
        with open(os.path.join(run, name), "w") as f:
            f.write(text)
    subprocess.run([REF_CLI] + ARGS.split() + ["-o", "Output"], cwd=run, check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    rec = {"args": np.array(ARGS.encode())}
    for name, text in files.items():
        rec["in:" + name] = np.array(text.encode())
        if name not in BAM_FILES:
            rec["out:" + name + "_m"] = np.array(open(os.path.join(run, name + "_m"), "rb").read())
    os.makedirs(os.path.join(HERE, "export"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "export", "o2_binary.npz"), **rec)
    print(sorted(rec))


if __name__ == "__main__":
    main()
