"""Regenerates tests/golden/configs/{config1,config2,config3}.npz: the fixed
point of the benchmark problems, sampled, for the GPU parity tests.

The three problems are the benchmark configurations as command lines
(tests/cases.py CONFIG1, CONFIG2, CONFIG3): the single boosted puncture at
2nd order (7 boxes), the equal-mass binary of pars/Punctures/TestBH.run at
4th order on 65^3 boxes (13 boxes) and the same binary at 8th order on
129^3 boxes (14 boxes).

For every problem the fixture holds:
  * the box geometry (level, points, ghost width, origin, spacing);
  * u after exactly two FAS V-cycles from u = 0, from the UNMODIFIED
    reference (oracle/_ref/ref_harness, built by `make -C oracle ref`), at
    the sample points -- the oracle must reproduce these bit for bit, which
    pins the restatement on this geometry;
  * the fixed point: u after the reference's stop rule and further V-cycles
    until max |du| <= 1e-14 on every box (or the cycle cap), at the sample
    points, with its ADM masses at 17 digits and the last cycles' changes.
    It comes from the reference itself where that run finishes in this
    container's time (config1, config2) and from the oracle otherwise
    (config3: the reference needs about 3.4 minutes a cycle there, and the
    oracle's first two cycles are checked against the reference's on every
    point before its fixed point is taken); the key `fixed_source` says which.
Sample points of a box: its three centre lines, the x, y and z lines through
the grid point nearest to each puncture (where the box holds it), and 2048
seeded points.

Needs the reference sources; run in the build container only:

    make -C oracle ref && python tests/golden/make_config_golden.py [config1 config2 config3]

Reference dumps are kept under /tmp/config_golden/ and reused when present.
CONFIG_GOLDEN_FIXED_TOL in the environment changes the fixed point's bound
on max |du| (default 1e-14), CONFIG_GOLDEN_FIXED_MAX its cycle cap (default
120) and CONFIG_GOLDEN_OUT the output folder; each
cycle of the oracle's fixed point is logged to stderr.  With
CONFIG_GOLDEN_ANDERSON=m (> 0) the oracle's V-cycle map is iterated with
Anderson mixing of depth m over all of u (the same fixed point; the
reference's own iteration contracts only about 0.93 a cycle on config3, so
plain cycles do not reach 1e-12 within the cycle cap); the recorded changes
are then those of a plain cycle from each iterate, and the fixed point is
the last plain cycle's result.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
OUT = os.environ.get("CONFIG_GOLDEN_OUT", os.path.join(HERE, "configs"))
WORK = "/tmp/config_golden"
sys.path.insert(0, ROOT)

from tests.cases import CONFIG1, CONFIG2, CONFIG3  # noqa: E402
from tests.golden.make_golden import read_meta  # noqa: E402

CONFIGS = {"config1": CONFIG1, "config2": CONFIG2, "config3": CONFIG3}
FIXED_FROM = {"config1": "reference", "config2": "reference", "config3": "oracle"}
FIXED_TOL = float(os.environ.get("CONFIG_GOLDEN_FIXED_TOL", "1e-14"))
FIXED_MAX = int(os.environ.get("CONFIG_GOLDEN_FIXED_MAX", "120"))
ANDERSON = int(os.environ.get("CONFIG_GOLDEN_ANDERSON", "0"))
RANDOM_POINTS = 2048


def harness(mode, args, out):
    """Runs the reference harness once; a finished dump is reused."""
    if os.path.exists(os.path.join(out, "meta.txt")):
        return out
    os.makedirs(WORK, exist_ok=True)
    subprocess.run([HARNESS, mode, out, "--"] + args.split() + ["-o", out + "_run"], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd=WORK)
    return out


def read_deltas(d):
    return np.array([float(line.split()[3]) for line in open(os.path.join(d, "meta.txt"))
                     if line.startswith("cycle ")])


def puncture_points(args):
    import ollipticid_gb300 as og
    P = og.parse_olliptic_args(args.split())
    return [(P.x[i], P.y[i], P.z[i]) for i in range(P.numbh)]


def sample_index(level, n, origin, d, punctures, seed):
    """Flat lexicographic indices (i fastest) of the sample points of a box."""
    nx, ny, nz = (int(v) for v in n)
    shape = (nz, ny, nx)
    lines = [((nz // 2,) * nx, (ny // 2,) * nx, range(nx)),
             ((nz // 2,) * ny, range(ny), (nx // 2,) * ny),
             (range(nz), (ny // 2,) * nz, (nx // 2,) * nz)]
    for (px, py, pz) in punctures:
        ijk = [int(round((p - o) / h)) for p, o, h in zip((px, py, pz), origin, d)]
        if all(0 <= ijk[a] < n[a] for a in range(3)):
            i, j, k = ijk
            lines += [((k,) * nx, (j,) * nx, range(nx)), ((k,) * ny, range(ny), (i,) * ny),
                      (range(nz), (j,) * nz, (i,) * nz)]
    idx = [np.ravel_multi_index((np.array(kk), np.array(jj), np.array(ii)), shape) for kk, jj, ii in lines]
    rng = np.random.default_rng(seed)
    idx.append(rng.integers(0, nx * ny * nz, RANDOM_POINTS))
    return np.unique(np.concatenate(idx)).astype(np.int32)


def oracle_fixed(args, cyc2_dir):
    """The oracle's fixed point: the reference stop rule, then V-cycles
    until max |du| <= FIXED_TOL.  Its first two cycles are checked first
    against the reference's own on every point of every box, bit for bit, so
    that the restatement is pinned on this geometry before it is used."""
    import ollipticid_gb300 as og
    from oracle import oracle as O
    orc = O.Oracle(og.parse_olliptic_args(args.split()).oracle_dict())
    for _ in range(2):
        orc.vcycle()
    for g in range(orc.nboxes):
        ref = np.fromfile(os.path.join(cyc2_dir, f"b{g}_u.f64"))
        if not np.array_equal(orc.field(g).ravel(), ref):
            raise SystemExit(f"oracle differs from the reference after two cycles on box {g}")
    orc.solve()
    if ANDERSON > 0:
        return anderson_fixed(orc, ANDERSON)
    prev = orc.all_u()
    deltas = []
    for _ in range(FIXED_MAX):
        orc.vcycle()
        cur = orc.all_u()
        deltas.append(max(float(np.max(np.abs(a - b))) for a, b in zip(cur, prev)))
        print(f"fixed-point cycle {len(deltas)}: max |du| = {deltas[-1]:.3e}", file=sys.stderr, flush=True)
        prev = cur
        if deltas[-1] <= FIXED_TOL:
            break
    return prev, np.array(orc.adm()), np.array(deltas)


def anderson_fixed(orc, m):
    """Fixed point of the oracle's V-cycle map G by Anderson mixing of depth
    m on the vector of every box's u: x <- x + f - (dX + dF) gamma with
    f = G(x) - x and gamma the least-squares fit of f by the last m changes
    of f (normal equations, slightly regularised).  Near the rounding floor
    of G the mixing stops helping; when four cycles in a row have not
    improved on the smallest change of a plain cycle seen, the history
    restarts from the best iterate.  Stops when a plain cycle from the current iterate changes u by
    at most FIXED_TOL, or after FIXED_MAX cycles; returns the plain cycle's
    result from the best iterate, and the changes up to it."""
    shapes = [(b.nz, b.ny, b.nx) for b in orc.boxes]
    sizes = [int(np.prod(sh)) for sh in shapes]

    def get():
        return np.concatenate([a.ravel() for a in orc.all_u()])

    def put(x):
        at = 0
        for g, (sh, n) in enumerate(zip(shapes, sizes)):
            orc.set_field(g, "u", x[at:at + n].reshape(sh))
            at += n

    x = get()
    dX, dF, deltas = [], [], []
    x_prev = f_prev = None
    best = (np.inf, None, None, 0)   # (change, x, G(x), cycles so far)
    since = 0                        # cycles since the best
    for _ in range(FIXED_MAX):
        put(x)
        orc.vcycle()
        gx = get()
        f = gx - x
        d = float(np.max(np.abs(f)))
        deltas.append(d)
        print(f"anderson cycle {len(deltas)}: max |du| of a plain cycle = {d:.3e}", file=sys.stderr, flush=True)
        if d < best[0]:
            best = (d, x, gx, len(deltas))
            since = 0
        else:
            since += 1
        if d <= FIXED_TOL:
            break
        if since >= 4:   # no progress: restart from the best iterate's plain step
            x, dX, dF, x_prev, f_prev = best[2], [], [], None, None
            since = 0
            continue
        if f_prev is not None:
            dX.append(x - x_prev)
            dF.append(f - f_prev)
            if len(dX) > m:
                dX.pop(0)
                dF.pop(0)
        x_prev, f_prev = x, f
        if dF:
            A = np.array([[float(np.dot(a, b)) for b in dF] for a in dF])
            r = np.array([float(np.dot(a, f)) for a in dF])
            A += np.eye(len(dF)) * 1e-12 * np.trace(A) / len(dF)
            gamma = np.linalg.solve(A, r)
            x = x + f
            for gk, dx, df in zip(gamma, dX, dF):
                x -= gk * (dx + df)
        else:
            x = gx
    put(best[2])
    return orc.all_u(), np.array(orc.adm()), np.array(deltas[:best[3]])


def make(name):
    args = CONFIGS[name]
    base = os.path.join(WORK, name)
    jobs = [("cycles:2", base + "_cyc2")]
    if FIXED_FROM[name] == "reference":
        jobs.append((f"fixed:{FIXED_TOL}:{FIXED_MAX}", base + "_fixed"))
    with ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(lambda j: harness(j[0], args, j[1]), jobs))
    boxes, cyc2_norms, cyc2_adm = read_meta(base + "_cyc2")
    rec = {"args": np.array(args), "fixed_source": np.array(FIXED_FROM[name]),
           "box_level": np.array([b[0] for b in boxes]), "box_n": np.array([b[1] for b in boxes]),
           "box_buf": np.array([b[2] for b in boxes]), "box_origin": np.array([b[3] for b in boxes]),
           "box_d": np.array([b[4] for b in boxes]), "cyc2_norms": cyc2_norms, "cyc2_adm": cyc2_adm}
    if FIXED_FROM[name] == "reference":
        _, fixed_norms, fixed_adm = read_meta(base + "_fixed")
        fixed_u = [np.fromfile(f"{base}_fixed/b{g}_u.f64") for g in range(len(boxes))]
        rec["fixed_deltas"] = read_deltas(base + "_fixed")
        rec["fixed_norms"] = fixed_norms
    else:
        u, fixed_adm, rec["fixed_deltas"] = oracle_fixed(args, base + "_cyc2")
        fixed_u = [x.ravel() for x in u]
    rec["fixed_adm"] = fixed_adm
    pts = puncture_points(args)
    for g, b in enumerate(boxes):
        idx = sample_index(b[0], b[1], b[3], b[4], pts, 2000 + g)
        rec[f"idx_b{g}"] = idx
        rec[f"cyc2_u_b{g}"] = np.fromfile(f"{base}_cyc2/b{g}_u.f64")[idx]
        rec[f"fixed_u_b{g}"] = fixed_u[g][idx]
    os.makedirs(OUT, exist_ok=True)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **rec)
    print(name, "boxes", len(boxes), "fixed from", FIXED_FROM[name], "last |du|", rec["fixed_deltas"][-1], flush=True)


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: make -C oracle ref")
    names = sys.argv[1:] or list(CONFIGS)
    for n in names:
        make(n)


if __name__ == "__main__":
    main()
