"""GPU parity: the red-black FP64 GPU solver and the CPU oracle (a bit-exact
restatement of the reference, pinned by tests/golden) converge to the same
discrete fixed point.  Red-black ordering changes the iterates, not the
fixed point, so both are driven until u stops changing and compared on every
box of every level.

Tolerances (from the reference's acceptance bar): max |u_gpu - u_oracle|
<= 1e-10 on every level, |ADM_gpu - ADM_oracle| <= 1e-9.

Points compared: every point of the base and refinement levels and the
interior of the multigrid coarse levels below the base.  The ghost layer of
those coarse levels is not fixed by the discrete system: their tau source is
S = W + OP(u) everywhere (src/elliptic.cc:1715-1721), so once W vanishes any
value there is a fixed point and what it holds depends on the path taken
(it only feeds the coarse solve, whose correction is then zero).
"""
import numpy as np
import pytest

from tests.cases import CASES, problem

U_TOL = 1e-10
ADM_TOL = 1e-9


def gpu_fixed_point(E, tol=1e-14, max_cycles=300):
    E.Solve()
    prev = [E.get_field(g) for g in range(len(E.boxes))]
    d = np.inf
    for _ in range(max_cycles):
        E.FASN()
        cur = [E.get_field(g) for g in range(len(E.boxes))]
        d = max(float(np.max(np.abs(a - b))) for a, b in zip(cur, prev))
        prev = cur
        if d <= tol:
            break
    return prev, d


@pytest.mark.gpu
@pytest.mark.parametrize("coarse", ["cluster", "one_block"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_fixed_point_matches_oracle(case, coarse, oracle_mod, monkeypatch):
    """coarse: the coarsest solve on a cluster (the default) or in one block
    (k_coarse_solve, which takes the grids no cluster does)."""
    import ollipticid_gb300 as og
    if coarse == "one_block":
        monkeypatch.setenv("OLGPU_COARSE_ONE_BLOCK", "1")
    P = problem(case)
    orc = oracle_mod.Oracle(P.oracle_dict())
    dorc = orc.fixed_point(tol=1e-14)
    uo = orc.all_u()
    with og.Elliptic(P) as E:
        assert [b.n for b in E.boxes] == [(b.nx, b.ny, b.nz) for b in orc.boxes]
        ug, dg = gpu_fixed_point(E)
        assert dg < 1e-12, f"GPU solve did not settle: last change {dg:.3e}"
        assert dorc < 1e-12, f"oracle did not settle: last change {dorc:.3e}"
        for g, (a, b) in enumerate(zip(ug, uo)):
            box = E.boxes[g]
            if box.level < E.mgrid_levels:
                w = box.buf
                a, b = a[w:-w, w:-w, w:-w], b[w:-w, w:-w, w:-w]
            err = float(np.max(np.abs(a - b)))
            assert err <= U_TOL, f"box {g} (level {E.boxes[g].level}): max|du| = {err:.3e}"
        adm_g, adm_o = E.ADM_mass, orc.adm()
        for i, (a, b) in enumerate(zip(adm_g, adm_o)):
            assert abs(a - b) <= ADM_TOL, f"ADM[{i}] {a!r} vs {b!r}"


@pytest.mark.gpu
def test_coefficients_match_oracle(oracle_mod):
    import ollipticid_gb300 as og
    P = problem("sf_binary")
    orc = oracle_mod.Oracle(P.oracle_dict())
    with og.Elliptic(P) as E:
        for g in range(len(E.boxes)):
            for name in ("b", "c", "d", "e"):
                a, b = E.get_field(g, name), orc.field(g, name)
                scale = max(1.0, float(np.max(np.abs(b))))
                assert float(np.max(np.abs(a - b))) <= 1e-13 * scale, (g, name)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["o4_binary_merge", "o8_offset", "sf_binary"])
@pytest.mark.parametrize("mixed", [False, True])
def test_row_transfers_equal_point_transfers(case, mixed, monkeypatch):
    """The separable row kernel (shared inner sums per target row) gives the
    per-point tensor sum's ghost fills and restrictions bit for bit."""
    import ollipticid_gb300 as og
    P = problem(case)
    out = []
    for points in (False, True):
        if points:
            monkeypatch.setenv("OLGPU_XFER_POINTS", "1")
        with og.Elliptic(P) as E:
            E.set_precision(mixed)
            for _ in range(3):
                E.FASN()
            out.append([E.get_field(g) for g in range(len(E.boxes))])
    for g, (a, b) in enumerate(zip(*out)):
        assert np.array_equal(a, b), f"box {g}: max diff {float(np.max(np.abs(a - b))):.3e}"


LAYOUTS = {
    "robin_split": {"OLGPU_ROBIN_SPLIT": "1"},
    "fp64_two_points": {"OLGPU_SMOOTH_PTS": "2"},
    "fp32_per_colour": {"OLGPU_SMOOTH32_LAUNCHES": "1"},
    "fp32_per_colour_two_points": {"OLGPU_SMOOTH32_LAUNCHES": "1", "OLGPU_SMOOTH32_PTS": "2"},
    "fp64_coarse_plain_slabs": {"OLGPU_COARSE_BAL": "0"},
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["o2_single", "o4_binary_merge", "o8_offset"])
@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("variant", sorted(LAYOUTS))
def test_launch_layouts_give_the_same_bits(case, mixed, variant, monkeypatch):
    """The Robin walk as separate face, edge and corner launches, the FP64
    smoother with two points a thread, the FP32 smoother as per-colour
    launches (two points or one a thread) instead of cluster-resident, and
    the FP64 coarsest solve in the plain slab layout instead of the balanced
    one give the default launches' u bit for bit, over five cycles (a
    difference of the compiler's fusion between two kernels once showed from
    the third)."""
    import ollipticid_gb300 as og
    P = problem(case)
    out = []
    for alt in (False, True):
        if alt:
            for k, v in LAYOUTS[variant].items():
                monkeypatch.setenv(k, v)
        with og.Elliptic(P) as E:
            E.set_precision(mixed)
            for _ in range(5):
                E.FASN()
            out.append([E.get_field(g) for g in range(len(E.boxes))])
    for g, (a, b) in enumerate(zip(*out)):
        assert np.array_equal(a, b), f"box {g}: max diff {float(np.max(np.abs(a - b))):.3e}"
