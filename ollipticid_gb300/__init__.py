"""ollipticid_gb300 -- GB300-native FAS multigrid solve of the puncture
Hamiltonian constraint on nested mesh-refinement boxes.

Python host mirror of the reference's elliptic/multigrid surface
(WuShichao/OllipticID include/elliptic.h, include/multigrid.h) over the C ABI
of libolgpu.so (include/olgpu.h).  All numerical work runs in CUDA kernels on
the GPU; there is no CPU path.  If the library cannot be built or loaded, or
no GPU is present, constructing an `Elliptic` raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, List, Sequence

import numpy as np

from . import _abi
from ._abi import OlgpuError, check

__all__ = ["Problem", "Elliptic", "parse_olliptic_args", "OlgpuError", "FIELDS", "smooth_box_noalloc",
           "solve_many"]

FIELDS = ("u", "b", "c", "d", "e", "rho", "r", "w", "ww", "v")


# the equations on the FAS path: the puncture constraint, with a scalar
# field, the reference's test equations (the Gaussian test, a known answer;
# Boundary-test; Multibox-test) and the Bowen-York momentum-constraint test
# (four unknowns V1, V2, V3, lambda: BY_VARS)
EQUATIONS = {"Punctures": 0, "Punctures_scalar_field": 1, "Poisson": 2, "Boundary-test": 3, "Multibox-test": 4,
             "Bowen-York": 5}
BY_VARS = ("V1", "V2", "V3", "lambda")
# the outer boundary conditions (-B): Robin, and Dirichlet, the reference's
# default when -B is not given
BOUNDARIES = {"Robin": 0, "Dirichlet": 1}
# the cycles of -m (elliptic::Set_Method): V-cycles, and W-cycles, where every
# level repeats until its own norm meets the tolerance
METHODS = {"Vcycle": 0, "Wcycle": 1}


@dataclass
class Problem:
    """The Olliptic.x parameters of a puncture problem (src/interface.cc:73-273)."""
    equation: str = "Punctures"          # or "Punctures_scalar_field", "Poisson" (the Gaussian test)
    mp: List[float] = field(default_factory=lambda: [0.0])
    x: List[float] = field(default_factory=lambda: [0.0])
    y: List[float] = field(default_factory=lambda: [0.0])
    z: List[float] = field(default_factory=lambda: [0.0])
    px: List[float] = field(default_factory=lambda: [0.0])
    py: List[float] = field(default_factory=lambda: [0.0])
    pz: List[float] = field(default_factory=lambda: [0.0])
    sx: List[float] = field(default_factory=lambda: [0.0])
    sy: List[float] = field(default_factory=lambda: [0.0])
    sz: List[float] = field(default_factory=lambda: [0.0])
    n: int = 30
    L: float = 2.0
    order: int = 4
    levels: int = 1
    nu1: int = 3
    nu2: int = 3
    tol: float = 1e-8
    ps_case: int = 1
    ps_phi0: float = 0.025
    ps_r0: float = 120.0
    ps_sigma: float = 8.0
    ps_a2: float = 1.0
    boundary: str = "Robin"              # or "Dirichlet" (the reference's default without -B)
    method: str = "Vcycle"               # or "Wcycle"

    @property
    def numbh(self) -> int:
        return len(self.mp)

    def to_c(self) -> _abi.Problem:
        p = _abi.Problem()
        p.equation = EQUATIONS[self.equation]
        p.numbh = self.numbh
        if not 1 <= p.numbh <= _abi.MAX_BH:
            raise ValueError("NumBH must be in 1..16")
        for name in ("mp", "x", "y", "z", "px", "py", "pz", "sx", "sy", "sz"):
            vals = list(getattr(self, name)) + [0.0] * _abi.MAX_BH
            arr = getattr(p, name)
            for i in range(_abi.MAX_BH):
                arr[i] = float(vals[i]) if i < p.numbh else 0.0
        for name in ("n", "order", "levels", "nu1", "nu2", "ps_case"):
            setattr(p, name, int(getattr(self, name)))
        for name in ("L", "tol", "ps_phi0", "ps_r0", "ps_sigma", "ps_a2"):
            setattr(p, name, float(getattr(self, name)))
        p.boundary = BOUNDARIES[self.boundary]
        p.method = METHODS[self.method]
        return p

    def oracle_dict(self) -> dict:
        d = {k: getattr(self, k) for k in ("mp", "x", "y", "z", "px", "py", "pz", "sx", "sy", "sz", "n", "L",
                                           "order", "levels", "nu1", "nu2", "tol", "ps_case", "ps_phi0", "ps_r0",
                                           "ps_sigma", "ps_a2")}
        d["equation"] = EQUATIONS[self.equation]
        d["boundary"] = BOUNDARIES[self.boundary]
        return d


def parse_olliptic_args(argv: Sequence[str]) -> Problem:
    """Olliptic.x command line -> Problem.  Flags outside the puncture FAS path
    are accepted and ignored, as the reference ignores unknown flags."""
    a = list(argv)
    kv = {}
    for i in range(len(a) - 1):
        kv.setdefault(a[i], a[i + 1])

    def get(keys, conv, default):
        for k in keys:
            if k in kv:
                return conv(kv[k])
        return default

    eq = get(["-eq", "--equation"], str, "Punctures")
    if eq not in EQUATIONS:
        raise ValueError(f"equation {eq!r} is not on the puncture FAS path")
    bc = get(["-B", "--boundary"], str, "Dirichlet")   # interface.cc:272
    if bc not in BOUNDARIES:
        raise ValueError(f"boundary {bc!r} is not on the GPU path")
    me = get(["-m", "--method"], str, "Vcycle")        # interface.cc:259, 1333-1354: unknown = Vcycle
    if me in ("Gauss-Seidel", "Full-Multigrid"):
        raise ValueError(f"method {me!r} is not on the GPU path")
    nb = get(["-NumBH", "--num-bh"], int, 1)
    # AppPuncture's hierarchy is the V-cycle's; Elliptic.ApproximateID runs it
    P = Problem(equation=eq, boundary=bc, method="Wcycle" if me == "Wcycle" else "Vcycle")
    for name, flag in (("mp", "-bhmp"), ("x", "-bhx"), ("y", "-bhy"), ("z", "-bhz"), ("px", "-bhpx"),
                       ("py", "-bhpy"), ("pz", "-bhpz"), ("sx", "-bhsx"), ("sy", "-bhsy"), ("sz", "-bhsz")):
        setattr(P, name, [get([f"{flag}{i + 1}"], float, 0.0) for i in range(nb)])
    P.n = get(["-N", "-n"], int, 30)
    P.L = get(["-L", "--length"], float, 2.0)
    P.order = get(["-O", "--order"], int, 4)
    P.levels = get(["-l", "--levels"], int, 1)
    P.nu1 = get(["-nu1", "--pre-smooth"], int, 3)
    P.nu2 = get(["-nu2", "--post-smooth"], int, 3)
    P.tol = get(["-s", "--tolerance"], float, 1e-8)
    P.ps_case = get(["-psc", "-ps_case"], int, 1)
    P.ps_phi0 = get(["-phi0", "--phi0_sf"], float, 0.025)
    P.ps_r0 = get(["-r0", "--radius_sf_r0"], float, 120.0)
    P.ps_sigma = get(["-sigma", "--sigma_sf"], float, 8.0)
    P.ps_a2 = get(["-a2", "--a2_sf"], float, 1.0)
    return P


@dataclass
class Box:
    level: int
    n: tuple
    buf: int
    order: int
    origin: tuple
    d: tuple
    center: tuple


class Elliptic:
    """Device-resident hierarchy of one puncture problem (elliptic::elliptic,
    src/elliptic.cc:30-221) with the reference's solve entry points."""

    def __init__(self, problem: Problem, device: int = 0):
        self.lib = _abi.load()
        self.problem = problem
        self._cp = problem.to_c()
        h = C.c_void_p()
        check(self.lib.olgpu_hierarchy_create(C.byref(self._cp), int(device), C.byref(h)))
        self._h = h
        self.levels = self.lib.olgpu_num_levels(h)
        self.mgrid_levels = self.lib.olgpu_mgrid_levels(h)
        self.boxes: List[Box] = []
        for g in range(self.lib.olgpu_num_boxes(h)):
            bi = _abi.BoxInfo()
            check(self.lib.olgpu_box(h, g, C.byref(bi)))
            self.boxes.append(Box(bi.level, (bi.nx, bi.ny, bi.nz), bi.buf, bi.order, (bi.xi, bi.yi, bi.zi),
                                  (bi.dx, bi.dy, bi.dz), (bi.cx, bi.cy, bi.cz)))
        self.last_report = None

    # -- lifecycle ----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.lib.olgpu_hierarchy_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- geometry -----------------------------------------------------------
    def Get_num_dom(self, level: int) -> int:
        return sum(1 for b in self.boxes if b.level == level)

    def box_index(self, level: int, ibox: int) -> int:
        return [g for g, b in enumerate(self.boxes) if b.level == level][ibox]

    # -- fields -------------------------------------------------------------
    def get_field(self, box: int, name: str = "u", out: Optional[np.ndarray] = None) -> np.ndarray:
        """A box's field as a (nz, ny, nx) array; `out` (C-contiguous float64
        of that shape, e.g. in pinned memory) receives it if given."""
        nx, ny, nz = self.boxes[box].n
        if out is None:
            out = np.empty((nz, ny, nx), dtype=np.float64)
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != nx * ny * nz:
            raise ValueError("out must be a C-contiguous float64 array of the box's size")
        check(self.lib.olgpu_download(self._h, box, name.encode(), out.ctypes.data_as(C.c_void_p)))
        return out

    def set_field(self, box: int, name: str, values: np.ndarray):
        nx, ny, nz = self.boxes[box].n
        arr = np.ascontiguousarray(values, dtype=np.float64).reshape(nz, ny, nx)
        check(self.lib.olgpu_upload(self._h, box, name.encode(), arr.ctypes.data_as(C.c_void_p)))

    def Get_ffunction(self, level: int, ibox: int, name: str = "u") -> np.ndarray:
        return self.get_field(self.box_index(level, ibox), name)

    # -- solve --------------------------------------------------------------
    def FASN(self) -> float:
        """One V-cycle from the finest level (elliptic::FASN)."""
        r = C.c_double()
        check(self.lib.olgpu_vcycle(self._h, C.byref(r)))
        return r.value

    def Solve(self, stop: int = _abi.STOP_REFERENCE, max_cycles: int = 100000, tol: float = 0.0,
              du_tol: float = 0.0) -> "_abi.Report":
        """elliptic::Solve -> Vcycle or Wcycle (the problem's method) with the
        reference stop rule by default.  STOP_ERROR also waits for the
        cycle's largest change of u to be <= du_tol (0: tol)."""
        rule = _abi.StopRule(stop, max_cycles, tol, du_tol)
        rep = _abi.Report()
        st = self.lib.olgpu_solve(self._h, C.byref(rule), C.byref(rep))
        self.last_report = rep
        check(st)
        return rep

    def set_precision(self, mixed: bool):
        """FP64 throughout (False) or FP32 correction cycles around FP64 (True)."""
        check(self.lib.olgpu_set_precision(self._h, _abi.PREC_MIXED if mixed else _abi.PREC_FP64))

    def set_inner_sweeps(self, nu1: int, nu2: int):
        """Pre-/post-smoothing sweeps of the FP32 correction cycle (mixed precision)."""
        check(self.lib.olgpu_set_inner_sweeps(self._h, int(nu1), int(nu2)))

    def set_smoother_blocks(self, max_blocks: int):
        """Largest cluster (8..16 blocks, or 0: per-colour launches) of the FP32 smoother."""
        check(self.lib.olgpu_set_smoother_blocks(self._h, int(max_blocks)))

    def set_acceleration(self, depth: int):
        """Anderson history depth of the mixed outer iteration (0 = off, 1..4)."""
        check(self.lib.olgpu_set_acceleration(self._h, int(depth)))

    def set_fp64_acceleration(self, depth: int):
        """Anderson history depth of the plain FP64 cycle (0 = the reference's
        iteration, 1..4), FP64 throughout; the fixed point is unchanged."""
        check(self.lib.olgpu_set_fp64_acceleration(self._h, int(depth)))

    def cycle_launch(self):
        """Enqueue one V-cycle without waiting (see cycle_poll)."""
        check(self.lib.olgpu_cycle_launch(self._h))

    def last_cycle(self):
        """(residual part, largest change of u on the fixed points) of the
        last finished cycle (olgpu_last_cycle)."""
        r, d = C.c_double(), C.c_double()
        check(self.lib.olgpu_last_cycle(self._h, C.byref(r), C.byref(d)))
        return r.value, d.value

    def cycle_poll(self, wait: bool = False):
        """(done, norm) of the last launched cycle."""
        done, r = C.c_int(), C.c_double()
        check(self.lib.olgpu_cycle_poll(self._h, int(wait), C.byref(done), C.byref(r)))
        return bool(done.value), r.value

    def reset(self):
        check(self.lib.olgpu_reset(self._h))

    def ApproximateID(self, as_guess: bool = True):
        """u = the perturbative puncture solution everywhere (elliptic::
        ApproximateID); a starting guess that leaves the fixed point as it is
        (as_guess=False: the formula exactly as the reference evaluates it)."""
        check(self.lib.olgpu_approximate_id(self._h, 1 if as_guess else 0))

    @property
    def ADM_mass(self) -> List[float]:
        out = (C.c_double * _abi.MAX_BH)()
        check(self.lib.olgpu_adm_mass(self._h, out))
        return [out[i] for i in range(self.problem.numbh)]

    def level_norms(self, cycle: int):
        """(pre, post) smoother norms per level of one cycle of the last solve
        (the reference's Loo[l] lines; level 0: the coarsest solve)."""
        pre = np.empty(self.levels, dtype=np.float64)
        post = np.empty(self.levels, dtype=np.float64)
        check(self.lib.olgpu_level_norms(self._h, int(cycle), pre.ctypes.data_as(C.POINTER(C.c_double)),
                                         post.ctypes.data_as(C.POINTER(C.c_double))))
        return pre, post

    def cycle_events(self):
        """Every Print_Pre_Cycle / Print_Post_Cycle call of the last solve as
        (level, post, cycle, norm) tuples, in the reference's order (level 0:
        the coarsest solve; Loo.gp holds the (cycle, norm) of the post = 0
        calls)."""
        total = C.c_longlong()
        check(self.lib.olgpu_cycle_events(self._h, 0, 0, None, C.byref(total)))
        buf = (_abi.CycleEvent * max(total.value, 1))()
        check(self.lib.olgpu_cycle_events(self._h, 0, total.value, buf, C.byref(total)))
        return [(e.level, e.post, e.cycle, e.norm) for e in buf[:total.value]]

    def interpolate(self, points, ord: Optional[int] = None, box: int = -1, first_level: int = 0,
                    field: str = "u") -> np.ndarray:
        """u at (npts, 3) points, as the reference prints it (Print_Interpol_1D
        / _2D with box=-1: the finest box whose interior holds each point, NaN
        outside the largest box; ffunction::Print_1D with box >= 0).  ord+1
        Lagrange nodes per axis, default order + 1 like the reference's
        printout.  first_level: with box=-1, only boxes of that level and
        finer take part (mgrid_levels for the analytic method's printout).
        field: any field get_field reads (Bowen-York's V1, V2, V3, lambda)."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.empty(len(pts), dtype=np.float64)
        k = self.problem.order + 1 if ord is None else int(ord)
        check(self.lib.olgpu_interpolate_field(self._h, field.encode(), int(box), int(first_level),
                                               pts.ctypes.data_as(C.c_void_p), len(pts), k,
                                               out.ctypes.data_as(C.c_void_p)))
        return out

    @property
    def last_device_ms(self) -> float:
        return self.lib.olgpu_last_device_ms(self._h)

    @property
    def kernels_per_cycle(self) -> int:
        return self.lib.olgpu_kernels_per_cycle(self._h)

    @property
    def last_coarse_iters(self) -> int:
        """Iterations of the coarsest-level solve in the last finished cycle."""
        return self.lib.olgpu_last_coarse_iters(self._h)

    def interior_points(self, level: int) -> int:
        return int(self.lib.olgpu_level_interior_points(self._h, level))

    def time_smoother(self, level: int, sweeps: int):
        """(device ms, kernel launches) of `sweeps` smoother sweeps on a level."""
        ms = C.c_double()
        n = C.c_int()
        check(self.lib.olgpu_time_smoother(self._h, level, sweeps, C.byref(ms), C.byref(n)))
        return ms.value, n.value


def smooth_box_noalloc(u: int, b: int, c: int, s: int, n, order: int, d, sweeps: int,
                       dfield: int = 0, efield: int = 0, stream: int = 0) -> List[float]:
    """Multicolour smoother sweeps on one caller-owned box, without any device
    allocation by the library (olgpu_smooth_box_noalloc).  u, b, c, s (and
    the scalar-field d, e) are device addresses of nx*ny*nz doubles; n is
    (nx, ny, nz), d the spacing (dx, dy, dz).  Returns the per-sweep residual
    norms.  For callers that own all device memory themselves."""
    lib = _abi.load()
    f = _abi.BoxFields(u, b, c, s, dfield or None, efield or None, int(n[0]), int(n[1]), int(n[2]), int(order),
                       float(d[0]), float(d[1]), float(d[2]))
    norms = (C.c_double * max(1, int(sweeps)))()
    check(lib.olgpu_smooth_box_noalloc(C.byref(f), int(sweeps), norms, C.c_void_p(stream or None)))
    return [norms[i] for i in range(int(sweeps))]


class Batch:
    """Uneven puncture solves stepped together (olgpu_batch_*): each FASN
    step of a level is one launch over the boxes of every solve at that level
    (solves grouped into unions with their levels aligned from the finest);
    a solve that meets its stop rule drops out of the launches.  Each result
    is the problem's solo result bit for bit."""

    def __init__(self, problems: Sequence[Problem], mixed: bool = True, inner_sweeps=None, blocks: int = -1,
                 device: int = 0):
        self.lib = _abi.load()
        self.problems = list(problems)
        arr = (_abi.Problem * len(self.problems))(*[p.to_c() for p in self.problems])
        cfg = _abi.BatchConfig()
        self.lib.olgpu_batch_config_defaults(C.byref(cfg))
        cfg.device = int(device)
        cfg.precision = _abi.PREC_MIXED if mixed else _abi.PREC_FP64
        if inner_sweeps:
            cfg.nu1, cfg.nu2 = int(inner_sweeps[0]), int(inner_sweeps[1])
        cfg.blocks = int(blocks)
        b = C.c_void_p()
        check(self.lib.olgpu_batch_create(arr, len(self.problems), C.byref(cfg), C.byref(b)))
        self._b = b
        self.last_reports = None

    def close(self):
        if getattr(self, "_b", None):
            self.lib.olgpu_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.problems)

    def solve(self, stop: int = _abi.STOP_REFERENCE, max_cycles: int = 100000, tol: float = 0.0,
              du_tol: float = 0.0, raise_on_error: bool = True) -> List["_abi.Report"]:
        rule = _abi.StopRule(stop, max_cycles, tol, du_tol)
        reps = (_abi.Report * len(self.problems))()
        st = self.lib.olgpu_batch_solve(self._b, C.byref(rule), reps)
        self.last_reports = list(reps)
        if raise_on_error or st not in (_abi.OK, _abi.ERR_NAN, _abi.ERR_DIVERGED):
            check(st)
        return list(reps)

    def reset(self):
        check(self.lib.olgpu_batch_reset(self._b))

    def _member(self, i: int):
        h = self.lib.olgpu_batch_member(self._b, int(i))
        if not h:
            raise IndexError(i)
        return C.c_void_p(h)

    def boxes(self, i: int):
        h = self._member(i)
        out = []
        for g in range(self.lib.olgpu_num_boxes(h)):
            bi = _abi.BoxInfo()
            check(self.lib.olgpu_box(h, g, C.byref(bi)))
            out.append(bi)
        return out

    def mgrid_levels(self, i: int) -> int:
        return self.lib.olgpu_mgrid_levels(self._member(i))

    def get_field(self, i: int, box: int, name: str = "u") -> np.ndarray:
        h = self._member(i)
        bi = _abi.BoxInfo()
        check(self.lib.olgpu_box(h, box, C.byref(bi)))
        out = np.empty((bi.nz, bi.ny, bi.nx), dtype=np.float64)
        check(self.lib.olgpu_download(h, box, name.encode(), out.ctypes.data_as(C.c_void_p)))
        return out

    def all_u(self, i: int) -> List[np.ndarray]:
        return [self.get_field(i, g) for g in range(self.lib.olgpu_num_boxes(self._member(i)))]

    def ADM_mass(self, i: int) -> List[float]:
        out = (C.c_double * _abi.MAX_BH)()
        check(self.lib.olgpu_adm_mass(self._member(i), out))
        return [out[j] for j in range(self.problems[i].numbh)]

    @property
    def unions(self) -> int:
        return self.lib.olgpu_batch_unions(self._b)

    @property
    def kernels_per_cycle(self) -> int:
        return self.lib.olgpu_batch_kernels_per_cycle(self._b)

    @property
    def last_ms(self) -> float:
        return self.lib.olgpu_batch_last_ms(self._b)


def device_pool_bytes(device: int = 0):
    """(reserved, used) bytes of the library's device-memory pool
    (olgpu_device_pool_bytes)."""
    lib = _abi.load()
    r, u = C.c_longlong(), C.c_longlong()
    check(lib.olgpu_device_pool_bytes(int(device), C.byref(r), C.byref(u)))
    return r.value, u.value


def time_smoother_many(solvers: Sequence[Elliptic], level: int, sweeps: int) -> float:
    """Device ms of `sweeps` smoother sweeps on one level of every solver at
    once, each on its own stream (olgpu_time_smoother_many)."""
    lib = _abi.load()
    hs = (C.c_void_p * len(solvers))(*[E._h.value for E in solvers])
    ms = C.c_double()
    check(lib.olgpu_time_smoother_many(hs, len(solvers), level, sweeps, C.byref(ms)))
    return ms.value


def fma_peak(fp64: bool = True, iters: int = 0) -> float:
    """Measured FMA throughput of the current device in TFLOP/s (FP64 or
    FP32), the instruction roofline of the stencil kernels
    (olgpu_fma_peak)."""
    lib = _abi.load()
    out = C.c_double()
    n = iters or (4096 if fp64 else 65536)
    check(lib.olgpu_fma_peak(_abi.PREC_FP64 if fp64 else _abi.PREC_MIXED, int(n), C.byref(out)))
    return out.value


def solve_many(solvers: Sequence["Elliptic"], stop: int = _abi.STOP_REFERENCE, max_cycles: int = 100000,
               tol: float = 0.0, du_tol: float = 0.0, raise_on_error: bool = True) -> List["_abi.Report"]:
    """Solve several problems concurrently on the GPU (olgpu_solve_many).
    With raise_on_error False a failed solve does not raise: each report's
    `status` tells how its problem ended."""
    lib = _abi.load()
    n = len(solvers)
    hs = (C.c_void_p * n)(*[s._h.value if isinstance(s._h, C.c_void_p) else s._h for s in solvers])
    reps = (_abi.Report * n)()
    rule = _abi.StopRule(stop, max_cycles, tol, du_tol)
    st = lib.olgpu_solve_many(hs, n, C.byref(rule), reps)
    for s, r in zip(solvers, reps):
        s.last_report = r
    if raise_on_error or st not in (_abi.OK, _abi.ERR_NAN, _abi.ERR_DIVERGED):
        check(st)
    return list(reps)
