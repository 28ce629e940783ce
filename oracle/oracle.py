"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle.

The oracle (olliptic_oracle.c) restates the reference's FAS puncture solve on
the CPU, bit for bit.  tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it as the checker; the GPU library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
CLI = os.path.join(HERE, "_build", "oracle_cli")
MAX_BH = 16
_D16 = C.c_double * MAX_BH


class OrcProblem(C.Structure):
    _fields_ = [
        ("equation", C.c_int), ("numbh", C.c_int),
        ("mp", _D16), ("x", _D16), ("y", _D16), ("z", _D16),
        ("px", _D16), ("py", _D16), ("pz", _D16),
        ("sx", _D16), ("sy", _D16), ("sz", _D16),
        ("n", C.c_int), ("L", C.c_double), ("order", C.c_int), ("levels", C.c_int),
        ("nu1", C.c_int), ("nu2", C.c_int), ("tol", C.c_double),
        ("ps_case", C.c_int), ("ps_phi0", C.c_double), ("ps_r0", C.c_double),
        ("ps_sigma", C.c_double), ("ps_a2", C.c_double), ("boundary", C.c_int), ("by_var", C.c_int),
    ]


class OrcBox(C.Structure):
    _fields_ = [("level", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("buf", C.c_int),
                ("order", C.c_int)] + [(n, C.c_double) for n in (
                    "xi", "yi", "zi", "xf", "yf", "zf", "dx", "dy", "dz", "cx", "cy", "cz",
                    "gxi", "gyi", "gzi", "gxf", "gyf", "gzf")]


class OrcEvent(C.Structure):
    _fields_ = [("level", C.c_int), ("post", C.c_int), ("cycle", C.c_long), ("norm", C.c_double)]


_lib = None


def build():
    """Compile the oracle (make -C oracle); no reference sources needed."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "olliptic_oracle.c")):
            build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcProblem)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_create_extra_coarse.restype = C.c_void_p
        L.orc_create_extra_coarse.argtypes = [C.POINTER(OrcProblem)]
        for f in ("orc_num_boxes", "orc_num_levels", "orc_mgrid_levels"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [C.c_void_p]
        L.orc_box.argtypes = [C.c_void_p, C.c_int, C.POINTER(OrcBox)]
        L.orc_get_field.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_void_p]
        L.orc_set_field.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_void_p]
        L.orc_vcycle.restype = C.c_double
        L.orc_vcycle.argtypes = [C.c_void_p]
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        L.orc_solve_wcycle.restype = C.c_int
        L.orc_solve_wcycle.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        L.orc_events.restype = C.c_long
        L.orc_events.argtypes = [C.c_void_p, C.c_long, C.c_long, C.POINTER(OrcEvent)]
        L.orc_set_wcycle_cap.argtypes = [C.c_void_p, C.c_long]
        L.orc_adm.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_approximate_id.argtypes = [C.c_void_p]
        L.orc_interpolate.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_int, C.c_void_p]
        L.orc_set_multicolor.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_coarse_cap.argtypes = [C.c_void_p, C.c_long]
        L.orc_set_wsmooth.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_coarse_omega.argtypes = [C.c_void_p, C.c_double]
        L.orc_set_coarse_rtol.argtypes = [C.c_void_p, C.c_double]
        L.orc_coarse_iters.restype = C.c_long
        L.orc_coarse_iters.argtypes = [C.c_void_p]
        L.orc_level_norm.restype = C.c_double
        L.orc_level_norm.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_set_divergence_source.argtypes = [C.c_void_p] * 4
        L.orc_valid_n.restype = C.c_int
        L.orc_valid_n.argtypes = [C.c_int]
        _lib = L
    return _lib


class Oracle:
    """One CPU hierarchy, driven like the reference's elliptic object."""

    def __init__(self, params: dict, extra_coarse: bool = False):
        L = load()
        p = OrcProblem()
        p.equation = int(params.get("equation", 0))
        mp = list(params["mp"])
        p.numbh = len(mp)
        for name in ("mp", "x", "y", "z", "px", "py", "pz", "sx", "sy", "sz"):
            vals = list(params.get(name, [0.0] * p.numbh))
            arr = getattr(p, name)
            for i in range(p.numbh):
                arr[i] = float(vals[i])
        p.n = int(params["n"]); p.L = float(params["L"]); p.order = int(params["order"])
        p.levels = int(params["levels"]); p.nu1 = int(params.get("nu1", 3)); p.nu2 = int(params.get("nu2", 3))
        p.tol = float(params.get("tol", 1e-8)); p.ps_case = int(params.get("ps_case", 1))
        p.ps_phi0 = float(params.get("ps_phi0", 0.025)); p.ps_r0 = float(params.get("ps_r0", 120.0))
        p.ps_sigma = float(params.get("ps_sigma", 8.0)); p.ps_a2 = float(params.get("ps_a2", 1.0))
        p.boundary = int(params.get("boundary", 0))
        p.by_var = int(params.get("by_var", 0))
        self.numbh = p.numbh
        self._p = p
        self._s = (L.orc_create_extra_coarse if extra_coarse else L.orc_create)(C.byref(p))
        if not self._s:
            raise ValueError("oracle could not build the hierarchy")
        self.L = L
        self.nboxes = L.orc_num_boxes(self._s)
        self.levels = L.orc_num_levels(self._s)
        self.mgrid_levels = L.orc_mgrid_levels(self._s)
        self.boxes = []
        for g in range(self.nboxes):
            b = OrcBox()
            L.orc_box(self._s, g, C.byref(b))
            self.boxes.append(b)

    def close(self):
        if self._s:
            self.L.orc_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, g: int, name: str = "u") -> np.ndarray:
        b = self.boxes[g]
        out = np.empty((b.nz, b.ny, b.nx), dtype=np.float64)
        if self.L.orc_get_field(self._s, g, name.encode(), out.ctypes.data_as(C.c_void_p)) != 0:
            raise KeyError(name)
        return out

    def set_field(self, g: int, name: str, values: np.ndarray):
        arr = np.ascontiguousarray(values, dtype=np.float64)
        self.L.orc_set_field(self._s, g, name.encode(), arr.ctypes.data_as(C.c_void_p))

    def set_multicolor(self, on: int = 1):
        """bit 0: colour the level smoothers, bit 1: colour the coarsest solve"""
        self.L.orc_set_multicolor(self._s, int(on))

    def set_wsmooth(self, on: int = 1):
        self.L.orc_set_wsmooth(self._s, int(on))

    def set_coarse_omega(self, omega: float):
        self.L.orc_set_coarse_omega(self._s, float(omega))

    def set_coarse_rtol(self, rtol: float):
        self.L.orc_set_coarse_rtol(self._s, float(rtol))

    def set_coarse_cap(self, cap: int):
        self.L.orc_set_coarse_cap(self._s, int(cap))

    @property
    def coarse_iters(self) -> int:
        return self.L.orc_coarse_iters(self._s)

    def level_norms(self):
        return [(self.L.orc_level_norm(self._s, l, 0), self.L.orc_level_norm(self._s, l, 1))
                for l in range(self.levels)]

    def vcycle(self) -> float:
        return self.L.orc_vcycle(self._s)

    def solve(self, max_cycles: int = 100000):
        r = C.c_double()
        c = self.L.orc_solve(self._s, max_cycles, C.byref(r))
        return c, r.value

    def solve_wcycle(self, max_cycles: int = 100000):
        r = C.c_double()
        c = self.L.orc_solve_wcycle(self._s, max_cycles, C.byref(r))
        return c, r.value

    def events(self):
        """Every Print_Pre_Cycle / Print_Post_Cycle call so far as
        (level, post, cycle, norm) tuples."""
        n = self.L.orc_events(self._s, 0, 0, None)
        buf = (OrcEvent * max(n, 1))()
        self.L.orc_events(self._s, 0, n, buf)
        return [(e.level, e.post, e.cycle, e.norm) for e in buf[:n]]

    def adm(self):
        out = (C.c_double * MAX_BH)()
        self.L.orc_adm(self._s, out)
        return [out[i] for i in range(self.numbh)]

    def approximate_id(self):
        self.L.orc_approximate_id(self._s)

    def interpolate(self, points, ord: int, box: int = -1, first_level: int = 0) -> np.ndarray:
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.empty(len(pts), dtype=np.float64)
        rc = self.L.orc_interpolate(self._s, int(box), int(first_level), pts.ctypes.data_as(C.c_void_p), len(pts), int(ord),
                                    out.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise ValueError("orc_interpolate: bad argument")
        return out

    def all_u(self):
        return [self.field(g, "u") for g in range(self.nboxes)]

    def fixed_point(self, tol: float = 1e-14, max_cycles: int = 400):
        """Solve with the reference stop rule, then keep cycling until the
        largest change of u over every box is <= tol (or it stalls)."""
        self.solve()
        prev = self.all_u()
        d = np.inf
        for c in range(max_cycles):
            self.vcycle()
            cur = self.all_u()
            d = max(float(np.max(np.abs(a - b))) for a, b in zip(cur, prev))
            prev = cur
            if d <= tol:
                break
        return d


BOWEN_YORK = 5
BY_VARS = ("V1", "V2", "V3", "lambda")


def bowen_york_fixed_point(params: dict, tol: float = 1e-14, max_cycles: int = 400):
    """The Bowen-York system's fixed point (include/elliptic.h:772-803): V1,
    V2, V3 solved one after another, each from its own source (rho0..rho2,
    src/operator.cc:3313-3408), then lambda with Dx V1 + Dy V2 + Dz V3 as its
    source.  Returns ({name: [u of every box]}, {name: last max|du|})."""
    fields, deltas, solved = {}, {}, []
    for v, name in enumerate(BY_VARS):
        o = Oracle(dict(params, equation=BOWEN_YORK, by_var=v))
        if v == 3:
            o.L.orc_set_divergence_source(o._s, *(s._s for s in solved))
        deltas[name] = o.fixed_point(tol, max_cycles)
        fields[name] = o.all_u()
        solved.append(o)
    return fields, deltas
