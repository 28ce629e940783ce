"""ctypes mirror of include/olgpu.h (the C ABI of libolgpu.so)."""
from __future__ import annotations

import ctypes as C
import os

MAX_BH = 16

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_NAN, ERR_DIVERGED, ERR_TIMEOUT, ERR_GEOMETRY, ERR_NO_DEVICE = range(9)
STOP_REFERENCE, STOP_TOLERANCE, STOP_FIXED, STOP_ERROR = range(4)
PREC_FP64, PREC_MIXED = range(2)

_D16 = C.c_double * MAX_BH


class Problem(C.Structure):
    _fields_ = [
        ("equation", C.c_int), ("numbh", C.c_int),
        ("mp", _D16), ("x", _D16), ("y", _D16), ("z", _D16),
        ("px", _D16), ("py", _D16), ("pz", _D16),
        ("sx", _D16), ("sy", _D16), ("sz", _D16),
        ("n", C.c_int), ("L", C.c_double), ("order", C.c_int), ("levels", C.c_int),
        ("nu1", C.c_int), ("nu2", C.c_int), ("tol", C.c_double),
        ("ps_case", C.c_int), ("ps_phi0", C.c_double), ("ps_r0", C.c_double),
        ("ps_sigma", C.c_double), ("ps_a2", C.c_double), ("boundary", C.c_int), ("method", C.c_int),
    ]


class BoxInfo(C.Structure):
    _fields_ = [
        ("level", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("buf", C.c_int), ("order", C.c_int),
        ("xi", C.c_double), ("yi", C.c_double), ("zi", C.c_double),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double),
        ("xf", C.c_double), ("yf", C.c_double), ("zf", C.c_double),
    ]


class CycleEvent(C.Structure):
    _fields_ = [("level", C.c_int), ("post", C.c_int), ("cycle", C.c_longlong), ("norm", C.c_double)]


class StopRule(C.Structure):
    _fields_ = [("stop", C.c_int), ("max_cycles", C.c_int), ("tol", C.c_double), ("du_tol", C.c_double)]


class Report(C.Structure):
    _fields_ = [
        ("cycles", C.c_int), ("status", C.c_int), ("final_res", C.c_double),
        ("adm", _D16), ("res", C.c_double * 256), ("final_du", C.c_double), ("final_part", C.c_double),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("mem_budget", C.c_longlong), ("max_active", C.c_int), ("precision", C.c_int),
        ("stop", C.c_int), ("max_cycles", C.c_int), ("tol", C.c_double), ("builders", C.c_int),
        ("nu1", C.c_int), ("nu2", C.c_int), ("blocks", C.c_int), ("busy", C.c_int), ("keep_solutions", C.c_int),
        ("du_tol", C.c_double), ("batch_max", C.c_int), ("batch_window", C.c_double),
    ]


class ServerResult(C.Structure):
    _fields_ = [
        ("id", C.c_longlong), ("status", C.c_int), ("cycles", C.c_int), ("final_res", C.c_double),
        ("adm", _D16), ("queue_s", C.c_double), ("latency_s", C.c_double), ("h", C.c_void_p),
        ("final_du", C.c_double),
    ]


class BatchConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("nu1", C.c_int), ("nu2", C.c_int),
                ("blocks", C.c_int)]


class BoxFields(C.Structure):
    _fields_ = [
        ("u", C.c_void_p), ("b", C.c_void_p), ("c", C.c_void_p), ("s", C.c_void_p),
        ("d", C.c_void_p), ("e", C.c_void_p),
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("order", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
    ]


NOALLOC_MAX_SWEEPS = 64

# every exported entry point: name -> (restype, argtypes)
SIGNATURES = {
    "olgpu_problem_defaults": (None, [C.POINTER(Problem)]),
    "olgpu_plan_boxes": (C.c_int, [C.POINTER(Problem), C.POINTER(BoxInfo), C.c_int, C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "olgpu_hierarchy_create": (C.c_int, [C.POINTER(Problem), C.c_int, C.POINTER(C.c_void_p)]),
    "olgpu_hierarchy_destroy": (C.c_int, [C.c_void_p]),
    "olgpu_num_boxes": (C.c_int, [C.c_void_p]),
    "olgpu_num_levels": (C.c_int, [C.c_void_p]),
    "olgpu_mgrid_levels": (C.c_int, [C.c_void_p]),
    "olgpu_box": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(BoxInfo)]),
    "olgpu_storage_order": (C.c_int, [C.POINTER(BoxInfo), C.c_void_p]),
    "olgpu_upload": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_void_p]),
    "olgpu_download": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_void_p]),
    "olgpu_vcycle": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "olgpu_solve": (C.c_int, [C.c_void_p, C.POINTER(StopRule), C.POINTER(Report)]),
    "olgpu_adm_mass": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "olgpu_last_cycle": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "olgpu_approximate_id": (C.c_int, [C.c_void_p, C.c_int]),
    "olgpu_level_norms": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "olgpu_cycle_events": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(CycleEvent),
                                     C.POINTER(C.c_longlong)]),
    "olgpu_interpolate": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p]),
    "olgpu_interpolate_field": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_int,
                                          C.c_void_p]),
    "olgpu_cycle_launch": (C.c_int, [C.c_void_p]),
    "olgpu_cycle_poll": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "olgpu_solve_many": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(StopRule), C.POINTER(Report)]),
    "olgpu_reset": (C.c_int, [C.c_void_p]),
    "olgpu_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "olgpu_set_acceleration": (C.c_int, [C.c_void_p, C.c_int]),
    "olgpu_set_fp64_acceleration": (C.c_int, [C.c_void_p, C.c_int]),
    "olgpu_last_device_ms": (C.c_double, [C.c_void_p]),
    "olgpu_last_coarse_iters": (C.c_int, [C.c_void_p]),
    "olgpu_set_inner_sweeps": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "olgpu_set_smoother_blocks": (C.c_int, [C.c_void_p, C.c_int]),
    "olgpu_kernels_per_cycle": (C.c_int, [C.c_void_p]),
    "olgpu_level_interior_points": (C.c_longlong, [C.c_void_p, C.c_int]),
    "olgpu_time_smoother": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "olgpu_device_pool_bytes": (C.c_int, [C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "olgpu_time_smoother_many": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int,
                                           C.POINTER(C.c_double)]),
    "olgpu_fma_peak": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "olgpu_smooth_box_noalloc": (C.c_int, [C.POINTER(BoxFields), C.c_int, C.POINTER(C.c_double), C.c_void_p]),
    "olgpu_server_config_defaults": (None, [C.POINTER(ServerConfig)]),
    "olgpu_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "olgpu_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(C.c_longlong)]),
    "olgpu_server_poll": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(C.c_int),
                                    C.POINTER(ServerResult)]),
    "olgpu_server_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]),
    "olgpu_server_destroy": (C.c_int, [C.c_void_p]),
    "olgpu_batch_config_defaults": (None, [C.POINTER(BatchConfig)]),
    "olgpu_batch_create": (C.c_int, [C.POINTER(Problem), C.c_int, C.POINTER(BatchConfig), C.POINTER(C.c_void_p)]),
    "olgpu_batch_solve": (C.c_int, [C.c_void_p, C.POINTER(StopRule), C.POINTER(Report)]),
    "olgpu_batch_reset": (C.c_int, [C.c_void_p]),
    "olgpu_batch_member": (C.c_void_p, [C.c_void_p, C.c_int]),
    "olgpu_batch_size": (C.c_int, [C.c_void_p]),
    "olgpu_batch_unions": (C.c_int, [C.c_void_p]),
    "olgpu_batch_kernels_per_cycle": (C.c_int, [C.c_void_p]),
    "olgpu_batch_last_ms": (C.c_double, [C.c_void_p]),
    "olgpu_batch_destroy": (C.c_int, [C.c_void_p]),
    "olgpu_last_error": (C.c_char_p, []),
    "olgpu_version": (C.c_char_p, []),
}

_lib = None


def lib_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libolgpu.so")


def load(build_if_missing: bool = True):
    """Load libolgpu.so; raise if it cannot be built or loaded (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libolgpu.so not found at {path}; run ollipticid_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class OlgpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"olgpu status {status}: {msg}")
        self.status = status


def check(status: int):
    if status != OK:
        raise OlgpuError(status, load(False).olgpu_last_error().decode())
