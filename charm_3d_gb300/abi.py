"""ctypes mirror of include/charm_gpu.h and the loader of libcharm_gpu.so.

The library is the product: every GPU computation goes through these C
entry points.  There is no Python or CPU fallback; if the shared library is
missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libcharm_gpu.so")

MAX_COMP = 8
MAX_CP = 8
MAX_BND = 16
BASIS = 4
BASIS_P2 = 10

# status codes
OK, EINVAL, ENOMEM, ECUDA, ENONFINITE, ENEGATIVE, EHLLC, ETIMEDOUT, ESTATE, ENOTSUP = range(10)
STATUS_NAMES = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ENONFINITE", 5: "ENEGATIVE", 6: "EHLLC",
                7: "ETIMEDOUT", 8: "ESTATE", 9: "ENOTSUP"}

MODEL = {"EULER": 0, "NS": 1}
FLUX = {"LF": 0, "GODUNOV": 1, "HLLC": 2, "CD": 3}
LIMITER = {"NONE": 0, "BJ": 1}
EOS = {"IDEAL": 0, "MIX": 1}
PRECISION = {"FP64": 0, "MIXED": 1, "DW": 2}
DT_MODE = {"TAU": 0, "CFL": 1}
BND = {"BOUND_INLET": 0, "BOUND_OUTLET": 1, "BOUND_WALL_SLIP": 2, "BOUND_WALL_NO_SLIP": 3, "BOUND_MASS_FLOW": 4}
CP_TYPE = {"CONST": 0, "POLYNOM": 1}
LAW = {"CONST": 0, "SATHERLAND": 1}


class Comp(C.Structure):
    _fields_ = [("m", C.c_double), ("ml0", C.c_double), ("kp0", C.c_double), ("t0", C.c_double),
                ("ts", C.c_double), ("sig", C.c_double), ("ek", C.c_double), ("h0", C.c_double),
                ("cp_type", C.c_int), ("kp_type", C.c_int), ("ml_type", C.c_int), ("n_cp", C.c_int),
                ("cp", C.c_double * MAX_CP)]


class Bnd(C.Structure):
    _fields_ = [("type", C.c_int), ("params", C.c_double * (7 + MAX_COMP))]


MAX_REACT = 8


class Reaction(C.Structure):
    _fields_ = [("left", C.c_int32 * 3), ("right", C.c_int32 * 3), ("a", C.c_double), ("e", C.c_double),
                ("n", C.c_double)]


class Config(C.Structure):
    _fields_ = [("model", C.c_int), ("flux", C.c_int), ("limiter", C.c_int), ("eos", C.c_int),
                ("precision", C.c_int), ("dt_mode", C.c_int), ("n_comp", C.c_int),
                ("comp", Comp * MAX_COMP), ("n_bnd", C.c_int), ("bnd", Bnd * MAX_BND),
                ("grav", C.c_double * 3), ("tau", C.c_double), ("cfl", C.c_double), ("t_ref", C.c_double),
                ("use_visc", C.c_int), ("check_every", C.c_int), ("use_diff", C.c_int), ("n_react", C.c_int),
                ("react", Reaction * MAX_REACT), ("p_order", C.c_int)]


MAX_REG = 16


class CaseRegion(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("id", C.c_int), ("material_id", C.c_int), ("v", C.c_double * 3),
                ("t", C.c_double), ("p", C.c_double), ("grav", C.c_double * 3), ("c", C.c_double * MAX_COMP)]


class CaseFile(C.Structure):
    """charm_case_t: task.yaml read by charm_case_read_yaml."""
    _fields_ = [("cfg", Config), ("tmax", C.c_double), ("max_error", C.c_double), ("refine_period", C.c_int),
                ("repartition_period", C.c_int), ("min_level", C.c_int), ("max_level", C.c_int),
                ("file_output_step", C.c_int), ("log_output_step", C.c_int), ("mesh_type", C.c_char * 32),
                ("mesh_name", C.c_char * 256), ("bnd_name", (C.c_char * 64) * MAX_BND),
                ("comp_name", (C.c_char * 64) * MAX_COMP), ("comp_id", C.c_int * MAX_COMP), ("n_reg", C.c_int),
                ("reg", CaseRegion * MAX_REG)]


class Objective(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32), ("lo", C.c_double * 3), ("hi", C.c_double * 3)]


class AdjointInfo(C.Structure):
    _fields_ = [("J", C.c_double), ("forward_steps", C.c_int64), ("reverse_steps", C.c_int64),
                ("snapshots", C.c_int32), ("pad", C.c_int32), ("seconds", C.c_double)]


OBJ_PRESSURE_BOX = 1


class Mesh(C.Structure):
    _fields_ = [("n_elem", C.c_int64), ("center", C.POINTER(C.c_double)), ("level", C.POINTER(C.c_int8)),
                ("tree_len", C.c_double * 3), ("n_face", C.c_int64), ("face_elem", C.POINTER(C.c_int32)),
                ("face_info", C.POINTER(C.c_uint8)), ("n_bface", C.c_int64),
                ("bface_elem", C.POINTER(C.c_int32)), ("bface_face", C.POINTER(C.c_int8)),
                ("bface_bnd", C.POINTER(C.c_int8))]


class Hex(C.Structure):
    """charm_gpu_hex_t: corners and face numbers of general hexahedra."""
    _fields_ = [("vertex", C.POINTER(C.c_double)), ("face_face", C.POINTER(C.c_int8))]


class AdaptPlan(C.Structure):
    """charm_gpu_adapt_plan_t: the projection passes of one adapt."""
    _fields_ = [("n_pass", C.c_int32), ("pad", C.c_int32), ("n_in", C.c_int64),
                ("n_out", C.POINTER(C.c_int64)), ("map", C.POINTER(C.POINTER(C.c_int32)))]


# Every entry point declared in include/charm_gpu.h: (name, restype, argtypes).
_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)
SIGNATURES = [
    ("charm_gpu_version", C.c_char_p, []),
    ("charm_gpu_last_error", C.c_char_p, []),
    ("charm_gpu_create", C.c_int, [C.POINTER(_P), C.POINTER(Config), C.c_int]),
    ("charm_gpu_destroy", C.c_int, [_P]),
    ("charm_gpu_upload_mesh", C.c_int, [_P, C.POINTER(Mesh)]),
    ("charm_gpu_upload_mesh_hex", C.c_int, [_P, C.POINTER(Mesh), C.POINTER(Hex)]),
    ("charm_gpu_set_state", C.c_int, [_P, _P, C.c_int]),
    ("charm_gpu_get_state", C.c_int, [_P, _P, C.c_int]),
    ("charm_gpu_step", C.c_int, [_P, C.c_double, _DP]),
    ("charm_gpu_run", C.c_int, [_P, C.c_int, C.c_double]),
    ("charm_gpu_get_dt", C.c_int, [_P, _DP]),
    ("charm_gpu_residual", C.c_int, [_P, _P, C.c_int]),
    ("charm_gpu_limit", C.c_int, [_P]),
    ("charm_gpu_refine_flags", C.c_int, [_P, C.c_double, _P, _P]),
    ("charm_gpu_set_stream", C.c_int, [_P, _P]),
    ("charm_gpu_sync", C.c_int, [_P, C.c_double]),
    ("charm_gpu_set_timing", C.c_int, [_P, C.c_int]),
    ("charm_gpu_kernel_stats", C.c_int, [_P, _I64P, _DP]),
    ("charm_gpu_reset_stats", C.c_int, [_P]),
    ("charm_gpu_time_run", C.c_int, [_P, C.c_int, C.c_double, _DP]),
    ("charm_gpu_probe_peak", C.c_int, [C.c_int, C.c_int, _DP]),
    ("charm_gpu_abi_sizes", C.c_int, [_I64P]),
    ("charm_gpu_residual_static", C.c_int, [C.POINTER(Config), C.POINTER(Mesh), _P, _P, _P]),
    ("charm_gpu_point_flux", C.c_int, [C.POINTER(Config), C.c_int64, _P, _P, _P]),
    ("charm_gpu_math_check", C.c_int, [C.c_int, C.c_int64, _P, _P, _P]),
    ("charm_gpu_p2_interp", C.c_int, [C.c_int, C.c_int64, C.c_int, _P, _P, _P, C.c_int, _DP]),
    ("charm_gpu_dims", C.c_int, [_P, _I64P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("charm_gpu_objective", C.c_int, [_P, C.POINTER(Objective), _DP, _P]),
    ("charm_gpu_residual_adjoint", C.c_int, [_P, _P, _P]),
    ("charm_gpu_adjoint", C.c_int, [_P, C.c_int, C.c_int, C.POINTER(Objective), _P, _P, C.POINTER(AdjointInfo)]),
    ("charm_gpu_refine_flags_adjoint", C.c_int, [_P, C.c_double, _P, _P]),
    ("charm_gpu_density_means", C.c_int, [_P, _P]),
    ("charm_gpu_refine_flags_relative", C.c_int, [_P, C.c_double, C.c_int, _P, _P]),
    ("charm_gpu_cell_fields", C.c_int, [_P, _P]),
    ("charm_gpu_adapt_upload", C.c_int, [_P, C.POINTER(AdaptPlan), C.POINTER(Mesh)]),
    ("charm_case_read_yaml", C.c_int, [C.c_char_p, C.POINTER(CaseFile)]),
    ("charm_case_parse_yaml", C.c_int, [C.c_char_p, C.POINTER(CaseFile)]),
    ("charm_host_forest_new", C.c_int, [C.POINTER(_P), _P, _P, _P, _P, C.c_int]),
    ("charm_host_forest_free", C.c_int, [_P]),
    ("charm_host_forest_count", C.c_int64, [_P]),
    ("charm_host_forest_set_bnd", C.c_int, [_P, _P]),
    ("charm_host_forest_adapt", C.c_int, [_P, _P, C.c_int, C.c_int, _I64P]),
    ("charm_host_forest_adapt_state", C.c_int, [_P, _P, C.c_double, C.c_int, C.c_int, C.c_int, _P, _I64P]),
    ("charm_host_forest_state", C.c_int, [_P, C.POINTER(_DP)]),
    ("charm_host_forest_adapt_plan", C.c_int, [_P, _P, _P, C.c_double, C.c_int, C.c_int, _I64P,
                                               C.POINTER(AdaptPlan)]),
    ("charm_host_forest_adapt_plan_flags", C.c_int, [_P, _P, C.c_int, C.c_int, _I64P, C.POINTER(AdaptPlan)]),
    ("charm_host_forest_flatten", C.c_int, [_P, C.POINTER(Mesh)]),
    ("charm_host_forest_leaves", C.c_int, [_P, _P, _P]),
    ("charm_host_forest_write_vtu", C.c_int, [_P, C.c_char_p, C.c_int, C.POINTER(C.c_char_p), _P]),
    ("charm_host_forest_new_hex", C.c_int, [C.POINTER(_P), C.c_int32, _P, C.c_int32, _P, _P, C.c_int]),
    ("charm_host_forest_new_gmsh", C.c_int, [C.POINTER(_P), C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_char_p)]),
    ("charm_host_forest_tree_count", C.c_int, [_P]),
    ("charm_host_forest_tree_region", C.c_int, [_P, _P]),
    ("charm_host_forest_flatten_hex", C.c_int, [_P, C.POINTER(Mesh), C.POINTER(Hex)]),
]

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libcharm_gpu.so (building it first if this checkout has not)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _build
        _build.build()
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class CharmGpuError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = ""
        if _lib is not None:
            raw = _lib.charm_gpu_last_error()
            msg = raw.decode() if raw else ""
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)} ({msg})")
        self.code = code


def check(code: int, where: str) -> None:
    if code != OK:
        raise CharmGpuError(code, where)


def ptr(a: np.ndarray, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


def read_case_yaml(path: str | None = None, text: str | None = None) -> CaseFile:
    """task.yaml (a file, or its text) read by the library's case reader."""
    lib = load()
    out = CaseFile()
    if text is not None:
        check(lib.charm_case_parse_yaml(text.encode(), C.byref(out)), "charm_case_parse_yaml")
    else:
        check(lib.charm_case_read_yaml(str(path).encode(), C.byref(out)), "charm_case_read_yaml")
    return out
