"""ctypes wrapper of the reference build (oracle/_ref/libcharm_ref*.so).  Oracle only.

Available only where the reference checkout exists (the libraries are built
from its sources by oracle/build_ref.py); tests skip otherwise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref


class Region(C.Structure):
    _fields_ = [("v", C.c_double * 3), ("t", C.c_double), ("p", C.c_double), ("c", C.c_double * 8)]


def available() -> bool:
    return build_ref.reference_root() is not None


_libs: dict[str, C.CDLL] = {}


def load(variant: str = "ref") -> C.CDLL:
    if variant not in _libs:
        paths = build_ref.build()
        lib = C.CDLL(paths[variant], mode=C.RTLD_LOCAL)
        lib.ref_setup.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int]
        lib.ref_setup_hex.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int]
        lib.ref_count.restype = C.c_int64
        lib.ref_set_state.argtypes = [C.c_void_p]
        lib.ref_get_state.argtypes = [C.c_void_p]
        lib.ref_run.argtypes = [C.c_int, C.c_void_p]
        lib.ref_residual.argtypes = [C.c_void_p]
        lib.ref_geometry.argtypes = [C.c_void_p]
        lib.ref_faces_count.restype = C.c_int64
        lib.ref_faces_copy.argtypes = [C.c_void_p]
        lib.ref_leaves.argtypes = [C.c_void_p]
        lib.ref_adapt.restype = C.c_int64
        lib.ref_grad.argtypes = [C.c_void_p]
        lib.ref_point_flux.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_rim.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
        lib.ref_cell_fields.argtypes = [C.c_void_p]
        lib.ref_refine_flags.argtypes = [C.c_void_p, C.c_int]
        lib.ref_refine_flags.restype = C.c_int64
        if variant == "plugin":
            lib.ref_plugin_flatten.argtypes = [C.c_void_p]
            lib.ref_plugin_flatten_hex.argtypes = [C.c_void_p, C.c_void_p]
            lib.ref_plugin_config.argtypes = [C.c_int, C.c_void_p]
            lib.ref_plugin_use_gpu.argtypes = [C.c_int]
        _libs[variant] = lib
    return _libs[variant]


class RefSolver:
    """The reference's own time step on a brick case, or with hexmesh =
    (vertices, tree corners, tree-face boundaries) on an unstructured
    hexahedral mesh (one at a time per variant)."""

    def __init__(self, case, variant: str = "ref", hexmesh=None):
        self.lib = load(variant)
        self.case = case
        self.cfg = case.config()
        reg = Region()
        r = case.ref_region()
        for k in range(3):
            reg.v[k] = r["v"][k]
        reg.t, reg.p = r["t"], r["p"]
        for k, v in enumerate(r["c"]):
            reg.c[k] = v
        self.n_var = 4 + case.n_comp
        if hexmesh is not None:
            vert, t2v, tb = hexmesh
            self._keep = [np.ascontiguousarray(vert, np.float64), np.ascontiguousarray(t2v, np.int32),
                          np.ascontiguousarray(tb, np.int8)]
            v, t, b = self._keep
            rc = self.lib.ref_setup_hex(C.addressof(self.cfg), len(v), v.ctypes.data, len(t), t.ctypes.data,
                                        b.ctypes.data, case.level, C.addressof(reg), case.max_err, case.min_level,
                                        case.max_level, case.refine_period)
            if rc:
                raise RuntimeError(f"ref_setup_hex failed: {rc}")
            return
        self._keep = [np.array(case.brick, np.int32), np.array(case.periodic, np.int32),
                      np.array(case.origin, np.float64), np.array(case.tree_len, np.float64),
                      np.array(case.bnd_of_side, np.int8)]
        b, p, o, t, s = self._keep
        rc = self.lib.ref_setup(C.addressof(self.cfg), b.ctypes.data, p.ctypes.data, o.ctypes.data, t.ctypes.data,
                                case.level, s.ctypes.data, C.addressof(reg), case.max_err, case.min_level,
                                case.max_level, case.refine_period)
        if rc:
            raise RuntimeError(f"ref_setup failed: {rc}")
        self.n_var = 4 + case.n_comp

    @property
    def n_elem(self) -> int:
        return int(self.lib.ref_count())

    def shape(self):
        return (self.n_var, 4, self.n_elem)

    def set_state(self, u: np.ndarray) -> None:
        a = np.ascontiguousarray(u, dtype=np.float64)
        assert a.shape == self.shape()
        self.lib.ref_set_state(a.ctypes.data)

    def get_state(self) -> np.ndarray:
        a = np.empty(self.shape())
        self.lib.ref_get_state(a.ctypes.data)
        return a

    def run(self, nsteps: int) -> float:
        dt = C.c_double()
        self.lib.ref_run(nsteps, C.byref(dt))
        return dt.value

    def cell_fields(self) -> np.ndarray:
        """[8 + n_comp][E]: R, P, E, E_TOT, U, V, W, T, C_i at the cell centres (the output's fields)."""
        a = np.empty((8 + self.case.n_comp, self.n_elem))
        self.lib.ref_cell_fields(a.ctypes.data)
        return a

    def residual(self) -> np.ndarray:
        a = np.empty(self.shape())
        self.lib.ref_residual(a.ctypes.data)
        return a

    def limit(self) -> None:
        self.lib.ref_limit()

    def geometry(self) -> np.ndarray:
        a = np.empty((self.n_elem, 29))
        self.lib.ref_geometry(a.ctypes.data)
        return a

    def faces(self) -> np.ndarray:
        n = self.lib.ref_faces_count()
        a = np.empty((n, 13), np.int64)
        self.lib.ref_faces_copy(a.ctypes.data)
        return a

    def leaves(self) -> np.ndarray:
        a = np.empty((self.n_elem, 5), np.int32)
        self.lib.ref_leaves(a.ctypes.data)
        return a

    def adapt(self) -> int:
        return int(self.lib.ref_adapt())

    def grad(self) -> np.ndarray:
        a = np.empty((self.n_elem, 3))
        self.lib.ref_grad(a.ctypes.data)
        return a

    def refine_flags(self, flags: np.ndarray, maxlevel: int) -> int:
        f = np.ascontiguousarray(flags, dtype=np.int8)
        return int(self.lib.ref_refine_flags(f.ctypes.data, maxlevel))

    def plugin_flatten(self):
        """Flattened mesh as the GPU model plugin builds it from p4est_iterate."""
        from charm_3d_gb300 import abi
        from charm_3d_gb300.solver import MeshArrays
        m = abi.Mesh()
        rc = self.lib.ref_plugin_flatten(C.addressof(m))
        if rc:
            raise RuntimeError(f"charm_model_gpu_flatten: {rc}")
        return MeshArrays(m)

    def plugin_flatten_hex(self):
        """(needs general hexahedra, mesh in that form) as the plugin builds it."""
        from charm_3d_gb300 import abi
        from charm_3d_gb300.solver import MeshArrays
        m = abi.Mesh()
        x = abi.Hex()
        rc = self.lib.ref_plugin_flatten_hex(C.addressof(m), C.addressof(x))
        if rc < 0:
            raise RuntimeError("charm_model_gpu_flatten failed")
        return bool(rc), MeshArrays(m, x)

    def plugin_config(self, precision: int = 0):
        from charm_3d_gb300 import abi
        cfg = abi.Config()
        rc = self.lib.ref_plugin_config(precision, C.addressof(cfg))
        if rc:
            raise RuntimeError(f"charm_model_gpu_config: {rc}")
        return cfg

    def plugin_use_gpu(self, precision: int = 0) -> None:
        """Step through the GPU model plugin from now on (charm_model_gpu_init)."""
        self.lib.ref_plugin_use_gpu(precision)

    def plugin_finish(self) -> int:
        """The plugin's state back into the quadrants, its handle released;
        the plugin's status (0 or a CHARM_GPU_* code)."""
        return int(self.lib.ref_plugin_finish())

    def point_flux(self, prim2, n) -> np.ndarray:
        p = np.ascontiguousarray(prim2, dtype=np.float64)
        nn = np.ascontiguousarray(n, dtype=np.float64)
        q = np.zeros(4 + self.case.n_comp)
        self.lib.ref_point_flux(p.ctypes.data, nn.ctypes.data, q.ctypes.data)
        return q


def rim(inputs: np.ndarray) -> np.ndarray:
    """The reference's rim_orig on rows (rL pL uL vL wL rR pR uR vR wR gam) -> rows (r e p u v w)."""
    a = np.ascontiguousarray(inputs, dtype=np.float64).reshape(-1, 11)
    out = np.empty((a.shape[0], 6))
    load("ref").ref_rim(a.shape[0], a.ctypes.data, out.ctypes.data)
    return out
