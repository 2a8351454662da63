"""ctypes wrapper of the CPU restatement (oracle/charm_oracle.c).  Oracle only."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_oracle

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(build_oracle.build())
        lib.oracle_new.restype = C.c_void_p
        lib.oracle_new.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_new_hex.restype = C.c_void_p
        lib.oracle_new_hex.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_free.argtypes = [C.c_void_p]
        for name in ("oracle_set_state", "oracle_get_state", "oracle_residual"):
            getattr(lib, name).argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_limit.argtypes = [C.c_void_p]
        lib.oracle_step.argtypes = [C.c_void_p, C.c_double]
        lib.oracle_run.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.oracle_point_flux.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_point_flux_cons.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_point_bflux_cons.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_point_vflux.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_amr_grad.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_rim.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
        lib.oracle_cfl_dt.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_hex_project.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


class Port:
    """The oracle on one flattened mesh (charm_3d_gb300.solver.MeshArrays)."""

    def __init__(self, cfg, mesh):
        self.lib = load()
        self.mesh = mesh
        self._m = mesh.struct()
        self.cfg = cfg
        if getattr(mesh, "is_hex", False):   # general hexahedra: geometry from the corners
            self._x = mesh.hex_struct()
            self.h = self.lib.oracle_new_hex(C.addressof(cfg), C.addressof(self._m), C.addressof(self._x))
        else:
            self.h = self.lib.oracle_new(C.addressof(cfg), C.addressof(self._m))
        if not self.h:
            raise MemoryError("oracle_new failed (or a general hexahedron with a non-positive Jacobian)")
        self.shape = (4 + cfg.n_comp, 10 if cfg.p_order == 2 else 4, mesh.n_elem)

    def close(self):
        if self.h:
            self.lib.oracle_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, u: np.ndarray) -> None:
        a = np.ascontiguousarray(u, dtype=np.float64)
        assert a.shape == self.shape
        self.lib.oracle_set_state(self.h, a.ctypes.data)

    def get_state(self) -> np.ndarray:
        a = np.empty(self.shape)
        self.lib.oracle_get_state(self.h, a.ctypes.data)
        return a

    def residual(self) -> np.ndarray:
        a = np.empty(self.shape)
        self.lib.oracle_residual(self.h, a.ctypes.data)
        return a

    def limit(self) -> None:
        self.lib.oracle_limit(self.h)

    def step(self, dt: float) -> None:
        self.lib.oracle_step(self.h, dt)

    def run(self, nsteps: int, dt: float) -> None:
        self.lib.oracle_run(self.h, nsteps, dt)

    def cfl_dt(self) -> float:
        """The reference's CFL step of the current state (min with TAU)."""
        d = C.c_double(0.0)
        self.lib.oracle_cfl_dt(self.h, C.byref(d))
        return d.value

    def amr_grad(self) -> np.ndarray:
        g = np.empty((3, self.mesh.n_elem))
        self.lib.oracle_amr_grad(self.h, g.ctypes.data)
        return g

    def point_flux_cons(self, U2, n) -> np.ndarray:
        """Numerical flux between two conserved states U2[2][V] along n."""
        U = np.ascontiguousarray(U2, dtype=np.float64)
        nn = np.ascontiguousarray(n, dtype=np.float64)
        q = np.zeros(4 + self.cfg.n_comp)
        self.lib.oracle_point_flux_cons(self.h, U.ctypes.data, nn.ctypes.data, q.ctypes.data)
        return q

    def point_bflux_cons(self, bid, U, n) -> np.ndarray:
        """Boundary flux of conserved state U through boundary bid, outward normal n."""
        Uc = np.ascontiguousarray(U, dtype=np.float64)
        nn = np.ascontiguousarray(n, dtype=np.float64)
        q = np.zeros(4 + self.cfg.n_comp)
        self.lib.oracle_point_bflux_cons(self.h, int(bid), Uc.ctypes.data, nn.ctypes.data, q.ctypes.data)
        return q

    def point_vflux(self, U) -> np.ndarray:
        """Volume fluxes F[3][V] of conserved state U."""
        Uc = np.ascontiguousarray(U, dtype=np.float64)
        F = np.zeros((3, 4 + self.cfg.n_comp))
        self.lib.oracle_point_vflux(self.h, Uc.ctypes.data, F.ctypes.data)
        return F

    def point_flux(self, prim2, n) -> np.ndarray:
        p = np.ascontiguousarray(prim2, dtype=np.float64)
        nn = np.ascontiguousarray(n, dtype=np.float64)
        q = np.zeros(4 + self.cfg.n_comp)
        self.lib.oracle_point_flux(self.h, p.ctypes.data, nn.ctypes.data, q.ctypes.data)
        return q


def rim(inputs: np.ndarray) -> np.ndarray:
    """The oracle's exact Riemann solver on rows (rL pL uL vL wL rR pR uR vR wR gam)
    -> rows (r e p u v w)."""
    a = np.ascontiguousarray(inputs, dtype=np.float64).reshape(-1, 11)
    out = np.empty((a.shape[0], 6))
    load().oracle_rim(a.shape[0], a.ctypes.data, out.ctypes.data)
    return out


def hex_project(cfg, parent_corners: np.ndarray, child_corners: np.ndarray, down: bool, src: np.ndarray) -> np.ndarray:
    """The reference's charm_replace_quads on one family of general
    hexahedra (oracle_hex_project): corners [8][3] and [8][8][3]; down: the
    children [8][V][4] from the parent [V][4], else the parent from the
    children."""
    lib = load()
    V = 4 + cfg.n_comp
    vp = np.ascontiguousarray(parent_corners, dtype=np.float64)
    vc = np.ascontiguousarray(child_corners, dtype=np.float64)
    a = np.ascontiguousarray(src, dtype=np.float64)
    out = np.empty((8, V, 4) if down else (V, 4))
    if lib.oracle_hex_project(C.addressof(cfg), vp.ctypes.data, vc.ctypes.data, 1 if down else 0, a.ctypes.data,
                              out.ctypes.data):
        raise ValueError("non-positive Jacobian")
    return out
