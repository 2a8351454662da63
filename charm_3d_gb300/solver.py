"""Host-side mirror of the reference's time-step plugin, over the C ABI.

The reference registers ``timestep_single_fn`` / ``get_dt_fn`` and calls
them from ``charm_timesteps`` (reference src/charm_timesteps.c:23-51).
``Solver.step()`` / ``Solver.get_dt()`` are those two calls; ``Forest`` is the
CPU octree (p4est's role) whose flattened arrays are uploaded after each
adapt.  All compute happens in libcharm_gpu.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .case import Case


class MeshArrays:
    """Owned numpy copies of a flattened mesh plus the ctypes view of them."""

    def __init__(self, m: abi.Mesh, hex: abi.Hex | None = None):
        E, F, Fb = m.n_elem, m.n_face, m.n_bface
        self.n_elem, self.n_face, self.n_bface = E, F, Fb
        self.tree_len = tuple(m.tree_len)
        self.center = np.ctypeslib.as_array(m.center, (3 * E,)).reshape(3, E).copy()
        self.level = np.ctypeslib.as_array(m.level, (E,)).copy()
        self.face_elem = np.ctypeslib.as_array(m.face_elem, (2 * F,)).reshape(2, F).copy() if F else np.zeros((2, 0), np.int32)
        self.face_info = np.ctypeslib.as_array(m.face_info, (F,)).copy() if F else np.zeros(0, np.uint8)
        self.bface_elem = np.ctypeslib.as_array(m.bface_elem, (Fb,)).copy() if Fb else np.zeros(0, np.int32)
        self.bface_face = np.ctypeslib.as_array(m.bface_face, (Fb,)).copy() if Fb else np.zeros(0, np.int8)
        self.bface_bnd = np.ctypeslib.as_array(m.bface_bnd, (Fb,)).copy() if Fb else np.zeros(0, np.int8)
        # general hexahedra: corners [8][3][E] (p4est corner order) and the
        # face numbers of both sides of every interior record [2][F]
        self.vertex = self.face_face = None
        if hex is not None:
            self.vertex = np.ctypeslib.as_array(hex.vertex, (24 * E,)).reshape(8, 3, E).copy()
            self.face_face = (np.ctypeslib.as_array(hex.face_face, (2 * F,)).reshape(2, F).copy() if F
                              else np.zeros((2, 0), np.int8))
        self._struct = None

    @property
    def is_hex(self) -> bool:
        return self.vertex is not None

    def hex_struct(self) -> abi.Hex:
        x = abi.Hex()
        self._keep_hex = [np.ascontiguousarray(self.vertex, dtype=np.float64),
                          np.ascontiguousarray(self.face_face, dtype=np.int8)]
        x.vertex = abi.ptr(self._keep_hex[0])
        x.face_face = abi.ptr(self._keep_hex[1], C.c_int8)
        return x

    def struct(self) -> abi.Mesh:
        m = abi.Mesh()
        m.n_elem, m.n_face, m.n_bface = self.n_elem, self.n_face, self.n_bface
        for d in range(3):
            m.tree_len[d] = self.tree_len[d]
        self._keep = [np.ascontiguousarray(a) for a in (self.center, self.level, self.face_elem, self.face_info,
                                                          self.bface_elem, self.bface_face, self.bface_bnd)]
        c, lv, fe, fi, be, bf, bb = self._keep
        m.center = abi.ptr(c)
        m.level = abi.ptr(lv, C.c_int8)
        m.face_elem = abi.ptr(fe, C.c_int32)
        m.face_info = abi.ptr(fi, C.c_uint8)
        m.bface_elem = abi.ptr(be, C.c_int32)
        m.bface_face = abi.ptr(bf, C.c_int8)
        m.bface_bnd = abi.ptr(bb, C.c_int8)
        self._struct = m
        return m


class Forest:
    """The CPU octree (charm_host_forest_* in the C ABI): a brick of cubic
    trees for a Case, or one tree per hexahedron of an unstructured mesh
    (Forest.from_gmsh, Forest.from_hex)."""

    hex = False

    @classmethod
    def from_gmsh(cls, path: str, level: int, bnd_names: list[str]) -> "Forest":
        """Forest over a gmsh 2.x hexahedral mesh; boundary patches bind to
        bnd_names[k] (the configuration's boundary k) by physical name."""
        self = cls.__new__(cls)
        self.lib = abi.load()
        self.h = C.c_void_p()
        self.hex = True
        arr = (C.c_char_p * max(1, len(bnd_names)))(*[n.encode() for n in bnd_names])
        abi.check(self.lib.charm_host_forest_new_gmsh(C.byref(self.h), str(path).encode(), level, len(bnd_names), arr),
                  "charm_host_forest_new_gmsh")
        return self

    @classmethod
    def from_hex(cls, vert: np.ndarray, t2v: np.ndarray, tree_bnd: np.ndarray, level: int) -> "Forest":
        """Forest over hexahedra given by vertices [n][3] and corner lists
        [T][8] (p4est order); tree_bnd [T][6]: boundary index of each tree
        face without a neighbour."""
        self = cls.__new__(cls)
        self.lib = abi.load()
        self.h = C.c_void_p()
        self.hex = True
        v = np.ascontiguousarray(vert, dtype=np.float64)
        t = np.ascontiguousarray(t2v, dtype=np.int32)
        b = np.ascontiguousarray(tree_bnd, dtype=np.int8)
        abi.check(self.lib.charm_host_forest_new_hex(C.byref(self.h), len(v), v.ctypes.data, len(t), t.ctypes.data,
                                                     b.ctypes.data, level), "charm_host_forest_new_hex")
        return self

    def tree_regions(self) -> np.ndarray:
        n = int(self.lib.charm_host_forest_tree_count(self.h))
        r = np.empty(n, np.int32)
        abi.check(self.lib.charm_host_forest_tree_region(self.h, r.ctypes.data), "charm_host_forest_tree_region")
        return r

    def __init__(self, case: Case, level: int | None = None):
        self.lib = abi.load()
        self.h = C.c_void_p()
        nt = np.array(case.brick, np.int32)
        per = np.array(case.periodic, np.int32)
        org = np.array(case.origin, np.float64)
        tl = np.array(case.tree_len, np.float64)
        lv = case.level if level is None else level
        abi.check(self.lib.charm_host_forest_new(C.byref(self.h), nt.ctypes.data, per.ctypes.data, org.ctypes.data,
                                                 tl.ctypes.data, lv), "charm_host_forest_new")
        bnd = np.array(case.bnd_of_side, np.int8)
        abi.check(self.lib.charm_host_forest_set_bnd(self.h, bnd.ctypes.data), "charm_host_forest_set_bnd")

    def __len__(self) -> int:
        return int(self.lib.charm_host_forest_count(self.h))

    def close(self) -> None:
        if self.h:
            self.lib.charm_host_forest_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def flatten(self) -> MeshArrays:
        m = abi.Mesh()
        if self.hex:
            x = abi.Hex()
            abi.check(self.lib.charm_host_forest_flatten_hex(self.h, C.byref(m), C.byref(x)),
                      "charm_host_forest_flatten_hex")
            return MeshArrays(m, x)
        abi.check(self.lib.charm_host_forest_flatten(self.h, C.byref(m)), "charm_host_forest_flatten")
        return MeshArrays(m)

    def adapt(self, flags: np.ndarray, minlevel: int, maxlevel: int) -> int:
        f = np.ascontiguousarray(flags, dtype=np.int8)
        n = C.c_int64()
        abi.check(self.lib.charm_host_forest_adapt(self.h, f.ctypes.data, minlevel, maxlevel, C.byref(n)),
                  "charm_host_forest_adapt")
        return n.value

    def adapt_state(self, grad: np.ndarray, max_err: float, minlevel: int, maxlevel: int, n_comp: int,
                    u: np.ndarray) -> np.ndarray:
        """One adapt (refine / coarsen / balance) carrying the state along; returns the new state."""
        g = np.ascontiguousarray(grad, dtype=np.float64)
        uu = np.ascontiguousarray(u, dtype=np.float64)
        n = C.c_int64()
        abi.check(self.lib.charm_host_forest_adapt_state(self.h, g.ctypes.data, max_err, minlevel, maxlevel, n_comp,
                                                         uu.ctypes.data, C.byref(n)), "charm_host_forest_adapt_state")
        p = C.POINTER(C.c_double)()
        abi.check(self.lib.charm_host_forest_state(self.h, C.byref(p)), "charm_host_forest_state")
        return np.ctypeslib.as_array(p, (4 + n_comp, 4, n.value)).copy()

    def adapt_plan(self, grad: np.ndarray, rho: np.ndarray, max_err: float, minlevel: int,
                   maxlevel: int) -> tuple[int, abi.AdaptPlan]:
        """The adapt of adapt_state without the state: the coarsening criterion
        reads the centre densities rho [E] (Solver.density_means) and the
        projections come back as a plan for Solver.adapt_upload (valid until
        the next adapt of this forest)."""
        g = np.ascontiguousarray(grad, dtype=np.float64)
        r = np.ascontiguousarray(rho, dtype=np.float64)
        n = C.c_int64()
        plan = abi.AdaptPlan()
        abi.check(self.lib.charm_host_forest_adapt_plan(self.h, g.ctypes.data, r.ctypes.data, max_err, minlevel,
                                                        maxlevel, C.byref(n), C.byref(plan)),
                  "charm_host_forest_adapt_plan")
        return n.value, plan

    def adapt_plan_flags(self, flags: np.ndarray, minlevel: int, maxlevel: int) -> tuple[int, abi.AdaptPlan]:
        """adapt_plan driven by flags (+1 refine, -1 coarsening candidate),
        e.g. from Solver.refine_flags_relative."""
        f = np.ascontiguousarray(flags, dtype=np.int8)
        n = C.c_int64()
        plan = abi.AdaptPlan()
        abi.check(self.lib.charm_host_forest_adapt_plan_flags(self.h, f.ctypes.data, minlevel, maxlevel, C.byref(n),
                                                              C.byref(plan)), "charm_host_forest_adapt_plan_flags")
        return n.value, plan

    def write_vtu(self, path: str, fields: np.ndarray, names: list[str]) -> None:
        """Leaves as a VTK XML unstructured grid with cell data `fields` [n][E] named `names`."""
        f = np.ascontiguousarray(fields, dtype=np.float64)
        arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
        abi.check(self.lib.charm_host_forest_write_vtu(self.h, path.encode(), len(names), arr, f.ctypes.data),
                  "charm_host_forest_write_vtu")

    def leaves(self) -> tuple[np.ndarray, np.ndarray]:
        n = len(self)
        q = np.empty((n, 4), np.int32)
        lv = np.empty(n, np.int8)
        abi.check(self.lib.charm_host_forest_leaves(self.h, q.ctypes.data, lv.ctypes.data), "charm_host_forest_leaves")
        return q, lv


class Solver:
    """One GPU solver handle (charm_gpu_* in the C ABI)."""

    def __init__(self, case: Case | abi.Config, device: int = 0):
        self.lib = abi.load()
        self.cfg = case.config() if isinstance(case, Case) else case
        self.h = C.c_void_p()
        abi.check(self.lib.charm_gpu_create(C.byref(self.h), C.byref(self.cfg), device), "charm_gpu_create")
        self.n_var = 4 + self.cfg.n_comp
        self.n_basis = abi.BASIS_P2 if self.cfg.p_order == 2 else abi.BASIS
        self.n_elem = 0
        self.mesh = None

    def close(self) -> None:
        if self.h:
            self.lib.charm_gpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, mesh: MeshArrays) -> None:
        self.mesh = mesh
        s = mesh.struct()
        if mesh.is_hex:
            x = mesh.hex_struct()
            abi.check(self.lib.charm_gpu_upload_mesh_hex(self.h, C.byref(s), C.byref(x)), "charm_gpu_upload_mesh_hex")
        else:
            abi.check(self.lib.charm_gpu_upload_mesh(self.h, C.byref(s)), "charm_gpu_upload_mesh")
        self.n_elem = mesh.n_elem

    def shape(self) -> tuple[int, int, int]:
        return (self.n_var, self.n_basis, self.n_elem)

    def set_state(self, u) -> None:
        if isinstance(u, np.ndarray):
            a = np.ascontiguousarray(u, dtype=np.float64)
            assert a.shape == self.shape(), (a.shape, self.shape())
            abi.check(self.lib.charm_gpu_set_state(self.h, a.ctypes.data, 0), "charm_gpu_set_state")
        else:   # device pointer (int)
            abi.check(self.lib.charm_gpu_set_state(self.h, C.c_void_p(int(u)), 1), "charm_gpu_set_state")

    def get_state(self, out=None) -> np.ndarray:
        if out is not None and not isinstance(out, np.ndarray):
            abi.check(self.lib.charm_gpu_get_state(self.h, C.c_void_p(int(out)), 1), "charm_gpu_get_state")
            return out
        a = out if out is not None else np.empty(self.shape())
        abi.check(self.lib.charm_gpu_get_state(self.h, a.ctypes.data, 0), "charm_gpu_get_state")
        return a

    def step(self, dt: float = 0.0) -> float:
        dto = C.c_double()
        abi.check(self.lib.charm_gpu_step(self.h, dt, C.byref(dto)), "charm_gpu_step")
        return dto.value

    def run(self, nsteps: int, dt: float = 0.0) -> None:
        abi.check(self.lib.charm_gpu_run(self.h, nsteps, dt), "charm_gpu_run")

    def time_run(self, nsteps: int, dt: float = 0.0) -> float:
        """Device time in ms of nsteps, from CUDA events on the solver's stream."""
        ms = C.c_double()
        abi.check(self.lib.charm_gpu_time_run(self.h, nsteps, dt, C.byref(ms)), "charm_gpu_time_run")
        return ms.value

    def get_dt(self) -> float:
        d = C.c_double()
        abi.check(self.lib.charm_gpu_get_dt(self.h, C.byref(d)), "charm_gpu_get_dt")
        return d.value

    def residual(self) -> np.ndarray:
        a = np.empty(self.shape())
        abi.check(self.lib.charm_gpu_residual(self.h, a.ctypes.data, 0), "charm_gpu_residual")
        return a

    def residual_adjoint(self, rbar: np.ndarray) -> np.ndarray:
        """(dR/du)^T rbar at the current state."""
        rb = np.ascontiguousarray(rbar, dtype=np.float64)
        out = np.empty(self.shape())
        abi.check(self.lib.charm_gpu_residual_adjoint(self.h, rb.ctypes.data, out.ctypes.data),
                  "charm_gpu_residual_adjoint")
        return out

    @staticmethod
    def pressure_box(lo, hi) -> abi.Objective:
        obj = abi.Objective()
        obj.kind = abi.OBJ_PRESSURE_BOX
        for k in range(3):
            obj.lo[k], obj.hi[k] = float(lo[k]), float(hi[k])
        return obj

    def objective(self, obj: abi.Objective, grad: bool = False):
        """J of the current state, and dJ/du when grad is set."""
        J = C.c_double()
        g = np.empty(self.shape()) if grad else None
        abi.check(self.lib.charm_gpu_objective(self.h, C.byref(obj), C.byref(J),
                                               g.ctypes.data if grad else None), "charm_gpu_objective")
        return (J.value, g) if grad else J.value

    def adjoint(self, n_steps: int, n_snapshots: int, obj: abi.Objective | None = None,
                dJdu_final: np.ndarray | None = None) -> tuple[np.ndarray, abi.AdjointInfo]:
        """dJ/du(0) through n_steps steps from the current state (which ends at step n_steps)."""
        out = np.empty(self.shape())
        info = abi.AdjointInfo()
        fin = None if dJdu_final is None else np.ascontiguousarray(dJdu_final, dtype=np.float64)
        abi.check(self.lib.charm_gpu_adjoint(self.h, int(n_steps), int(n_snapshots),
                                             C.byref(obj) if obj is not None else None,
                                             fin.ctypes.data if fin is not None else None, out.ctypes.data,
                                             C.byref(info)), "charm_gpu_adjoint")
        return out, info

    def limit(self) -> None:
        abi.check(self.lib.charm_gpu_limit(self.h), "charm_gpu_limit")

    def refine_flags(self, max_err: float) -> tuple[np.ndarray, np.ndarray]:
        """Reference refine criterion per leaf and the density-gradient estimate [3][E]."""
        flags = np.empty(self.n_elem, np.int8)
        grad = np.empty((3, self.n_elem))
        abi.check(self.lib.charm_gpu_refine_flags(self.h, max_err, flags.ctypes.data, grad.ctypes.data),
                  "charm_gpu_refine_flags")
        return flags, grad

    def refine_flags_relative(self, threshold: float, per_cell: bool = True) -> tuple[np.ndarray, np.ndarray]:
        """Flags of the |grad rho| * L / rho criterion (+1 refine, -1 coarsen
        candidate, 0 keep) and the gradient estimate [3][E]."""
        flags = np.empty(self.n_elem, np.int8)
        grad = np.empty((3, self.n_elem))
        abi.check(self.lib.charm_gpu_refine_flags_relative(self.h, threshold, 1 if per_cell else 0, flags.ctypes.data,
                                                           grad.ctypes.data), "charm_gpu_refine_flags_relative")
        return flags, grad

    def cell_fields(self) -> np.ndarray:
        """Cell-centre R, P, E, E_TOT, U, V, W, T and the mass fractions [8 + n_comp][E]."""
        out = np.empty((8 + self.cfg.n_comp, self.n_elem))
        abi.check(self.lib.charm_gpu_cell_fields(self.h, out.ctypes.data), "charm_gpu_cell_fields")
        return out

    def density_means(self) -> np.ndarray:
        """Sum of the species' mean coefficients per leaf (the coarsening criterion's densities)."""
        rho = np.empty(self.n_elem)
        abi.check(self.lib.charm_gpu_density_means(self.h, rho.ctypes.data), "charm_gpu_density_means")
        return rho

    def adapt_upload(self, plan: abi.AdaptPlan, mesh: MeshArrays) -> None:
        """Carry the device state through an adapt plan and upload the adapted mesh."""
        abi.check(self.lib.charm_gpu_adapt_upload(self.h, C.byref(plan), C.byref(mesh.struct())),
                  "charm_gpu_adapt_upload")
        self.n_elem = mesh.n_elem
        self.mesh = mesh

    def refine_flags_adjoint(self, max_err: float) -> tuple[np.ndarray, np.ndarray]:
        """Adjoint-weighted refine flags and the weighted gradient [3][E] (after adjoint())."""
        flags = np.empty(self.n_elem, np.int8)
        grad = np.empty((3, self.n_elem))
        abi.check(self.lib.charm_gpu_refine_flags_adjoint(self.h, max_err, flags.ctypes.data, grad.ctypes.data),
                  "charm_gpu_refine_flags_adjoint")
        return flags, grad

    def sync(self, timeout_s: float = 600.0) -> None:
        abi.check(self.lib.charm_gpu_sync(self.h, timeout_s), "charm_gpu_sync")

    def sync_status(self, timeout_s: float = 600.0) -> int:
        return int(self.lib.charm_gpu_sync(self.h, timeout_s))

    def set_stream(self, stream: int | None) -> None:
        abi.check(self.lib.charm_gpu_set_stream(self.h, C.c_void_p(stream or 0)), "charm_gpu_set_stream")

    def set_timing(self, on: bool) -> None:
        abi.check(self.lib.charm_gpu_set_timing(self.h, 1 if on else 0), "charm_gpu_set_timing")

    def kernel_stats(self) -> tuple[np.ndarray, np.ndarray]:
        n = np.zeros(4, np.int64)
        ms = np.zeros(4, np.float64)
        abi.check(self.lib.charm_gpu_kernel_stats(self.h, n.ctypes.data_as(C.POINTER(C.c_int64)),
                                                  ms.ctypes.data_as(C.POINTER(C.c_double))), "charm_gpu_kernel_stats")
        return n, ms

    def reset_stats(self) -> None:
        abi.check(self.lib.charm_gpu_reset_stats(self.h), "charm_gpu_reset_stats")


def point_flux(case: Case | abi.Config, U2: np.ndarray, normals: np.ndarray) -> np.ndarray:
    """Numerical flux of the case's flux function between state pairs
    U2[n][2][V] (conserved) along unit normals[n][3], on the current device
    (charm_gpu_point_flux)."""
    lib = abi.load()
    cfg = case.config() if isinstance(case, Case) else case
    U = np.ascontiguousarray(U2, dtype=np.float64)
    nn = np.ascontiguousarray(normals, dtype=np.float64)
    n = U.shape[0]
    assert U.shape == (n, 2, 4 + cfg.n_comp) and nn.shape == (n, 3)
    q = np.empty((n, 4 + cfg.n_comp))
    abi.check(lib.charm_gpu_point_flux(C.byref(cfg), n, U.ctypes.data, nn.ctypes.data, q.ctypes.data),
              "charm_gpu_point_flux")
    return q


def build_case(case: Case, device: int = 0, precision: str | None = None):
    """Forest + flattened mesh + solver with the case's initial state uploaded."""
    if precision is not None:
        case.precision = precision
    forest = Forest(case)
    mesh = forest.flatten()
    solver = Solver(case, device)
    solver.upload(mesh)
    u0 = case.initial_state(mesh.center)
    solver.set_state(u0)
    return forest, mesh, solver, u0
