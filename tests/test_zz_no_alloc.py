"""charm_gpu_residual_static: the residual entry point that allocates no device memory.

Some callers cannot call cudaMalloc, or let a library call it for them: their
device memory belongs to another allocator (a framework's memory pool), or
they run where allocation is not allowed.  This entry point takes only device
buffers the caller owns (here: torch tensors) and keeps its intermediate
face projections in a static device array inside the library.  It is checked
through the C ABI against the regular entry point charm_gpu_residual, within
the parity tolerance (FP64: 1e-12; the mixed form's FP32 residual: 1e-6),
on two calls in a row (the second call must not see anything the first left
in the shared array), for one and two species, conforming and hanging
meshes.  A warm call leaves the free device memory unchanged; invalid states
and face records are reported as the regular entry points report them.
"""
import ctypes as C

import numpy as np
import pytest

from charm_3d_gb300 import abi
from charm_3d_gb300.solver import Forest, Solver

from .common import hanging_forest, rel_max, small_case

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _device_mesh(mesh):
    """The flattened mesh copied into caller-owned device tensors."""
    import torch
    arrs = {k: torch.from_numpy(np.ascontiguousarray(getattr(mesh, k))).cuda()
            for k in ("center", "level", "face_elem", "face_info", "bface_elem", "bface_face", "bface_bnd")}
    m = abi.Mesh()
    m.n_elem, m.n_face, m.n_bface = mesh.n_elem, mesh.n_face, mesh.n_bface
    for d in range(3):
        m.tree_len[d] = mesh.tree_len[d]
    m.center = C.cast(C.c_void_p(arrs["center"].data_ptr()), C.POINTER(C.c_double))
    m.level = C.cast(C.c_void_p(arrs["level"].data_ptr()), C.POINTER(C.c_int8))
    m.face_elem = C.cast(C.c_void_p(arrs["face_elem"].data_ptr()), C.POINTER(C.c_int32))
    m.face_info = C.cast(C.c_void_p(arrs["face_info"].data_ptr()), C.POINTER(C.c_uint8))
    m.bface_elem = C.cast(C.c_void_p(arrs["bface_elem"].data_ptr()), C.POINTER(C.c_int32))
    m.bface_face = C.cast(C.c_void_p(arrs["bface_face"].data_ptr()), C.POINTER(C.c_int8))
    m.bface_bnd = C.cast(C.c_void_p(arrs["bface_bnd"].data_ptr()), C.POINTER(C.c_int8))
    return m, arrs


MIXED_TOL = 1e-6   # the mixed form's FP32 residual (tests/test_gpu_parity.py)


def _static(lib, cfg, dmesh, u_d, r_d, stream=None):
    return lib.charm_gpu_residual_static(C.byref(cfg), C.byref(dmesh), C.c_void_p(u_d.data_ptr()),
                                         C.c_void_p(r_d.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("kind,flux,hang,precision", [("random", "HLLC", True, "FP64"), ("walls", "LF", False, "FP64"),
                                                      ("mix2", "HLLC", True, "FP64"), ("random", "HLLC", True, "MIXED"),
                                                      ("mix2", "LF", False, "MIXED")])
def test_static_residual_matches_regular_entry_point_on_two_calls(kind, flux, hang, precision):
    import torch
    lib = abi.load()
    case = small_case(kind, flux, "BJ", level=3)
    case.precision = precision
    tol = TOL if precision == "FP64" else MIXED_TOL
    forest = hanging_forest(case)[0] if hang else Forest(case)
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    dmesh, keep = _device_mesh(mesh)
    cfg = case.config()
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (3, 4):
        case.seed = seed
        u = case.initial_state(mesh.center)
        gpu.set_state(u)
        want = gpu.residual()
        u_d = torch.from_numpy(u).cuda()
        r_d = torch.full_like(u_d, float("nan"))
        rc = lib.charm_gpu_residual_static(C.byref(cfg), C.byref(dmesh), C.c_void_p(u_d.data_ptr()),
                                           C.c_void_p(r_d.data_ptr()), C.c_void_p(stream))
        assert rc == abi.OK, lib.charm_gpu_last_error()
        got = r_d.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_max(got, want) < tol
    gpu.close()


def test_static_residual_warm_call_allocates_nothing():
    """After a first call on the device, a call changes the free device memory by nothing."""
    import torch
    lib = abi.load()
    case = small_case("random", "HLLC", "NONE", level=4)
    mesh = hanging_forest(case)[0].flatten()
    dmesh, keep = _device_mesh(mesh)
    cfg = case.config()
    u_d = torch.from_numpy(case.initial_state(mesh.center)).cuda()
    r_d = torch.empty_like(u_d)
    stream = torch.cuda.current_stream().cuda_stream
    assert _static(lib, cfg, dmesh, u_d, r_d, stream) == abi.OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _static(lib, cfg, dmesh, u_d, r_d, stream) == abi.OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_static_residual_reports_non_positive_pressure_like_the_handle():
    """A cell whose energy leaves no internal energy: ENEGATIVE from the static
    entry point, and from the regular residual at its next sync."""
    import torch
    lib = abi.load()
    case = small_case("random", "LF", "NONE", level=2)
    mesh = Forest(case).flatten()
    u = case.initial_state(mesh.center)
    u[3, :, 5] = 0.0          # rho E = 0 with a non-zero velocity: p < 0 at every Gauss point
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u)
    res = np.empty_like(u)
    assert lib.charm_gpu_residual(gpu.h, res.ctypes.data, 0) == abi.OK
    assert gpu.sync_status(60.0) == abi.ENEGATIVE
    gpu.close()
    dmesh, keep = _device_mesh(mesh)
    cfg = case.config()
    u_d = torch.from_numpy(u).cuda()
    r_d = torch.empty_like(u_d)
    assert _static(lib, cfg, dmesh, u_d, r_d) == abi.ENEGATIVE
    # the next call with a valid state is clean (the error word starts at zero)
    u_d = torch.from_numpy(case.initial_state(mesh.center)).cuda()
    assert _static(lib, cfg, dmesh, u_d, r_d) == abi.OK


@pytest.mark.parametrize("corrupt", ["element past the end", "mortar out of order", "one face twice"])
def test_static_residual_rejects_bad_face_records(corrupt):
    import torch
    lib = abi.load()
    case = small_case("random", "HLLC", "NONE", level=2)
    mesh = hanging_forest(case)[0].flatten()
    kind = (mesh.face_info >> 2) & 3
    conf, mort = int(np.flatnonzero(kind == 0)[0]), int(np.flatnonzero(kind != 0)[0])
    if corrupt == "element past the end":
        mesh.face_elem[1, conf] = mesh.n_elem
    elif corrupt == "mortar out of order":
        mesh.face_info[[mort, mort + 1]] = mesh.face_info[[mort + 1, mort]]
    else:
        mesh.bface_elem[1], mesh.bface_face[1] = mesh.bface_elem[0], mesh.bface_face[0]
    dmesh, keep = _device_mesh(mesh)
    cfg = case.config()
    u_d = torch.from_numpy(case.initial_state(mesh.center)).cuda()
    r_d = torch.full_like(u_d, float("nan"))
    assert _static(lib, cfg, dmesh, u_d, r_d) == abi.EINVAL
    assert torch.isnan(r_d).all()


def test_static_residual_rejects_meshes_beyond_its_array():
    import torch
    lib = abi.load()
    case = small_case("random", "HLLC", "NONE", level=6)        # 262,144 elements
    mesh = Forest(case).flatten()
    dmesh, keep = _device_mesh(mesh)
    u_d = torch.zeros((case.n_var, 4, mesh.n_elem), dtype=torch.float64, device="cuda")
    r_d = torch.zeros_like(u_d)
    cfg = case.config()
    rc = lib.charm_gpu_residual_static(C.byref(cfg), C.byref(dmesh), C.c_void_p(u_d.data_ptr()),
                                       C.c_void_p(r_d.data_ptr()), None)
    assert rc == abi.EINVAL
    assert b"too large" in lib.charm_gpu_last_error()
