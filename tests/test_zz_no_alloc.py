"""charm_gpu_residual_static: the residual entry point that allocates no device memory.

Some callers cannot call cudaMalloc, or let a library call it for them: their
device memory belongs to another allocator (a framework's memory pool), or
they run where allocation is not allowed.  This entry point takes only device
buffers the caller owns (here: torch tensors) and keeps its intermediate
face projections in a static device array inside the library.  It is checked
through the C ABI against the regular entry point charm_gpu_residual, within
the FP64 parity tolerance, on two calls in a row (the second call must not
see anything the first left in the shared array).
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


@pytest.mark.parametrize("kind,flux,hang", [("random", "HLLC", True), ("walls", "LF", False)])
def test_static_residual_matches_regular_entry_point_on_two_calls(kind, flux, hang):
    import torch
    lib = abi.load()
    case = small_case(kind, flux, "BJ", level=3)
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
        assert rel_max(got, want) < TOL
    gpu.close()


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
