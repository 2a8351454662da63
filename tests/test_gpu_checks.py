"""Parts of the GPU path that the step parity tests do not reach on their own.

- The device flux functions point by point against the reference's own
  fluxes (tests/golden/point_fluxes.npz, made from the reference build):
  LF, HLLC, CD, and Godunov through the reference's exact Riemann solver
  rim_orig (src/charm_fluxes.c:8-180).  Bar: 1e-12 relative (FP64); the
  mixed form's FP32 flux 1e-5.
- The CFL step (warp-shuffle reduction) against the oracle's restatement of
  the reference's CFL formula (src/models/ns/charm_model.c:21-36, 50-59).
- The bounded wait: charm_gpu_sync with no time left reports
  CHARM_GPU_ETIMEDOUT while a run is still on the GPU, and the run then
  completes with the same state as an unhurried one.
- Corrupted face records passed to charm_gpu_upload_mesh return
  CHARM_GPU_EINVAL and leave the handle's mesh and state usable.
- The flux kernels' FP64 reciprocal and quotient (hardware seed + Newton
  steps) against IEEE division: within 1 and 2 ulp.
"""
import copy
import os

import numpy as np
import pytest

from charm_3d_gb300 import abi
from charm_3d_gb300.solver import Forest, Solver, point_flux
from oracle.port import Port

from .common import hanging_forest, rel_l2, small_case
from .golden_cases import GOLDEN

pytestmark = pytest.mark.gpu


def _cons(case, prim):
    """Conserved states of primitive rows (r u v w p) for the case's single-species ideal gas."""
    _, gam = case.gas_constants()
    r, u, v, w, p = (prim[..., k] for k in range(5))
    e = p / ((gam - 1.0) * r)
    return np.stack([r * u, r * v, r * w, r * (e + 0.5 * (u * u + v * v + w * w)), r], axis=-1)


@pytest.mark.parametrize("flux", ["LF", "HLLC", "CD", "GODUNOV"])
@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_point_fluxes_match_reference(flux, precision):
    d = np.load(os.path.join(GOLDEN, "point_fluxes.npz"))
    case = small_case("random", flux, "NONE", level=1)
    case.precision = precision
    prim2 = d["prim2"]
    q = point_flux(case, _cons(case, prim2), d["normals"])
    want = d[flux]
    tol = 1e-12 if precision == "FP64" else 1e-5
    scale = np.abs(want).max(axis=1, keepdims=True)
    assert (np.abs(q - want) <= tol * scale).all(), np.abs(q - want).max()


def test_exact_riemann_solver_matches_reference():
    """Godunov flux along +x on the wide rim_orig input set: the device's
    exact solver against the reference's (flux assembled from its output)."""
    d = np.load(os.path.join(GOLDEN, "point_fluxes.npz"))
    rin, rout = d["rim_in"], d["rim_out"]
    case = small_case("random", "GODUNOV", "NONE", level=1)
    prim = np.stack([rin[:, [0, 2, 3, 4, 1]], rin[:, [5, 7, 8, 9, 6]]], axis=1)   # (r u v w p) per side
    n = np.tile([1.0, 0.0, 0.0], (rin.shape[0], 1))
    q = point_flux(case, _cons(case, prim), n)
    ri, ei, pi, uu = rout[:, 0], rout[:, 1], rout[:, 2], rout[:, 3:]
    qr = ri * uu[:, 0]
    want = np.stack([qr * uu[:, 0] + pi, qr * uu[:, 1], qr * uu[:, 2],
                     (ri * (ei + 0.5 * (uu * uu).sum(axis=1)) + pi) * uu[:, 0], qr], axis=1)
    scale = np.abs(want).max(axis=1, keepdims=True)
    assert (np.abs(q - want) <= 1e-11 * scale).all(), np.abs(q - want).max()


@pytest.mark.parametrize("kind,hanging", [("random", False), ("vortex", False), ("mix2", False), ("random", True)])
def test_cfl_dt_matches_oracle(kind, hanging):
    case = small_case(kind, "HLLC", "NONE", level=3)
    case.dt_mode = "CFL"
    case.cfl = 0.3
    forest = hanging_forest(case)[0] if hanging else Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    for tau in (1.0, 1e-9):   # the reduction starts from TAU, as the reference's
        case.tau = tau
        gpu = Solver(case)
        gpu.upload(mesh)
        gpu.set_state(u0)
        port = Port(case.config(), mesh)
        port.set_state(u0)
        want = port.cfl_dt()
        assert abs(gpu.get_dt() - want) <= 1e-14 * want
        if tau == 1e-9:
            assert want == tau


@pytest.mark.parametrize("model,lim", [("NS", "NONE"), ("NS", "BJ"), ("EULER", "NONE"), ("EULER", "BJ")])
def test_cfl_step_matches_oracle(model, lim):
    """Steps in CFL mode: each step takes the CFL step of its own start state.
    The first comes from the CFL kernel, the next ones from the reduction
    fused into the last stage's cell or limiter kernel of the step before."""
    case = small_case("random", "HLLC", lim, level=3, model=model)
    case.dt_mode = "CFL"
    case.cfl = 0.05
    case.tau = 1.0
    mesh = hanging_forest(case)[0].flatten()
    u0 = case.initial_state(mesh.center)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.reset_stats()
    port = Port(case.config(), mesh)
    port.set_state(u0)
    for _ in range(4):
        dt = port.cfl_dt()
        port.step(dt)
        got = gpu.step(0.0)
        assert abs(got - dt) <= 1e-14 * dt
    gpu.sync()
    assert rel_l2(gpu.get_state(), port.get_state()) < 1e-12
    n, _ = gpu.kernel_stats()
    assert n[3] == 1      # one CFL kernel launch (the first step); the rest fused
    # a new state starts over with the CFL kernel
    gpu.set_state(u0)
    p0 = Port(case.config(), mesh)
    p0.set_state(u0)
    want = p0.cfl_dt()
    assert abs(gpu.step(0.0) - want) <= 1e-14 * want


def test_sync_times_out_while_running_then_completes():
    case = small_case("vortex", "HLLC", "NONE", level=6)
    case.tau = 0.01
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    a = Solver(case)
    a.upload(mesh)
    a.set_state(u0)
    a.run(40, case.tau)
    assert a.sync_status(0.0) == abi.ETIMEDOUT
    assert a.sync_status(600.0) == abi.OK
    b = Solver(case)
    b.upload(mesh)
    b.set_state(u0)
    b.run(40, case.tau)
    b.sync()
    assert np.array_equal(a.get_state(), b.get_state())


def _corruptions(mesh):
    """(description, corrupted copy) pairs of a flattened mesh with hanging faces."""
    out = []

    def variant(name, fn):
        m = copy.copy(mesh)
        m.face_elem, m.face_info = mesh.face_elem.copy(), mesh.face_info.copy()
        m.bface_elem, m.bface_face, m.bface_bnd = mesh.bface_elem.copy(), mesh.bface_face.copy(), mesh.bface_bnd.copy()
        fn(m)
        out.append((name, m))

    kind = (mesh.face_info >> 2) & 3
    conf = int(np.flatnonzero(kind == 0)[0])
    mort = int(np.flatnonzero(kind != 0)[0])
    variant("element index past the end", lambda m: m.face_elem.__setitem__((1, conf), mesh.n_elem))
    variant("negative element index", lambda m: m.face_elem.__setitem__((0, conf), -1))
    variant("direction bits 3", lambda m: m.face_info.__setitem__(conf, m.face_info[conf] | 3))
    variant("mortar kind 3", lambda m: m.face_info.__setitem__(mort, m.face_info[mort] | 12))
    variant("mortar sub-faces out of order",
            lambda m: m.face_info.__setitem__(slice(mort, mort + 2), m.face_info[[mort + 1, mort]]))
    variant("boundary id past the table", lambda m: m.bface_bnd.__setitem__(0, 7))
    variant("boundary face 6", lambda m: m.bface_face.__setitem__(0, 6))

    def duplicate(m):   # one boundary record repeated in place of another: one face twice, one face missing
        m.bface_elem[1], m.bface_face[1] = m.bface_elem[0], m.bface_face[0]
    variant("element face with two records", duplicate)

    def drop(m):        # one boundary record fewer
        m.n_bface -= 1
        m.bface_elem, m.bface_face, m.bface_bnd = m.bface_elem[1:], m.bface_face[1:], m.bface_bnd[1:]
    variant("element face without a record", drop)
    return out


def test_upload_rejects_corrupted_faces_and_keeps_mesh():
    case = small_case("random", "HLLC", "BJ", level=2)
    forest, _ = hanging_forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u0)
    lib = abi.load()
    for name, bad in _corruptions(mesh):
        s = bad.struct()
        rc = lib.charm_gpu_upload_mesh(gpu.h, s)
        assert rc == abi.EINVAL, name
    # the handle still holds the good mesh and the state set before
    port = Port(case.config(), mesh)
    port.set_state(u0)
    gpu.run(2, case.tau)
    gpu.sync()
    port.run(2, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < 1e-12
    # and takes a valid upload again
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.run(2, case.tau)
    gpu.sync()
    assert rel_l2(gpu.get_state(), port.get_state()) < 1e-12


def _ulps(got, want):
    """Distance in units in the last place of want."""
    return np.abs(got - want) / np.spacing(np.abs(want))


def test_fp64_reciprocal_and_quotient_error_bounds():
    """The flux kernels' FP64 reciprocal (hardware seed + two Newton steps)
    within 1 ulp of IEEE 1/x, and their quotient a * (1/b) within 2 ulp of
    IEEE a/b, over normal operands of every magnitude the state can hold."""
    lib = abi.load()
    rng = np.random.default_rng(5)
    n = 1 << 20
    b = rng.uniform(1.0, 2.0, n) * 2.0 ** rng.integers(-300, 300, n) * rng.choice([-1.0, 1.0], n)
    b[:4] = [1.0, 2.0, 0.75, 3.0]
    a = rng.uniform(1.0, 2.0, n) * 2.0 ** rng.integers(-20, 20, n)
    out = np.empty(n)
    assert lib.charm_gpu_math_check(0, n, None, b.ctypes.data, out.ctypes.data) == abi.OK
    assert _ulps(out, 1.0 / b).max() <= 1.0
    assert out[0] == 1.0 and out[1] == 0.5
    assert lib.charm_gpu_math_check(1, n, a.ctypes.data, b.ctypes.data, out.ctypes.data) == abi.OK
    assert _ulps(out, a / b).max() <= 2.0
