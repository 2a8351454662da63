"""The time step on general (trilinear) hexahedra, GPU against the oracle.

Meshes are forests over unstructured hexahedral meshes whose trees meet in
all 24 face orientations (tests/hexmesh.py), with non-affine cells, mortars
across tree faces, and a channel with a ramp shaped like the reference's
sample case (samples/klin_amr: Euler, HLLC, Barth-Jespersen, inlet, outlet
and slip walls).  The bar is the drop-in's: 1e-12 relative (residuals by
max-norm, states by L2).

Reference: src/charm_geom.c (geometry), src/models/ns/charm_model_ns_conv.c
(face and volume integrals), src/limiters/charm_limiter_bj.c,
src/models/ns/charm_model.c:68-99 (update with the full inverse mass matrix).
"""
import numpy as np
import pytest

from charm_3d_gb300 import Boundary, synthetic
from charm_3d_gb300.abi import EINVAL, CharmGpuError
from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import rel_l2, rel_max, small_case
from .hexmesh import SIDE_PATCHES, WEDGE_PATCHES, block_forest, block_mesh, wedge_mesh

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _pair(case, forest):
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    u0 = case.initial_state(mesh.center)
    gpu.set_state(u0)
    port.set_state(u0)
    return mesh, gpu, port, u0


CASES = [("random", "LF", "BJ", "keystone"), ("random", "HLLC", "BJ", "keystone"), ("random", "CD", "NONE", "keystone"),
         ("random", "GODUNOV", "NONE", "keystone"), ("walls", "HLLC", "BJ", "keystone"),
         ("mix2", "HLLC", "BJ", "keystone"), ("massflow", "HLLC", "NONE", "keystone"),
         ("random", "HLLC", "BJ", "distorted")]


@pytest.mark.parametrize("kind,flux,lim,shape", CASES)
def test_hex_residual_and_steps_match_oracle(kind, flux, lim, shape):
    case = small_case(kind, flux, lim)
    if shape == "keystone":
        forest, _ = block_forest(case, level=1)
    else:   # smooth interior distortion: curved (non-planar) cell faces
        forest, _ = block_forest(case, level=1, shape=None, distort=0.12)
    _, gpu, port, u0 = _pair(case, forest)
    assert rel_max(gpu.residual(), port.residual()) < TOL
    gpu.set_state(u0)
    gpu.run(case.steps, case.tau)
    gpu.sync()
    port.run(case.steps, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL


@pytest.mark.parametrize("model", ["NS", "EULER"])
def test_hex_mortars_across_rotated_trees_match_oracle(model):
    case = small_case("random", "HLLC", "BJ", model=model)
    case.tau *= 0.25
    forest, _ = block_forest(case, level=1, seed=6)
    rng = np.random.default_rng(2)
    forest.adapt((rng.uniform(size=len(forest)) < 0.25).astype(np.int8), 0, 3)
    mesh, gpu, port, u0 = _pair(case, forest)
    assert ((mesh.face_info >> 2) & 3).any()
    assert rel_max(gpu.residual(), port.residual()) < TOL
    gpu.set_state(u0)
    gpu.run(case.steps, case.tau)
    gpu.sync()
    port.run(case.steps, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL


def ramp_case(level: int = 0, n: int = 3):
    """The sample case's physics on the ramp channel: Euler, HLLC, BJ, air at
    300 K and 101325 Pa entering at 697.7082 m/s (samples/klin_amr/task.yaml's
    values), outlet, slip walls; seeded +-1 % density noise."""
    case = synthetic("sod", level=level)
    case.model, case.flux, case.limiter = "EULER", "HLLC", "BJ"
    T, P, V = 300.0, 101325.0, 697.7082
    case.boundaries = [Boundary("LEFT", "BOUND_INLET", (V, 0.0, 0.0, T, P)), Boundary("RIGHT", "BOUND_OUTLET"),
                       Boundary("BOTTOM", "BOUND_WALL_SLIP"), Boundary("TOP", "BOUND_WALL_SLIP"),
                       Boundary("FRONT", "BOUND_WALL_SLIP"), Boundary("BACK", "BOUND_WALL_SLIP")]
    m = wedge_mesh(n, rotate=True, seed=9)
    forest = Forest.from_hex(m.vert, m.trees, m.tree_bnd(WEDGE_PATCHES), level)
    mesh = forest.flatten()
    comp = case.components[0]
    rho = P * comp.m / (8.31446261815324 * T)
    E = mesh.n_elem
    rng = np.random.default_rng(4)
    r = rho * (1.0 + 0.01 * rng.uniform(-1, 1, E))
    one = np.ones(E)
    u0 = np.zeros((case.n_var, 4, E))
    u0[:, 0, :] = case.cons_from_prim(r, V * one, 0 * one, 0 * one, P * one)
    # CFL 0.1 with the smallest edge (the ramp block's cells) and |u| + c
    h = 1000.0 / n / 2 ** level
    case.tau = 0.1 * h / (V + np.sqrt(1.4 * P / rho))
    return case, forest, mesh, u0


@pytest.mark.parametrize("level,n", [(0, 3), (1, 3), (0, 10)])
def test_hex_ramp_channel_matches_oracle(level, n):
    """n = 10: the sample case samples/klin_amr on its own mesh geometry
    (tests/test_hexmesh.py pins the generated mesh to the sample's file)."""
    case, forest, mesh, u0 = ramp_case(level, n)
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    gpu.set_state(u0)
    port.set_state(u0)
    assert rel_max(gpu.residual(), port.residual()) < TOL
    gpu.set_state(u0)
    gpu.run(10, case.tau)
    gpu.sync()
    port.run(10, case.tau)
    got, want = gpu.get_state(), port.get_state()
    assert np.isfinite(got).all()
    assert rel_l2(got, want) < TOL
    # the ramp turns the flow: the state has left the uniform inflow
    assert np.abs(want[1, 0] / want[4, 0]).max() > 1.0


def test_hex_on_a_brick_equals_the_box_path():
    """Identity-oriented cubic trees: the general-hexahedron kernels give the
    box kernels' step on the same leaves."""
    case = small_case("random", "HLLC", "BJ", level=2)
    case.brick, case.tree_len = (2, 1, 1), (0.5, 1.0, 1.0)
    box = Forest(case).flatten()
    m = block_mesh(2, 1, 1)
    hexm = Forest.from_hex(m.vert, m.trees, np.zeros((2, 6), np.int8), 2).flatten()
    order = np.array([np.argmin(((hexm.center.T - c) ** 2).sum(1)) for c in box.center.T])
    u0 = case.initial_state(box.center)
    uh = np.empty_like(u0)
    uh[:, :, order] = u0
    gb, gh = Solver(case), Solver(case)
    gb.upload(box)
    gh.upload(hexm)
    gb.set_state(u0)
    gh.set_state(uh)
    gb.run(3, case.tau)
    gh.run(3, case.tau)
    gb.sync()
    gh.sync()
    assert rel_l2(gh.get_state()[:, :, order], gb.get_state()) < TOL


def test_hex_cfl_step_matches_oracle():
    case, forest, mesh, u0 = ramp_case(0)
    case.dt_mode, case.cfl, case.tau = "CFL", 0.1, 1.0
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    gpu.set_state(u0)
    port.set_state(u0)
    for _ in range(3):
        dt_gpu = gpu.step()
        dt_port = port.cfl_dt()
        assert abs(dt_gpu - dt_port) <= 1e-14 * dt_port
        port.step(dt_port)
    gpu.sync()
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL


def test_hex_upload_rejects_inverted_elements_and_keeps_the_mesh():
    case = small_case("random", "HLLC", "BJ")
    forest, _ = block_forest(case, level=1)
    mesh, gpu, port, u0 = _pair(case, forest)
    good = mesh.vertex.copy()
    mesh.vertex = good[[4, 5, 6, 7, 0, 1, 2, 3]]   # mirrored corners: negative Jacobians
    with pytest.raises(CharmGpuError) as ei:
        gpu.upload(mesh)
    assert ei.value.code == EINVAL
    mesh.vertex = good
    gpu.run(2, case.tau)   # the previous mesh and state are untouched
    gpu.sync()
    port.run(2, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL
