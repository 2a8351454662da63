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
from charm_3d_gb300.hexmesh import ramp_channel

from .hexmesh import WEDGE_PATCHES, block_forest, block_mesh, wedge_mesh

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
    """The sample case's physics on the ramp channel (charm_3d_gb300.hexmesh.ramp_channel)."""
    return ramp_channel(level, n, rotate=True, seed=9)


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


def _amr_loop(case, forest, u0, steps, period, max_err, max_level, gpu_side):
    """The AMR time loop of the sample case (charm_model_ns_timestep_single's
    adapt every REFINE_PERIOD steps, src/charm_amr.c:575-610) on an
    unstructured forest: the density-gradient estimate from the GPU or the
    oracle, the host octree's adapt with the quadrature projections, then
    the steps on the new mesh."""
    mesh = forest.flatten()
    u = u0
    n_adapt = 0
    for step in range(steps):
        if step and step % period == 0:
            if gpu_side:
                grad = solver.refine_flags(max_err)[1]
                u = solver.get_state()
            else:
                grad = solver.amr_grad()
                u = solver.get_state()
            n0 = len(forest)
            u = forest.adapt_state(grad, max_err, 0, max_level, case.n_comp, u)
            n_adapt += len(forest) != n0
            mesh = forest.flatten()
        if step == 0 or (step % period == 0):
            if gpu_side:
                solver = Solver(case)
                solver.upload(mesh)
            else:
                solver = Port(case.config(), mesh)
            solver.set_state(u)
        solver.step(case.tau)
    if gpu_side:
        solver.sync()
    return solver.get_state(), forest.leaves(), n_adapt


def test_hex_refine_indicator_matches_oracle():
    case, forest, mesh, u0 = ramp_case(0)
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    gpu.set_state(u0)
    port.set_state(u0)
    gpu.run(4, case.tau)
    port.run(4, case.tau)
    gpu.sync()
    port.set_state(gpu.get_state())
    _, grad = gpu.refine_flags(0.01)
    assert rel_max(grad, port.amr_grad()) < TOL


def test_hex_amr_loop_matches_oracle():
    """The sample case's controls (MAX_ERROR 0.01, MAX_LEVEL 1, REFINE_PERIOD
    10) on the ramp channel over 40 steps: the same leaves and states 1e-12
    apart."""
    case, _, _, u0 = ramp_case(0)
    m = wedge_mesh(3, rotate=True, seed=9)
    fo = Forest.from_hex(m.vert, m.trees, m.tree_bnd(WEDGE_PATCHES), 0)
    fg = Forest.from_hex(m.vert, m.trees, m.tree_bnd(WEDGE_PATCHES), 0)
    uo, (qo, lo), nao = _amr_loop(case, fo, u0, 40, 10, 0.01, 1, False)
    ug, (qg, lg), nag = _amr_loop(case, fg, u0, 40, 10, 0.01, 1, True)
    assert nao > 0 and (lo == 1).any(), "the shock off the ramp refines"
    assert np.array_equal(qo, qg) and np.array_equal(lo, lg)
    assert rel_l2(ug, uo) < TOL
