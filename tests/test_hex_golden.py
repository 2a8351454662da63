"""General hexahedra against the reference's own code: fixtures made by
tests/golden/make_golden.py from the reference's sources (its trilinear
geometry, src/charm_geom.c; face and volume integrals, limiter, update,
and its adapt with the quadrature projections of charm_replace_quads) on
the sample case's ramp geometry and on a keystone block, trees in random
orientations.  The oracle (CPU) and the GPU are checked against them."""
import os

import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import rel_l2, rel_max
from .golden_cases import GOLDEN, HEX_AMR_STEPS, HEX_NAMES, hex_case

TOL = 1e-12


def _fixture(name):
    path = os.path.join(GOLDEN, name + ".npz")
    return np.load(path)


@pytest.mark.parametrize("name", list(HEX_NAMES))
def test_oracle_matches_reference_on_hexahedra(name):
    case, forest, mesh, u0, _ = hex_case(name)
    d = _fixture(name)
    assert np.array_equal(u0, d["u0"])
    port = Port(case.config(), mesh)
    port.set_state(u0)
    assert rel_max(port.residual(), d["residual"]) < TOL
    port.set_state(u0)
    port.run(int(d["steps"]), float(d["dt"]))
    assert rel_l2(port.get_state(), d["state"]) < TOL


def _amr_loop(case, forest, u0, steps, gpu_side):
    """charm_model_*_timestep_single's adapt every REFINE_PERIOD steps (not
    at step 0) with the host octree's adapt and projections, then the step."""
    mesh = forest.flatten()
    u = u0
    solver = None
    for step in range(steps):
        if step and step % case.refine_period == 0:
            if gpu_side:
                _, grad = solver.refine_flags(case.max_err)
            else:
                grad = solver.amr_grad()
            u = forest.adapt_state(grad, case.max_err, case.min_level, case.max_level, case.n_comp, solver.get_state())
            mesh = forest.flatten()
            solver = None
        if solver is None:
            if gpu_side:
                solver = Solver(case)
                solver.upload(mesh)
            else:
                solver = Port(case.config(), mesh)
            solver.set_state(u)
        solver.step(case.tau)
    if gpu_side:
        solver.sync()
    return solver.get_state()


def _amr_case():
    case, forest, mesh, u0, _ = hex_case("hex_ramp_amr")
    case.max_err, case.min_level, case.max_level, case.refine_period = 0.01, 0, 1, 10
    return case, forest, u0


def test_oracle_amr_loop_matches_reference_on_hexahedra():
    case, forest, u0 = _amr_case()
    d = _fixture("hex_ramp_amr")
    u = _amr_loop(case, forest, u0, HEX_AMR_STEPS, False)
    q, lv = forest.leaves()
    rl = d["leaves"]
    assert (rl[:, 4] == 1).any(), "the fixture's run refines"
    assert np.array_equal(rl[:, :4], q) and np.array_equal(rl[:, 4], lv)
    assert rel_l2(u, d["state"]) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(HEX_NAMES))
def test_gpu_matches_reference_on_hexahedra(name):
    case, forest, mesh, u0, _ = hex_case(name)
    d = _fixture(name)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u0)
    assert rel_max(gpu.residual(), d["residual"]) < TOL
    gpu.set_state(u0)
    gpu.run(int(d["steps"]), float(d["dt"]))
    gpu.sync()
    assert rel_l2(gpu.get_state(), d["state"]) < TOL


@pytest.mark.gpu
def test_gpu_amr_loop_matches_reference_on_hexahedra():
    case, forest, u0 = _amr_case()
    d = _fixture("hex_ramp_amr")
    u = _amr_loop(case, forest, u0, HEX_AMR_STEPS, True)
    q, lv = forest.leaves()
    rl = d["leaves"]
    assert np.array_equal(rl[:, :4], q) and np.array_equal(rl[:, 4], lv)
    assert rel_l2(u, d["state"]) < TOL
