"""Adaptive refinement: indicator, refine flags, host adapt with projection, and the AMR time loop.

Against the reference's own charm_adapt (oracle/_ref, patched limiter variant
for hanging faces) on CPU, and GPU against the oracle on the GPU machine.
"""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port
from oracle.ref import RefSolver

from .common import amr_case, amr_run_oracle, rel_l2, small_case


@pytest.mark.reference
@pytest.mark.parametrize("kind,max_err,minl,level", [("sod", 0.05, 1, 2), ("random", 0.3, 1, 2), ("random", 0.6, 1, 2),
                                                      ("sod", 0.02, 2, 3), ("walls", 0.2, 1, 2)])
def test_host_adapt_matches_reference_adapt(kind, max_err, minl, level):
    case = small_case(kind, "HLLC", "BJ", level=level)
    case.max_err, case.min_level, case.max_level = max_err, minl, level + 2
    ref = RefSolver(case, "patched")
    forest = Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    ref.set_state(u0)
    n_ref = ref.adapt()
    port = Port(case.config(), mesh)
    port.set_state(u0)
    u1 = forest.adapt_state(port.amr_grad(), case.max_err, case.min_level, case.max_level, case.n_comp, u0)
    q, lv = forest.leaves()
    rl = ref.leaves()
    assert n_ref == len(forest)
    assert (rl[:, :4] == q).all() and (rl[:, 4] == lv).all(), "refine/coarsen/balance differ from charm_adapt"
    ru = ref.get_state()
    assert np.abs(u1 - ru).max() <= 1e-13 * np.abs(ru).max()


@pytest.mark.reference
def test_oracle_amr_loop_matches_reference_time_loop():
    case = amr_case("sod", level=2, max_level=4, max_err=0.05)
    steps = 7
    ref = RefSolver(case, "patched")
    f0 = Forest(case)
    m0 = f0.flatten()
    ref.set_state(case.initial_state(m0.center))
    ref.run(steps)
    forest, mesh, u = amr_run_oracle(case, steps)
    rl = ref.leaves()
    q, lv = forest.leaves()
    assert len(rl) == len(forest) and (rl[:, :4] == q).all() and (rl[:, 4] == lv).all()
    assert mesh.n_elem > m0.n_elem, "the case must refine"
    assert rel_l2(u, ref.get_state()) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_gpu_amr_loop_matches_oracle(prec):
    case = amr_case("sod", level=2, max_level=4, max_err=0.05)
    steps = 7
    forest_o, mesh_o, u_o = amr_run_oracle(case, steps)
    case.precision = prec
    forest = Forest(case)
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(case.initial_state(mesh.center))
    for step in range(steps):
        if step and step % case.refine_period == 0:
            _, grad = gpu.refine_flags(case.max_err)
            u = forest.adapt_state(grad, case.max_err, case.min_level, case.max_level, case.n_comp, gpu.get_state())
            mesh = forest.flatten()
            gpu.upload(mesh)
            gpu.set_state(u)
        gpu.step(case.tau)
    gpu.sync()
    q, lv = forest.leaves()
    qo, lvo = forest_o.leaves()
    assert np.array_equal(q, qo) and np.array_equal(lv, lvo), "GPU refine flags differ from the oracle's"
    assert rel_l2(gpu.get_state(), u_o) < (1e-12 if prec == "FP64" else 1e-6)


@pytest.mark.parametrize("name", ["amr_adapt_sod", "amr_adapt_random", "amr_adapt_walls"])
def test_host_adapt_matches_reference_adapt_fixture(name):
    """The host octree's adapt (refine, coarsen, balance, projections) against
    the reference's charm_adapt recorded in tests/golden/ (no reference build
    needed): the same leaves, the projected state to 1e-13."""
    import json
    import os
    from .golden_cases import GOLDEN
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    case = small_case(meta["kind"], "HLLC", "BJ", level=meta["level"])
    case.max_err, case.min_level, case.max_level = meta["max_err"], meta["min_level"], meta["level"] + 2
    forest = Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    assert np.array_equal(u0, d["u0"]), "fixture inputs not reproduced"
    port = Port(case.config(), mesh)
    port.set_state(u0)
    u1 = forest.adapt_state(port.amr_grad(), case.max_err, case.min_level, case.max_level, case.n_comp, u0)
    q, lv = forest.leaves()
    rl = d["leaves"]
    assert len(rl) == len(forest) and len(rl) != mesh.n_elem
    assert (rl[:, :4] == q).all() and (rl[:, 4] == lv).all(), "refine/coarsen/balance differ from charm_adapt"
    assert np.abs(u1 - d["state"]).max() <= 1e-13 * np.abs(d["state"]).max()


def test_oracle_amr_loop_matches_reference_fixture():
    """The oracle's AMR time loop (adapt every 2 steps) against the
    reference's own loop recorded in tests/golden/amr_loop_sod.npz."""
    import os
    from .golden_cases import GOLDEN
    d = np.load(os.path.join(GOLDEN, "amr_loop_sod.npz"))
    case = amr_case("sod", level=2, max_level=4, max_err=0.05)
    forest, mesh, u = amr_run_oracle(case, int(d["steps"]))
    rl = d["leaves"]
    q, lv = forest.leaves()
    assert len(rl) == len(forest) and (rl[:, :4] == q).all() and (rl[:, 4] == lv).all()
    assert rel_l2(u, d["state"]) < 1e-12
