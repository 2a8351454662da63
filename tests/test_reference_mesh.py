"""Connectivity, geometry and refinement of the host octree against the reference build.

These tests run the reference's own code (oracle/_ref) and therefore only
where the reference checkout exists.
"""
import numpy as np
import pytest

from charm_3d_gb300 import Case
from charm_3d_gb300.solver import Forest
from oracle.ref import RefSolver

from .common import face_sets_of_mesh, face_sets_of_reference, hanging_forest, small_case

pytestmark = pytest.mark.reference


@pytest.mark.parametrize("hang", [False, True])
def test_reference_face_iteration_matches_flattened_mesh(hang):
    case = small_case("random", "LF", "NONE", level=2)
    if hang:
        forest, flags = hanging_forest(case)
        ref = RefSolver(case, "patched")
        ref.refine_flags(flags, case.level + 1)
    else:
        forest = Forest(case)
        ref = RefSolver(case)
    mesh = forest.flatten()
    assert face_sets_of_mesh(mesh) == face_sets_of_reference(ref.faces())


def test_reference_geometry_matches_box_formulas():
    case = Case(level=2, tree_len=(1.0, 2.0, 0.5), brick=(2, 1, 1))
    ref = RefSolver(case)
    mesh = Forest(case).flatten()
    g = ref.geometry()
    h = np.array(case.tree_len)[:, None] / (2.0 ** mesh.level[None, :])
    assert np.allclose(g[:, 0:3], mesh.center.T, rtol=0, atol=1e-15)
    assert np.allclose(g[:, 3:6], h.T, rtol=1e-15)
    vol = h.prod(axis=0)
    assert np.allclose(g[:, 6], vol, rtol=1e-14)
    ainv = g[:, 7:23].reshape(-1, 4, 4)
    diag = np.stack([1 / vol, 12 / vol, 12 / vol, 12 / vol], axis=1)
    assert np.allclose(np.diagonal(ainv, axis1=1, axis2=2), diag, rtol=1e-13)
    off = ainv - np.einsum("ij,jk->ijk", diag, np.eye(4))
    assert np.abs(off).max() <= 1e-13 * np.abs(diag).max()


def test_reference_refinement_matches_host_adapt():
    case = small_case("random", "HLLC", "BJ", level=2)
    forest, flags = hanging_forest(case, frac=0.3, seed=17)
    ref = RefSolver(case, "patched")
    n = ref.refine_flags(flags, case.level + 1)
    q, lv = forest.leaves()
    rl = ref.leaves()
    assert n == len(forest)
    assert (rl[:, :4] == q).all() and (rl[:, 4] == lv).all()


@pytest.mark.reference
def test_config1_sod_per_step_parity_along_100_steps():
    """The CPU-runnable benchmark case at full size: Sod tube, level 4 (4096
    hex), LF, BJ limiter, outlet boundaries, 100 SSP-RK3 steps.  Parity is
    per step (the bar of the drop-in): every 10th step of the oracle's
    trajectory, one step of the oracle and one of the reference's own code
    from the same state agree to 1e-12 relative L2."""
    from charm_3d_gb300 import synthetic
    from oracle.port import Port
    case = synthetic("sod")
    mesh = Forest(case).flatten()
    u = case.initial_state(mesh.center)
    ref = RefSolver(case, "ref")
    port = Port(case.config(), mesh)
    port.set_state(u)
    for n in range(case.steps):
        if n % 10 == 0:
            u = port.get_state()
            ref.set_state(u)
            ref.run(1)
            port.step(case.tau)
            a, b = port.get_state(), ref.get_state()
            assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(b), f"step {n}"
        else:
            port.step(case.tau)
