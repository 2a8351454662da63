"""The configuration's AMR criterion |grad rho| L / rho (no counterpart in the
reference, whose criterion is charm_gpu_refine_flags'), driving the host
adapt through charm_host_forest_adapt_plan_flags and the device projection."""
import numpy as np
import pytest

from charm_3d_gb300 import synthetic
from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import hanging_forest, small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("per_cell", [True, False])
def test_relative_flags_follow_the_formula_on_the_oracle_gradient(per_cell):
    case = small_case("random", "HLLC", "BJ", level=3)
    forest, _ = hanging_forest(case)
    mesh = forest.flatten()
    u = case.initial_state(mesh.center)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u)
    port = Port(case.config(), mesh)
    port.set_state(u)
    thr = 0.1 if per_cell else 1.0
    flags, grad = gpu.refine_flags_relative(thr, per_cell)
    g = port.amr_grad()
    assert np.abs(grad - g).max() < 1e-12 * np.abs(g).max()
    rho = np.maximum(u[4:, 0, :].sum(axis=0), 1e-12)
    L = 0.5 ** mesh.level.astype(np.float64) if per_cell else 1.0   # unit-cube leaves: edge 2^-level
    ind = np.sqrt((g ** 2).sum(axis=0)) * L / rho
    want = np.where(ind > thr, 1, np.where(ind <= 0.5 * thr, -1, 0))
    clear = (np.abs(ind - thr) > 1e-9 * thr) & (np.abs(ind - 0.5 * thr) > 1e-9 * thr)
    assert clear.sum() > 0.9 * len(ind)
    assert np.array_equal(flags[clear], want[clear])
    assert set(np.unique(flags)) <= {-1, 0, 1} and (flags == 1).any() and (flags == -1).any()


def test_blast_with_the_relative_criterion_follows_the_shock():
    """A short blast run: adapts every 5 steps by |grad rho| h / rho > 0.1
    refine the shell around the blast, coarsen away from it, and the device
    projections keep the total mass."""
    case = synthetic("blast", level=4)   # at level 4 the 0.1 blast radius holds whole cells
    case.min_level, case.max_level = 4, 6
    case.tau *= 4.0
    forest = Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u0)

    def mass(m, x):
        return float((x[4:, 0].sum(axis=0) * 8.0 ** (-m.level.astype(np.float64))).sum())

    m0 = mass(mesh, u0)
    for _ in range(4):
        gpu.run(5, case.tau)
        flags, _ = gpu.refine_flags_relative(0.1, True)
        _, plan = forest.adapt_plan_flags(flags, case.min_level, case.max_level)
        mesh = forest.flatten()
        gpu.adapt_upload(plan, mesh)
    gpu.sync()
    u = gpu.get_state()
    assert np.isfinite(u).all()
    assert mesh.level.max() >= 5 and mesh.level.min() == 4
    r = np.sqrt(((mesh.center - 0.5) ** 2).sum(axis=0))
    fine = mesh.level >= 5
    assert np.median(r[fine]) < 0.35
    assert abs(mass(mesh, u) - m0) < 1e-12 * m0
