"""Viscous terms (src/models/ns/charm_model_ns_diff*.c) and chemistry
(src/models/ns/charm_model_ns_chem.c) on the GPU against the
oracle (itself pinned to the reference's code in tests/test_visc_oracle.py),
FP64: residual with the viscous terms, its viscous part alone, and time
steps with viscosity, species diffusion and reactions, on uniform, hanging
and all-boundary-type meshes."""
import numpy as np
import pytest

from charm_3d_gb300.abi import CharmGpuError
from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import hanging_forest, rel_l2, rel_max, small_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _pair(case, hang=False):
    case.precision = "FP64"
    forest = hanging_forest(case)[0] if hang else Forest(case)
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    u0 = case.initial_state(mesh.center)
    gpu.set_state(u0)
    port.set_state(u0)
    return mesh, gpu, port, u0


CASES = [("visc", "LF", False), ("visc", "HLLC", True), ("visc_walls", "HLLC", False), ("visc_walls", "LF", True),
         ("visc2", "HLLC", False), ("visc2", "LF", True)]


@pytest.mark.parametrize("kind,flux,hang", CASES)
def test_viscous_residual_matches_oracle(kind, flux, hang):
    case = small_case(kind, flux, "NONE", level=2)
    mesh, gpu, port, u0 = _pair(case, hang)
    r_gpu, r_port = gpu.residual(), port.residual()
    assert rel_max(r_gpu, r_port) < FP64_TOL
    case.use_visc = 0
    _, gpu0, port0, _ = _pair(case, hang)
    d_gpu, d_port = r_gpu - gpu0.residual(), r_port - port0.residual()
    assert np.abs(d_port).max() > 1e-6 * np.abs(r_port).max()
    assert rel_max(d_gpu, d_port) < 1e-10


STEP_CASES = [("visc", "HLLC", "BJ", False), ("visc_walls", "LF", "NONE", False), ("visc2", "HLLC", "NONE", True),
              ("react", "HLLC", "NONE", False), ("react", "LF", "BJ", True)]


@pytest.mark.parametrize("kind,flux,lim,hang", STEP_CASES)
def test_viscous_reacting_steps_match_oracle(kind, flux, lim, hang):
    case = small_case(kind, flux, lim, level=2)
    mesh, gpu, port, u0 = _pair(case, hang)
    gpu.run(3, case.tau)
    gpu.sync()
    port.run(3, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


def test_viscous_rejected_where_not_built():
    case = small_case("visc", "HLLC", "NONE", level=1)
    case.precision = "MIXED"
    with pytest.raises(CharmGpuError):
        Solver(case)
    mesh, gpu, _, _ = _pair(small_case("visc", "HLLC", "NONE", level=1))
    with pytest.raises(CharmGpuError):
        gpu.adjoint(1, 3, Solver.pressure_box((0, 0, 0), (1, 1, 1)))


def test_flame_workload_matches_oracle():
    """The reacting workload of the bench (viscous, diffusion, chemistry) at
    level 3, two steps, against the oracle."""
    from charm_3d_gb300 import synthetic
    case = synthetic("flame", level=3)
    mesh, gpu, port, u0 = _pair(case)
    gpu.run(2, case.tau)
    gpu.sync()
    port.run(2, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL
