"""p2 basis on the GPU (FP64) against the oracle's p2 restatement: residuals
and time steps for every flux, all boundary types, periodic meshes, two
species, viscous terms, diffusion and chemistry; and the configurations the
p2 path does not take."""
import numpy as np
import pytest

from charm_3d_gb300.abi import CharmGpuError
from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import hanging_forest, rel_l2, rel_max, small_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _p2(kind, flux, level=2):
    case = small_case(kind, flux, "NONE", level=level)
    case.p_order = 2
    case.precision = "FP64"
    return case


def _pair(case):
    mesh = Forest(case).flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    u0 = case.initial_state(mesh.center)
    assert u0.shape[1] == 10
    gpu.set_state(u0)
    port.set_state(u0)
    return mesh, gpu, port, u0


CASES = [("random", "LF"), ("random", "HLLC"), ("random", "CD"), ("random", "GODUNOV"), ("walls", "HLLC"),
         ("vortex", "HLLC"), ("mix2", "LF"), ("visc", "HLLC"), ("visc_walls", "LF"), ("visc2", "HLLC")]


@pytest.mark.parametrize("kind,flux", CASES)
def test_p2_residual_matches_oracle(kind, flux):
    case = _p2(kind, flux)
    _, gpu, port, _ = _pair(case)
    assert rel_max(gpu.residual(), port.residual()) < FP64_TOL


STEP_CASES = [("random", "HLLC"), ("walls", "LF"), ("vortex", "HLLC"), ("visc_walls", "HLLC"), ("visc2", "LF"),
              ("react", "HLLC")]


@pytest.mark.parametrize("kind,flux", STEP_CASES)
def test_p2_steps_match_oracle(kind, flux):
    case = _p2(kind, flux)
    _, gpu, port, _ = _pair(case)
    gpu.run(3, case.tau)
    gpu.sync()
    port.run(3, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


def test_p2_flame_matches_oracle():
    from charm_3d_gb300 import synthetic
    case = synthetic("flame", level=3, p_order=2)
    case.tau *= 0.5
    _, gpu, port, _ = _pair(case)
    gpu.run(2, case.tau)
    gpu.sync()
    port.run(2, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


@pytest.mark.parametrize("kind,flux,model", [("random", "HLLC", "NS"), ("walls", "LF", "NS"), ("mix2", "HLLC", "NS"),
                                             ("random", "HLLC", "EULER")])
def test_p2_limiter_steps_match_oracle(kind, flux, model):
    """The Barth-Jespersen limiter on the p2 basis (the reference's loops
    over CHARM_BASE_FN_COUNT, src/limiters/charm_limiter_bj.c:241-315):
    quadrature means, the p2 field at the corners, coefficients 1..9
    scaled; alone and inside the SSP-RK3 steps."""
    case = small_case(kind, flux, "BJ", level=2, model=model)
    case.p_order, case.precision = 2, "FP64"
    _, gpu, port, u0 = _pair(case)
    gpu.limit()
    port.limit()
    lim = port.get_state()
    assert not np.array_equal(lim, u0), "the limiter acts on this state"
    assert rel_l2(gpu.get_state(), lim) < FP64_TOL
    gpu.set_state(u0)
    port.set_state(u0)
    gpu.run(3, case.tau)
    gpu.sync()
    port.run(3, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


def test_p2_rejected_where_not_built():
    case = _p2("random", "HLLC", level=1)
    case.limiter = "BJ"
    case.precision = "MIXED"
    with pytest.raises(CharmGpuError):
        Solver(case)
    case = _p2("random", "HLLC", level=2)
    forest, _ = hanging_forest(case)
    gpu = Solver(case)
    with pytest.raises(CharmGpuError):
        gpu.upload(forest.flatten())
