"""GPU path (libcharm_gpu.so) against the CPU oracle on the same seeded inputs.

Tolerances: the plain FP64 path must match to 1e-12 relative (the drop-in
bar); it differs from the oracle only by rounding order and fused
multiply-adds.  The mixed form (FP32 residual, FP64 state) must stay within
1e-6 relative L2 of the FP64 path.
"""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import hanging_forest, rel_l2, rel_max, small_case

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-6


def _pair(case, forest=None, precision="FP64"):
    case.precision = precision
    forest = forest or Forest(case)
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    u0 = case.initial_state(mesh.center)
    gpu.set_state(u0)
    port.set_state(u0)
    return forest, mesh, gpu, port, u0


CASES = [("random", "LF", "BJ"), ("random", "HLLC", "BJ"), ("random", "CD", "NONE"), ("random", "GODUNOV", "NONE"),
         ("vortex", "HLLC", "NONE"), ("vortex", "LF", "BJ"), ("walls", "HLLC", "BJ"), ("walls", "LF", "NONE"),
         ("sod", "LF", "BJ")]


@pytest.mark.parametrize("kind,flux,lim", CASES)
def test_residual_matches_oracle(kind, flux, lim):
    case = small_case(kind, flux, lim)
    _, _, gpu, port, _ = _pair(case)
    assert rel_max(gpu.residual(), port.residual()) < FP64_TOL


@pytest.mark.parametrize("kind,flux,lim", CASES)
def test_steps_match_oracle(kind, flux, lim):
    case = small_case(kind, flux, lim)
    _, _, gpu, port, _ = _pair(case)
    gpu.run(case.steps, case.tau)
    gpu.sync()
    port.run(case.steps, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


@pytest.mark.parametrize("flux,lim", [("HLLC", "BJ"), ("LF", "BJ"), ("HLLC", "NONE")])
def test_hanging_faces_match_oracle(flux, lim):
    case = small_case("random", flux, lim)
    forest, _ = hanging_forest(case)
    _, mesh, gpu, port, _ = _pair(case, forest)
    assert mesh.face_info.size and ((mesh.face_info >> 2) & 3).max() > 0, "mesh has no mortars"
    assert rel_max(gpu.residual(), port.residual()) < FP64_TOL
    gpu.run(case.steps, case.tau)
    gpu.sync()
    port.run(case.steps, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


def test_euler_model_matches_oracle():
    case = small_case("random", "HLLC", "BJ", model="EULER")
    _, _, gpu, port, _ = _pair(case)
    gpu.run(2, case.tau)
    port.run(2, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < FP64_TOL


def test_limiter_alone_matches_oracle():
    case = small_case("random", "LF", "BJ")
    case.init_args = {"slope": 0.5}
    _, _, gpu, port, _ = _pair(case)
    gpu.limit()
    port.limit()
    assert rel_max(gpu.get_state(), port.get_state()) < FP64_TOL


@pytest.mark.parametrize("kind,flux,lim", [("vortex", "HLLC", "NONE"), ("sod", "LF", "BJ")])
def test_mixed_precision_error(kind, flux, lim):
    case = small_case(kind, flux, lim, level=4)
    _, _, g64, _, u0 = _pair(case)
    case32 = small_case(kind, flux, lim, level=4)
    case32.precision = "MIXED"
    g32 = Solver(case32)
    g32.upload(g64.mesh)
    g32.set_state(u0)
    g64.run(5, case.tau)
    g32.run(5, case.tau)
    a, b = g32.get_state(), g64.get_state()
    rho32, rho64 = a[4:].sum(axis=0)[0], b[4:].sum(axis=0)[0]
    assert rel_l2(rho32, rho64) < MIXED_TOL
    assert rel_l2(a, b) < MIXED_TOL


def test_nonfinite_state_reports_status_and_gpu_stays_usable():
    case = small_case("random", "HLLC", "NONE")
    _, _, gpu, _, u0 = _pair(case)
    bad = u0.copy()
    bad[4, 0, 5] = np.nan
    gpu.set_state(bad)
    gpu.step(case.tau)
    from charm_3d_gb300 import abi
    assert gpu.sync_status() in (abi.ENONFINITE, abi.ENEGATIVE)
    gpu.set_state(u0)
    gpu.step(case.tau)
    gpu.sync()
    assert np.isfinite(gpu.get_state()).all()
