"""The double-word form (CHARM_GPU_PREC_DW): FP64 state, fluxes and volume
terms in double-word arithmetic on the FP32 pipe (two floats, ~48 bits).

It is held to the drop-in's bar: 1e-12 relative against the oracle and the
reference's own fixtures (residuals by max-norm, states by L2), on every
flux, boundary type, two species, hanging faces and the limiter (which runs
in FP64 on the state), and on the bench workload.
"""
import os

import numpy as np
import pytest

from charm_3d_gb300.abi import ENOTSUP, CharmGpuError
from charm_3d_gb300.solver import Forest, Solver, point_flux
from charm_3d_gb300 import synthetic
from oracle.port import Port

from .common import hanging_forest, rel_l2, rel_max, small_case
from .golden_cases import GOLDEN, NAMES, load

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _pair(case, forest=None):
    case.precision = "DW"
    forest = forest or Forest(case)
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    port = Port(case.config(), mesh)
    u0 = case.initial_state(mesh.center)
    gpu.set_state(u0)
    port.set_state(u0)
    return mesh, gpu, port, u0


CASES = [("random", "LF", "BJ"), ("random", "HLLC", "BJ"), ("random", "CD", "NONE"),
         ("vortex", "HLLC", "NONE"), ("walls", "HLLC", "BJ"), ("massflow", "HLLC", "NONE")]


def _dw_supported(case) -> bool:
    """The form covers an ideal gas with constant cp (the EOS in FP32 pairs)."""
    return case.eos == "IDEAL" and all(c.cp_type == "CONST" for c in case.components)


def test_dw_rejects_the_mixture_eos():
    case = small_case("mix2", "HLLC", "BJ")
    case.precision = "DW"
    with pytest.raises(CharmGpuError) as ei:
        Solver(case)
    assert ei.value.code == ENOTSUP


def test_dw_rejects_the_godunov_flux():
    """The form has LF, HLLC and CD; the exact Riemann solver's iteration
    stays FP64-only, and a DW handle or point-flux call with it is refused."""
    case = small_case("random", "GODUNOV", "NONE")
    case.precision = "DW"
    with pytest.raises(CharmGpuError) as ei:
        Solver(case)
    assert ei.value.code == ENOTSUP
    with pytest.raises(CharmGpuError) as ei:
        point_flux(case, np.ones((1, 2, 5)), np.array([[1.0, 0.0, 0.0]]))
    assert ei.value.code == ENOTSUP


@pytest.mark.parametrize("kind,flux,lim", CASES)
def test_dw_residual_and_steps_match_oracle(kind, flux, lim):
    case = small_case(kind, flux, lim)
    _, gpu, port, u0 = _pair(case)
    assert rel_max(gpu.residual(), port.residual()) < TOL
    gpu.set_state(u0)
    gpu.run(case.steps, case.tau)
    gpu.sync()
    port.run(case.steps, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL


@pytest.mark.parametrize("flux", ["HLLC", "LF"])
def test_dw_hanging_faces_match_oracle(flux):
    case = small_case("random", flux, "BJ")
    forest, _ = hanging_forest(case)
    _, gpu, port, _ = _pair(case, forest)
    gpu.run(case.steps, case.tau)
    gpu.sync()
    port.run(case.steps, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL


@pytest.mark.parametrize("name", NAMES)
def test_dw_matches_reference_fixture(name):
    case, _, mesh, d, meta = load(name)
    if not _dw_supported(case):
        pytest.skip("fixture with a mixture EOS or T-dependent cp: the double-word form refuses it")
    case.precision = "DW"
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(d["u0"])
    assert rel_max(gpu.residual(), d["residual"]) < TOL
    gpu.set_state(d["u0"])
    gpu.run(meta["steps"], float(d["dt"]))
    gpu.sync()
    assert rel_l2(gpu.get_state(), d["state"]) < TOL


@pytest.mark.parametrize("flux", ["LF", "HLLC", "CD"])
def test_dw_point_fluxes_match_reference(flux):
    d = np.load(os.path.join(GOLDEN, "point_fluxes.npz"))
    case = small_case("random", flux, "NONE", level=1)
    case.precision = "DW"
    _, gam = case.gas_constants()
    prim = d["prim2"]
    r, u, v, w, p = (prim[..., k] for k in range(5))
    e = p / ((gam - 1.0) * r)
    U2 = np.stack([r * u, r * v, r * w, r * (e + 0.5 * (u * u + v * v + w * w)), r], axis=-1)
    q = point_flux(case, U2, d["normals"])
    want = d[flux]
    scale = np.abs(want).max(axis=1, keepdims=True)
    assert (np.abs(q - want) <= 1e-12 * scale).all(), (np.abs(q - want) / scale).max()


def test_dw_bench_workload_matches_oracle():
    """The vortex of the bench at level 5 over the bench's 20 steps."""
    case = synthetic("vortex", level=5)
    _, gpu, port, u0 = _pair(case)
    gpu.run(20, case.tau)
    gpu.sync()
    port.run(20, case.tau)
    assert rel_l2(gpu.get_state(), port.get_state()) < TOL
