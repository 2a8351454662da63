"""Viscous terms (src/models/ns/charm_model_ns_diff*.c) and chemistry
(src/models/ns/charm_model_ns_chem.c) of the oracle against the
reference's own code (oracle/_ref): charm_model_ns_timestep_diff (diffusion
coefficients, lifted stress and heat flux, viscous integrals) and
charm_model_ns_timestep_chem, on the same meshes and seeded states.

The viscous part of the residual is compared on its own (residual with
use_visc = 1 minus residual with use_visc = 0, on both sides), so that the
bar is not hidden by the larger convective part."""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest
from oracle.port import Port
from oracle.ref import RefSolver

from .common import hanging_forest, rel_l2, rel_max, small_case

pytestmark = pytest.mark.reference

TOL = 1e-11


def _pair(case, hang=False):
    if hang:
        forest, flags = hanging_forest(case)
        ref = RefSolver(case, "patched")
        assert ref.refine_flags(flags, case.level + 1) == len(forest)
    else:
        forest = Forest(case)
        ref = RefSolver(case)
    mesh = forest.flatten()
    port = Port(case.config(), mesh)
    u0 = case.initial_state(mesh.center)
    return mesh, ref, port, u0


@pytest.mark.parametrize("kind,flux,hang", [("visc", "LF", False), ("visc", "HLLC", True), ("visc_walls", "HLLC", False),
                                            ("visc2", "LF", False), ("visc2", "HLLC", True)])
def test_viscous_residual_matches_reference(kind, flux, hang):
    case = small_case(kind, flux, "NONE", level=2)
    mesh, ref, port, u0 = _pair(case, hang)
    ref.set_state(u0)
    port.set_state(u0)
    r_ref, r_port = ref.residual(), port.residual()
    assert rel_max(r_port, r_ref) < TOL
    # the viscous part alone
    case.use_visc = 0
    _, ref0, port0, _ = _pair(case, hang)
    ref0.set_state(u0)
    port0.set_state(u0)
    d_ref, d_port = r_ref - ref0.residual(), r_port - port0.residual()
    assert np.abs(d_ref).max() > 1e-6 * np.abs(r_ref).max()
    assert rel_max(d_port, d_ref) < 1e-10


@pytest.mark.parametrize("kind,flux,lim", [("visc", "HLLC", "BJ"), ("visc_walls", "LF", "NONE"), ("visc2", "HLLC", "NONE"),
                                           ("react", "HLLC", "NONE"), ("react", "LF", "BJ")])
def test_viscous_reacting_steps_match_reference(kind, flux, lim):
    case = small_case(kind, flux, lim, level=2)
    mesh, ref, port, u0 = _pair(case)
    ref.set_state(u0)
    port.set_state(u0)
    ref.run(3)
    port.run(3, case.tau)
    assert rel_l2(port.get_state(), ref.get_state()) < TOL


def test_chemistry_changes_species():
    case = small_case("react", "HLLC", "NONE", level=2)
    mesh, ref, port, u0 = _pair(case)
    port.set_state(u0)
    port.run(1, case.tau)
    u1 = port.get_state()
    case.reactions = []
    _, _, port0, _ = _pair(case)
    port0.set_state(u0)
    port0.run(1, case.tau)
    assert np.abs(u1[4] - port0.get_state()[4]).max() > 1e-4 * np.abs(u0[4]).max()
