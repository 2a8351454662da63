"""The CPU oracle (oracle/charm_oracle.c) against fixtures made by the reference's own code.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py
from the reference sources compiled in oracle/_ref: Euler / Navier-Stokes
convective cases, and viscous, multi-species diffusion and Arrhenius
reacting cases (VISC_NAMES).  Bar: 1e-12 relative.
"""
import os

import numpy as np
import pytest

from oracle.port import Port

from .common import rel_l2, rel_max
from .golden_cases import GOLDEN, NAMES, VISC_NAMES, load

TOL = 1e-12


@pytest.mark.parametrize("name", NAMES + VISC_NAMES)
def test_oracle_residual_matches_reference_fixture(name):
    case, _, mesh, d, _ = load(name)
    port = Port(case.config(), mesh)
    assert np.array_equal(case.initial_state(mesh.center), d["u0"]), "fixture inputs not reproduced"
    port.set_state(d["u0"])
    assert rel_max(port.residual(), d["residual"]) < TOL


@pytest.mark.parametrize("name", NAMES + VISC_NAMES)
def test_oracle_steps_match_reference_fixture(name):
    case, _, mesh, d, meta = load(name)
    port = Port(case.config(), mesh)
    port.set_state(d["u0"])
    port.run(meta["steps"], float(d["dt"]))
    assert rel_l2(port.get_state(), d["state"]) < TOL
    assert np.isfinite(d["state"]).all()


@pytest.mark.parametrize("flux", ["LF", "HLLC", "CD", "GODUNOV"])
def test_oracle_point_fluxes_match_reference(flux):
    from .common import small_case
    from charm_3d_gb300.solver import Forest
    d = np.load(os.path.join(GOLDEN, "point_fluxes.npz"))
    case = small_case("random", flux, "NONE", level=1)
    port = Port(case.config(), Forest(case).flatten())
    got = np.stack([port.point_flux(d["prim2"][i].ravel(), d["normals"][i]) for i in range(d["prim2"].shape[0])])
    want = d[flux]
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_oracle_exact_riemann_solver_matches_reference():
    """The oracle's rim_orig against the reference's own rim_orig
    (src/charm_fluxes.c:8-180) over shocks, rarefactions, sonic fans and
    supersonic states; every sampled region occurs."""
    from oracle.port import rim
    d = np.load(os.path.join(GOLDEN, "point_fluxes.npz"))
    got, want = rim(d["rim_in"]), d["rim_out"]
    assert np.isfinite(want).all()
    assert (np.abs(got - want) <= 1e-12 * np.abs(want) + 1e-300).all()
    rin = d["rim_in"]
    left = (want[:, 0] == rin[:, 0]) & (want[:, 3] == rin[:, 2])
    right = (want[:, 0] == rin[:, 5]) & (want[:, 3] == rin[:, 7])
    gam = rin[:, 10]
    sonic = np.isclose(np.abs(want[:, 3]), np.sqrt(gam * want[:, 2] / want[:, 0]), rtol=1e-9)
    assert left.sum() > 10 and right.sum() > 10 and sonic.sum() > 10 and (~(left | right | sonic)).sum() > 10


def test_oracle_adjoint_fd_fixture():
    """The oracle reproduces the reference's J(u0 +- eps d) of the adjoint
    finite-difference fixture (so FD through the oracle is FD through the
    reference)."""
    from charm_3d_gb300.solver import Forest
    from .common import pressure_box_J, small_case
    d = np.load(os.path.join(GOLDEN, "adjoint_fd_vortex.npz"))
    case = small_case("vortex", "HLLC", "NONE", level=3)
    mesh = Forest(case).flatten()
    assert np.allclose(case.initial_state(mesh.center), d["u0"], rtol=1e-13, atol=0.0)
    u0 = d["u0"]
    port = Port(case.config(), mesh)
    n = int(d["steps"])

    def J(u):
        port.set_state(u)
        port.run(n, case.tau)
        return pressure_box_J(case, mesh, port.get_state(), d["lo"], d["hi"])

    assert abs(J(u0) - float(d["J0"])) <= 1e-12 * abs(float(d["J0"]))
    eps = float(d["eps"])
    for k in range(2):
        fd_port = (J(u0 + eps * d["dirs"][k]) - J(u0 - eps * d["dirs"][k])) / (2 * eps)
        fd_ref = (d["Jp"][k] - d["Jm"][k]) / (2 * eps)
        assert abs(fd_port - fd_ref) <= 1e-8 * abs(fd_ref)
