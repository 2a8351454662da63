"""Cell-centre output fields (charm_gpu_cell_fields: the values the
reference's output writes per cell, src/charm_output.c:10-52) against the
reference's own values (tests/golden/cell_fields.npz: its charm_get_fields
and charm_param_cons_to_prim at every leaf centre, one and two species),
and against the same primitive-variable formulas in numpy for both forms
and both bases; and the VTK file written from them."""
import os

import numpy as np
import pytest

from charm_3d_gb300.case import GAS_R
from charm_3d_gb300.solver import Forest, Solver

from .common import small_case

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("kind", ["random", "mix2", "vortex"])
def test_cell_fields_match_reference_output(kind):
    d = np.load(os.path.join(GOLDEN, "cell_fields.npz"))
    case = small_case(kind, "HLLC", "NONE", level=2)
    mesh = Forest(case).flatten()
    g = Solver(case)
    g.upload(mesh)
    g.set_state(d[kind + "_u"])
    f = g.cell_fields()
    g.close()
    want = d[kind + "_fields"]
    assert f.shape == want.shape
    scale = np.abs(want).max(axis=1, keepdims=True)
    assert (np.abs(f - want) <= 1e-12 * scale).all(), np.abs(f - want).max(axis=1)


@pytest.mark.parametrize("kind,prec,p_order", [("random", "FP64", 1), ("random", "MIXED", 1), ("mix2", "FP64", 1),
                                               ("random", "FP64", 2)])
def test_cell_fields_match_numpy(kind, prec, p_order):
    case = small_case(kind, "HLLC", "NONE", level=3)
    case.precision, case.p_order = prec, p_order
    mesh = Forest(case).flatten()
    u = case.initial_state(mesh.center)
    g = Solver(case)
    g.upload(mesh)
    g.set_state(u)
    f = g.cell_fields()
    u = g.get_state()      # the state as stored (hi + lo in the mixed form)
    g.close()
    V = case.n_var
    U = u[:, 0]            # the Taylor basis at the centre: coefficient 0
    r = U[4:V].sum(axis=0)
    vel = U[:3] / r
    e_tot = U[3] / r
    e = e_tot - 0.5 * (vel ** 2).sum(axis=0)
    want = {"R": r, "E_TOT": e_tot, "E": e, "U": vel[0], "V": vel[1], "W": vel[2]}
    if kind == "random":     # ideal gas with constant cp: p and T in closed form
        c0 = case.components[0]
        cv = c0.cp[0] - GAS_R / c0.m
        want["P"] = r * e * (c0.cp[0] / cv - 1.0)
        want["T"] = e / cv
    names = ["R", "P", "E", "E_TOT", "U", "V", "W", "T"]
    for k, n in enumerate(names):
        if n in want:
            assert np.allclose(f[k], want[n], rtol=1e-13, atol=1e-14 * np.abs(want[n]).max()), n
    c = np.clip(U[4:V] / r, 0.0, 1.0)
    assert np.allclose(f[8:], c, rtol=1e-13, atol=1e-15)


def test_vtu_from_device_fields(tmp_path):
    case = small_case("mix2", "HLLC", "NONE", level=2)
    forest = Forest(case)
    mesh = forest.flatten()
    g = Solver(case)
    g.upload(mesh)
    g.set_state(case.initial_state(mesh.center))
    f = g.cell_fields()
    g.close()
    names = ["R", "P", "E", "E_TOT", "U", "V", "W", "T"] + ["C_" + c.name for c in case.components]
    path = str(tmp_path / "charm_00000000.vtu")
    forest.write_vtu(path, f, names)
    text = open(path).read()
    for n in names:
        assert f'Name="{n}"' in text
