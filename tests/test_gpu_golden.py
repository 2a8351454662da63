"""GPU path against fixtures produced by the reference's own code (tests/golden/).

Bar: 1e-12 relative for the plain FP64 path.
"""
import numpy as np
import pytest

from charm_3d_gb300.solver import Solver

from .common import rel_l2, rel_max
from .golden_cases import NAMES, load

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_reference_fixture(name):
    case, _, mesh, d, meta = load(name)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(d["u0"])
    assert rel_max(gpu.residual(), d["residual"]) < TOL
    gpu.set_state(d["u0"])
    gpu.run(meta["steps"], float(d["dt"]))
    gpu.sync()
    assert rel_l2(gpu.get_state(), d["state"]) < TOL
