"""The benchmark's own workload against the oracle.

The bench times the isentropic vortex (periodic [0,10]^3, p1, HLLC, no
limiter, seeded 1e-3 density noise) at level 7 for 20 SSP-RK3 steps.  Here
the same workload, through the same C ABI, is compared with the CPU oracle
from the same seeded state: at level 5 over the bench's 20 steps, and at the
bench's level 7 over its first 2 steps (the oracle needs ~1 min and ~5 GB of
host memory for them).  Bar: 1e-12 relative L2 of the state (FP64 drop-in).
"""
import numpy as np
import pytest

from charm_3d_gb300 import synthetic
from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12
BENCH_STEPS = 20


def _compare(level: int, steps: int):
    case = synthetic("vortex", level=level)
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.run(steps, case.tau)
    gpu.sync()
    got = gpu.get_state()
    gpu.close()
    port = Port(case.config(), mesh)
    port.set_state(u0)
    port.run(steps, case.tau)
    want = port.get_state()
    port.close()
    assert np.isfinite(got).all()
    # the state moved: the comparison is not of two copies of u0
    assert rel_l2(want, u0) > 1e-6
    return rel_l2(got, want)


def test_vortex_level5_bench_steps_match_oracle():
    err = _compare(5, BENCH_STEPS)
    assert err < TOL, err


def test_vortex_level7_first_steps_match_oracle():
    err = _compare(7, 2)
    assert err < TOL, err
