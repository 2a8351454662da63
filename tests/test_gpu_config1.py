"""The CPU-runnable benchmark case at full size on the GPU: Sod tube, level 4
(4096 hex), LF, BJ limiter, outlet boundaries, 100 SSP-RK3 steps.  Every
step of the GPU's trajectory is checked against one oracle step from the
same state (1e-12 relative L2, the drop-in's bar).  End states of separate
100-step runs are not comparable at that level: with the BJ limiter this
case turns a 1e-12 relative perturbation of the initial state into a 0.7 %
difference by step 100 (limiter switches), in the reference as in the
oracle."""
import numpy as np
import pytest

from charm_3d_gb300 import synthetic
from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

pytestmark = pytest.mark.gpu


def test_config1_sod_every_step_matches_oracle():
    case = synthetic("sod")
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    gpu = Solver(case)
    gpu.upload(mesh)
    gpu.set_state(u0)
    port = Port(case.config(), mesh)
    worst = 0.0
    for n in range(case.steps):
        u = gpu.get_state()
        port.set_state(u)
        port.step(case.tau)
        gpu.run(1, case.tau)
        a, b = gpu.get_state(), port.get_state()
        worst = max(worst, float(np.linalg.norm(a - b) / np.linalg.norm(b)))
    gpu.sync()
    assert worst <= 1e-12
    gpu.close()
