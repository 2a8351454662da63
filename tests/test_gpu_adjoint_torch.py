"""The C-ABI adjoint inside torch.autograd (tests/adjoint_torch.py): the
gradient of a torch expression of the final state, back-propagated through
the GPU time steps, equals the adjoint with the built-in objective and
central differences."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from charm_3d_gb300.solver import Forest, Solver  # noqa: E402

from .adjoint_torch import CharmSteps, pressure_box_J_torch  # noqa: E402
from .common import small_case  # noqa: E402

pytestmark = pytest.mark.gpu


def test_autograd_through_gpu_steps():
    case = small_case("vortex", "HLLC", "NONE", level=3)
    case.precision = "FP64"
    mesh = Forest(case).flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    u0 = case.initial_state(mesh.center)
    lo, hi = (2.5, 2.5, 2.5), (7.5, 7.5, 7.5)
    n = 6
    x = torch.from_numpy(u0.copy()).requires_grad_(True)
    J = pressure_box_J_torch(case, mesh, CharmSteps.apply(x, gpu, n), lo, hi)
    (g_torch,) = torch.autograd.grad(J, x)
    # the same gradient from the built-in objective
    gpu.set_state(u0)
    g_obj, info = gpu.adjoint(n, 3 * n, Solver.pressure_box(lo, hi))
    assert abs(info.J - J.item()) <= 1e-12 * abs(info.J)
    assert np.abs(g_torch.numpy() - g_obj).max() <= 1e-10 * np.abs(g_obj).max()
    # and central differences along a density direction
    rng = np.random.default_rng(9)
    d = np.zeros_like(u0)
    d[4, 0] = rng.uniform(-1, 1, mesh.n_elem)
    eps = 1e-6
    Js = []
    for s in (1, -1):
        gpu.set_state(u0 + s * eps * d)
        gpu.run(n)
        Js.append(gpu.objective(Solver.pressure_box(lo, hi)))
    fd = (Js[0] - Js[1]) / (2 * eps)
    ad = float((g_torch.numpy() * d).sum())
    assert abs(ad - fd) <= 1e-6 * abs(fd)
