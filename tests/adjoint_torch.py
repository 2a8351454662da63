"""torch.autograd.Function over the C-ABI adjoint (test harness only).

CharmSteps.apply(u0, solver, n_steps) returns u(n_steps) as a CPU float64
tensor computed by the GPU solver; its backward calls charm_gpu_adjoint
with dJ/du(n_steps) = the incoming gradient, so any torch expression of the
final state can be differentiated back to the initial state."""
from __future__ import annotations

import numpy as np
import torch


class CharmSteps(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0: torch.Tensor, solver, n_steps: int, n_snapshots: int = 0) -> torch.Tensor:
        ctx.solver, ctx.n_steps = solver, n_steps
        ctx.n_snapshots = n_snapshots if n_snapshots > 0 else 3 * n_steps
        ctx.u0 = u0.detach().cpu().numpy().copy()
        solver.set_state(ctx.u0)
        solver.run(n_steps)
        return torch.from_numpy(solver.get_state())

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        ctx.solver.set_state(ctx.u0)
        g, _ = ctx.solver.adjoint(ctx.n_steps, ctx.n_snapshots, None,
                                  dJdu_final=np.ascontiguousarray(grad_out.detach().cpu().numpy()))
        return torch.from_numpy(g), None, None, None


def pressure_box_J_torch(case, mesh, u: torch.Tensor, lo, hi) -> torch.Tensor:
    """Integral of p over the elements centred in [lo, hi), in torch (differentiable)."""
    _, gam = case.gas_constants()
    c = mesh.center
    inside = np.ones(mesh.n_elem, bool)
    for d in range(3):
        inside &= (c[d] >= lo[d]) & (c[d] < hi[d])
    h = np.stack([np.asarray(mesh.tree_len[d]) * 2.0 ** (-mesh.level.astype(np.float64)) for d in range(3)])
    w8 = torch.from_numpy(np.where(inside, h[0] * h[1] * h[2] * 0.125, 0.0))
    phi0 = 0.28867513459481288225
    J = u.new_zeros(())
    for g in range(8):
        phi = [phi0 if (g >> d) & 1 else -phi0 for d in range(3)]
        U = u[:, 0, :] + phi[0] * u[:, 1, :] + phi[1] * u[:, 2, :] + phi[2] * u[:, 3, :]
        r = U[4:].sum(dim=0)
        vel = U[:3] / r
        e = U[3] / r - 0.5 * (vel * vel).sum(dim=0)
        J = J + (w8 * (r * e * (gam - 1.0))).sum()
    return J
