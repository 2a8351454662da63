"""The oracle's p2 path (10-function Taylor basis, 27/9-point Gauss rules).

The reference has no p2 oracle (its 8/6-point rules under-integrate the p2
mass matrix), so the p2 restatement is checked by properties: free-stream
preservation, conservation, and the order of accuracy on a smooth periodic
density wave advected at constant velocity and pressure (p2 error must fall
at least ~2^2.5 per refinement, p1 ~2^1.5)."""
import math

import numpy as np
import pytest

from charm_3d_gb300 import Boundary, Case
from charm_3d_gb300.solver import Forest
from oracle.port import Port

GL = np.array([-math.sqrt(0.6) / 2, 0.0, math.sqrt(0.6) / 2])
GW = np.array([5.0, 8.0, 5.0]) / 18.0


def basis(xi, nb):
    x, y, z = xi
    phi = [np.ones_like(x), x, y, z]
    if nb == 10:
        phi += [x * x, y * y, z * z, x * y, x * z, y * z]
    return np.stack(phi)


def wave_case(level, order, flux="LF"):
    c = Case(name="wave", model="NS", flux=flux, limiter="NONE", level=level, periodic=(1, 1, 1),
             boundaries=[Boundary("ALL", "BOUND_OUTLET")], p_order=order)
    c.tau = 0.02 * (1.0 / 2 ** level)
    return c


def project(case, mesh, f):
    """L2 projection of the conserved field f(x) [V, n] onto the basis (27-point rule)."""
    nb = case.n_basis
    E = mesh.n_elem
    h = np.asarray(mesh.tree_len)[:, None] * 2.0 ** (-mesh.level.astype(float))[None, :]
    xi = np.stack(np.meshgrid(GL, GL, GL, indexing="ij"), axis=0).reshape(3, -1)   # [3, 27]
    w = np.einsum("i,j,k->ijk", GW, GW, GW).reshape(-1)
    phi = basis(xi, nb)                                                            # [nb, 27]
    M = (phi * w) @ phi.T
    Minv = np.linalg.inv(M)
    out = np.zeros((case.n_var, nb, E))
    for e in range(E):
        x = mesh.center[:, e:e + 1] + xi * h[:, e:e + 1]
        F = f(x)                                                                    # [V, 27]
        out[:, :, e] = (F * w) @ phi.T @ Minv.T
    return out


def exact(case, t):
    cv, gam = case.gas_constants()

    def f(x):
        rho = 1.0 + 0.2 * np.sin(2 * math.pi * (x[0] - t))
        p = np.ones_like(rho)
        return case.cons_from_prim(rho, np.ones_like(rho), np.zeros_like(rho), np.zeros_like(rho), p)
    return f


def l2_density_error(case, mesh, u, t):
    return float(np.sqrt(((u[4, 0] - project(case, mesh, exact(case, t))[4, 0]) ** 2).mean()))


def test_p2_free_stream_and_conservation():
    case = wave_case(2, 2)
    mesh = Forest(case).flatten()
    port = Port(case.config(), mesh)
    U = case.cons_from_prim(np.full(mesh.n_elem, 1.3), np.full(mesh.n_elem, 0.4), np.full(mesh.n_elem, -0.2),
                            np.full(mesh.n_elem, 0.1), np.full(mesh.n_elem, 0.9))
    u = np.zeros((case.n_var, 10, mesh.n_elem))
    u[:, 0] = U
    port.set_state(u)
    assert np.abs(port.residual()).max() < 1e-13 * np.abs(U).max()
    u0 = project(case, mesh, exact(case, 0.0))
    port.set_state(u0)
    port.run(5, case.tau)
    u1 = port.get_state()
    # the mean of a p2 field is c0 + (c4 + c5 + c6) / 12 on a box
    mean = lambda u: u[:, 0] + (u[:, 4] + u[:, 5] + u[:, 6]) / 12.0
    assert np.abs(mean(u1).sum(axis=1) - mean(u0).sum(axis=1)).max() < 1e-12 * np.abs(mean(u0)).sum()


@pytest.mark.parametrize("order,levels,rate", [(1, (2, 3), 2 ** 1.5), (2, (3, 4), 2 ** 2.5)])
def test_order_of_accuracy(order, levels, rate):
    """(p2 is pre-asymptotic below level 3 on this wave: rates 1.9, 3.3, 6.5 from level 1 to 4.)"""
    errs = []
    for level in levels:
        case = wave_case(level, order)
        mesh = Forest(case).flatten()
        port = Port(case.config(), mesh)
        port.set_state(project(case, mesh, exact(case, 0.0)))
        T = 0.05
        n = int(round(T / case.tau))
        port.run(n, T / n)
        errs.append(l2_density_error(case, mesh, port.get_state(), T))
    assert errs[0] / errs[1] > rate, errs
