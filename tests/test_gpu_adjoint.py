"""Discrete adjoint on the GPU (charm_gpu_residual_adjoint, charm_gpu_adjoint)
against central finite differences, eps = 1e-6, through the GPU solver and
through the oracle, and the checkpointing schedule.

Bar: |<dJ/du0, d> - (J(u0 + eps d) - J(u0 - eps d)) / (2 eps)| <= 1e-6
relative, on random directions d."""
import math

import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver
from oracle.port import Port

from .common import hanging_forest, pressure_box_J, small_case

pytestmark = pytest.mark.gpu

FD_EPS = 1e-6
FD_TOL = 1e-6


def _setup(case, forest=None):
    case.precision = "FP64"
    forest = forest or Forest(case)
    mesh = forest.flatten()
    gpu = Solver(case)
    gpu.upload(mesh)
    u0 = case.initial_state(mesh.center)
    gpu.set_state(u0)
    return mesh, gpu, u0


def _direction(rng, u0, var=None):
    """A random direction scaled like the state (or only in one variable)."""
    scale = np.abs(u0).mean(axis=2, keepdims=True) + 1e-3
    d = rng.normal(size=u0.shape) * scale
    if var is not None:
        m = np.zeros_like(d)
        m[var] = d[var]
        d = m
    return d


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


RESIDUAL_CASES = [("random", "LF"), ("random", "HLLC"), ("random", "CD"), ("walls", "HLLC"), ("walls", "LF"),
                  ("vortex", "HLLC")]


@pytest.mark.parametrize("kind,flux", RESIDUAL_CASES)
def test_residual_adjoint_matches_fd(kind, flux):
    case = small_case(kind, flux, "NONE")
    mesh, gpu, u0 = _setup(case)
    port = Port(case.config(), mesh)
    rng = np.random.default_rng(3)
    rbar = rng.normal(size=u0.shape)
    ubar = gpu.residual_adjoint(rbar)
    for trial in range(3):
        d = _direction(rng, u0)
        lhs = float((ubar * d).sum())
        Rp, Rm = [], []
        for sgn, out in ((1, Rp), (-1, Rm)):
            gpu.set_state(u0 + sgn * FD_EPS * d)
            out.append(gpu.residual())
            port.set_state(u0 + sgn * FD_EPS * d)
            out.append(port.residual())
        fd_gpu = float((rbar * (Rp[0] - Rm[0])).sum()) / (2 * FD_EPS)
        fd_port = float((rbar * (Rp[1] - Rm[1])).sum()) / (2 * FD_EPS)
        assert _rel(lhs, fd_gpu) < FD_TOL, (trial, lhs, fd_gpu)
        assert _rel(lhs, fd_port) < FD_TOL, (trial, lhs, fd_port)
        gpu.set_state(u0)


def test_residual_adjoint_hanging_faces():
    case = small_case("random", "HLLC", "NONE")
    forest, _ = hanging_forest(case)
    mesh, gpu, u0 = _setup(case, forest)
    port = Port(case.config(), mesh)
    rng = np.random.default_rng(5)
    rbar = rng.normal(size=u0.shape)
    ubar = gpu.residual_adjoint(rbar)
    for trial in range(3):
        d = _direction(rng, u0)
        port.set_state(u0 + FD_EPS * d)
        Rp = port.residual()
        port.set_state(u0 - FD_EPS * d)
        Rm = port.residual()
        fd = float((rbar * (Rp - Rm)).sum()) / (2 * FD_EPS)
        assert _rel(float((ubar * d).sum()), fd) < FD_TOL


def _box(case):
    """The middle half of the domain along each axis."""
    lo = list(case.origin)
    hi = [o + b * t for o, b, t in zip(case.origin, case.brick, case.tree_len)]
    mid = [0.5 * (a + b) for a, b in zip(lo, hi)]
    q = [0.25 * (b - a) for a, b in zip(lo, hi)]
    return [m - x for m, x in zip(mid, q)], [m + x for m, x in zip(mid, q)]


ADJ_CASES = [("vortex", "HLLC", "NS", 3, 8), ("random", "LF", "NS", 2, 6), ("walls", "HLLC", "NS", 2, 5),
             ("random", "HLLC", "EULER", 2, 6)]


@pytest.mark.parametrize("kind,flux,model,level,nsteps", ADJ_CASES)
def test_adjoint_matches_fd_gpu_and_oracle(kind, flux, model, level, nsteps):
    case = small_case(kind, flux, "NONE", level=level, model=model)
    mesh, gpu, u0 = _setup(case)
    lo, hi = _box(case)
    obj = Solver.pressure_box(lo, hi)
    grad, info = gpu.adjoint(nsteps, 3, obj)
    assert np.isfinite(grad).all() and info.reverse_steps == nsteps
    # J matches the forward run and the numpy objective on the oracle's final state
    port = Port(case.config(), mesh)
    port.set_state(u0)
    port.run(nsteps, case.tau)
    J_port = pressure_box_J(case, mesh, port.get_state(), lo, hi)
    assert _rel(info.J, J_port) < 1e-12
    rng = np.random.default_rng(11)
    for trial in range(4):
        d = _direction(rng, u0, var=4 if trial % 2 else None)
        lhs = float((grad * d).sum())
        Js = []
        for sgn in (1, -1):
            gpu.set_state(u0 + sgn * FD_EPS * d)
            gpu.run(nsteps, case.tau)
            Js.append(gpu.objective(obj))
        fd = (Js[0] - Js[1]) / (2 * FD_EPS)
        assert _rel(lhs, fd) < FD_TOL, (trial, lhs, fd)
        if trial < 2:
            Jp = []
            for sgn in (1, -1):
                port.set_state(u0 + sgn * FD_EPS * d)
                port.run(nsteps, case.tau)
                Jp.append(pressure_box_J(case, mesh, port.get_state(), lo, hi))
            assert _rel(lhs, (Jp[0] - Jp[1]) / (2 * FD_EPS)) < FD_TOL


def _revolve_cost(n, s):
    """Forward steps of the optimal binomial schedule (recomputations of the
    adjoint steps themselves not counted)."""
    if n <= 1:
        return 0
    if s <= 1:
        return n * (n - 1) // 2
    t = 0
    while math.comb(s + t, s) < n:
        t += 1
    return t * n - math.comb(s + 1 + t - 1, s + 1)


@pytest.mark.parametrize("snaps", [1, 2, 3, 5, 40, 60])
def test_checkpointing_schedule(snaps):
    case = small_case("vortex", "HLLC", "NONE", level=2)
    mesh, gpu, u0 = _setup(case)
    obj = Solver.pressure_box(*_box(case))
    n = 17
    ref_grad, ref_info = gpu.adjoint(n, n, obj)
    gpu.set_state(u0)
    grad, info = gpu.adjoint(n, snaps, obj)
    # the same arithmetic whatever the schedule
    assert np.array_equal(grad, ref_grad)
    assert info.J == ref_info.J
    if snaps >= 3 * n:
        # every stage state kept: one forward sweep, no recomputation
        assert info.forward_steps == n and info.snapshots == 3 * n
    else:
        s = min(snaps, n)
        assert info.forward_steps == _revolve_cost(n, s) + n
        assert info.snapshots <= s


def test_adjoint_leaves_final_state():
    case = small_case("vortex", "HLLC", "NONE", level=2)
    mesh, gpu, u0 = _setup(case)
    gpu.adjoint(5, 2, Solver.pressure_box(*_box(case)))
    after = gpu.get_state()
    gpu.set_state(u0)
    gpu.run(5, case.tau)
    assert np.array_equal(after, gpu.get_state())


def test_adjoint_linear_functional():
    """dJdu_final given: J = <g, u(N)>."""
    case = small_case("random", "HLLC", "NONE", level=2)
    mesh, gpu, u0 = _setup(case)
    rng = np.random.default_rng(21)
    g = rng.normal(size=u0.shape)
    grad, _ = gpu.adjoint(4, 2, None, dJdu_final=g)
    d = _direction(rng, u0)
    Js = []
    for sgn in (1, -1):
        gpu.set_state(u0 + sgn * FD_EPS * d)
        gpu.run(4, case.tau)
        Js.append(float((g * gpu.get_state()).sum()))
    assert _rel(float((grad * d).sum()), (Js[0] - Js[1]) / (2 * FD_EPS)) < FD_TOL


@pytest.mark.parametrize("model", ["NS", "EULER"])
def test_adjoint_limiter_schedules_agree(model):
    """With the BJ limiter: the stored limiter scalings of the keep-everything
    mode and the recomputed ones of the checkpointed mode give the same
    gradient."""
    case = small_case("vortex", "LF", "BJ", level=2, model=model)
    mesh, gpu, u0 = _setup(case)
    obj = Solver.pressure_box(*_box(case))
    g1, _ = gpu.adjoint(6, 2, obj)
    gpu.set_state(u0)
    g2, info = gpu.adjoint(6, 18, obj)
    assert info.forward_steps == 6
    assert np.array_equal(g1, g2)


def test_adjoint_limiter_frozen_runs():
    """With the BJ limiter the adjoint differentiates the stages with the
    limiter scaling held at its forward value; where no element is limited it
    is the exact gradient."""
    case = small_case("vortex", "LF", "BJ", level=3)
    mesh, gpu, u0 = _setup(case)
    grad, info = gpu.adjoint(4, 2, Solver.pressure_box(*_box(case)))
    assert np.isfinite(grad).all()


def test_adjoint_rejects_unsupported():
    from charm_3d_gb300.abi import CharmGpuError
    case = small_case("mix2", "HLLC", "NONE", level=1)
    mesh, gpu, u0 = _setup(case)
    with pytest.raises(CharmGpuError):
        gpu.adjoint(2, 1, Solver.pressure_box((0, 0, 0), (1, 1, 1)))


def test_adjoint_matches_reference_fd_fixture():
    """dJ/du0 from the GPU adjoint against central differences of the
    reference's own solver (tests/golden/adjoint_fd_vortex.npz)."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "adjoint_fd_vortex.npz"))
    case = small_case("vortex", "HLLC", "NONE", level=3)
    mesh, gpu, u0 = _setup(case)
    # the fixture's own initial state (libm exp may differ in the last bit across hosts)
    assert np.allclose(u0, d["u0"], rtol=1e-13, atol=0.0)
    u0 = d["u0"]
    gpu.set_state(u0)
    grad, info = gpu.adjoint(int(d["steps"]), 3 * int(d["steps"]), Solver.pressure_box(d["lo"], d["hi"]))
    assert _rel(info.J, float(d["J0"])) < 1e-12
    eps = float(d["eps"])
    for k in range(d["dirs"].shape[0]):
        fd = (d["Jp"][k] - d["Jm"][k]) / (2 * eps)
        assert _rel(float((grad * d["dirs"][k]).sum()), fd) < FD_TOL, k


def test_adjoint_weighted_refine_flags():
    from charm_3d_gb300.abi import CharmGpuError
    case = small_case("vortex", "HLLC", "NONE", level=4)
    mesh, gpu, u0 = _setup(case)
    with pytest.raises(CharmGpuError):
        gpu.refine_flags_adjoint(0.01)            # no adjoint yet
    lo, hi = (4.0, 4.0, 4.0), (6.0, 6.0, 6.0)
    g, _ = gpu.adjoint(1, 3, Solver.pressure_box(lo, hi))
    gpu.set_state(u0)
    _, grad0 = gpu.refine_flags(1.0)
    h = np.stack([np.asarray(mesh.tree_len[d]) * 2.0 ** (-mesh.level.astype(np.float64)) for d in range(3)])
    vol = h[0] * h[1] * h[2]
    w = np.abs(g[4:, 0, :].sum(axis=0)) / vol
    want = grad0 * np.sqrt(w / w.mean())
    # a threshold that flags about a fifth of the weighted leaves
    crit = np.sqrt((want ** 2).sum(axis=0) / 12.0 * vol ** (5.0 / 3.0) / vol)
    max_err = float(np.quantile(crit[crit > 0], 0.8))
    flags, gw = gpu.refine_flags_adjoint(max_err)
    assert np.allclose(gw, want, rtol=1e-13, atol=0.0)
    err2 = (gw ** 2).sum(axis=0) / 12.0 * np.exp(np.log(vol) * 5.0 / 3.0)
    assert np.array_equal(flags, (err2 > max_err ** 2 * vol).astype(np.int8))
    assert flags.sum() > 0
    assert flags[w == 0].sum() == 0 and (w == 0).any()   # outside the adjoint's support: never refined
    # the weighted gradient drives the host octree's refine/coarsen callbacks:
    # flagged leaves refined, families the objective does not see coarsened
    forest = Forest(case)
    u_new = forest.adapt_state(gw, max_err, case.level - 1, case.level + 1, case.n_comp, u0)
    assert u_new.shape[2] == len(forest)
    _, lv = forest.leaves()
    assert (lv == case.level + 1).any() and (lv == case.level - 1).any()
