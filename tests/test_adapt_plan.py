"""The adapt without the state (charm_host_forest_adapt_plan): the same
forest as charm_host_forest_adapt_state, and its projection plan, applied
with the host's arithmetic (numpy, one rounding per operation as the host
C code without FMA contraction), gives the state adapt_state projects, bit
for bit.  Cases that refine, coarsen and need balance ripples.  CPU only
(the device applies the same plan: tests/test_gpu_adapt_plan.py)."""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest
from oracle.port import Port

from .common import small_case


def apply_plan(plan, u: np.ndarray) -> np.ndarray:
    """The passes of an AdaptPlan on a state [V][4][E] (the host octree's
    project_down / project_up, in the same order of operations)."""
    for p in range(plan.n_pass):
        Eo = plan.n_out[p]
        m = np.ctypeslib.as_array(plan.map[p], (2 * Eo,)).reshape(Eo, 2)
        src, op = m[:, 0].astype(np.int64), m[:, 1]
        V = u.shape[0]
        out = np.empty((V, 4, Eo))
        cp, dn, up = op < 0, (op >= 0) & (op < 8), op == 8
        out[:, :, cp] = u[:, :, src[cp]]
        if dn.any():
            s, c = src[dn], op[dn]
            o = [np.where((c >> d) & 1, 0.25, -0.25) for d in range(3)]
            x = u[:, 0, s] + o[0] * u[:, 1, s]
            x = x + o[1] * u[:, 2, s]
            x = x + o[2] * u[:, 3, s]
            out[:, 0, dn] = x
            out[:, 1:, dn] = 0.5 * u[:, 1:, s]
        if up.any():
            s = src[up]
            mm = np.zeros((V, s.size))
            sk = np.zeros((V, 3, s.size))
            for i in range(8):
                c0 = u[:, 0, s + i]
                mm = mm + c0
                for d in range(3):
                    sg = 0.375 if (i >> d) & 1 else -0.375
                    sk[:, d] = sk[:, d] + (sg * c0 + u[:, d + 1, s + i] * (1.0 / 16.0))
            out[:, 0, up] = mm * 0.125
            out[:, 1:, up] = sk
        u = out
    return u


@pytest.mark.parametrize("kind,max_err,minl,level,rounds", [("sod", 0.05, 1, 2, 3), ("random", 0.3, 1, 2, 3),
                                                             ("random", 0.6, 1, 3, 2), ("mix2", 0.3, 1, 2, 3)])
def test_adapt_plan_matches_adapt_state(kind, max_err, minl, level, rounds):
    case = small_case(kind, "HLLC", "BJ", level=level)
    fa, fb = Forest(case), Forest(case)
    mesh = fa.flatten()
    u = case.initial_state(mesh.center)
    V = case.n_var
    for r in range(rounds):
        port = Port(case.config(), mesh)
        port.set_state(u)
        grad = port.amr_grad()
        port.close()
        rho = u[4:V, 0].sum(axis=0) if V > 5 else u[4, 0].copy()
        n_a = len(fa)
        ua = fa.adapt_state(grad, max_err, minl, level + 2, case.n_comp, u)
        n_b, plan = fb.adapt_plan(grad, rho, max_err, minl, level + 2)
        assert plan.n_in == n_a
        qa, la = fa.leaves()
        qb, lb = fb.leaves()
        assert n_b == len(fa) and (qa == qb).all() and (la == lb).all()
        ub = apply_plan(plan, u)
        assert ub.shape == ua.shape
        assert np.array_equal(ub, ua), f"adapt {r}"
        mesh = fa.flatten()
        u = ua


def test_adapt_plan_balance_ripples():
    """A point refined three times in a row: the second and third adapts need
    2:1 balance ripples (passes after the refine pass)."""
    case = small_case("random", "HLLC", "BJ", level=2)
    fa, fb = Forest(case), Forest(case)
    mesh = fa.flatten()
    u = case.initial_state(mesh.center)
    V = case.n_var
    ripple = 0
    for r in range(3):
        # refine the leaf holding the point (0.30, 0.30, 0.30)
        d = np.abs(mesh.center - 0.30).max(axis=0)
        grad = np.zeros((3, mesh.n_elem))
        grad[0, int(np.argmin(d))] = 1.0e6
        rho = u[4:V, 0].sum(axis=0)
        ua = fa.adapt_state(grad, 0.01, 1, 6, case.n_comp, u)
        n_b, plan = fb.adapt_plan(grad, rho, 0.01, 1, 6)
        qa, la = fa.leaves()
        qb, lb = fb.leaves()
        assert n_b == len(fa) and (qa == qb).all() and (la == lb).all()
        ub = apply_plan(plan, u)
        assert np.array_equal(ub, ua), f"adapt {r}"
        ripple += max(0, plan.n_pass - 1)
        mesh = fa.flatten()
        u = ua
    assert ripple > 0


def test_restricted_ripples_equal_full_balance():
    """adapt_state's balance passes after the first check only the new
    leaves and their face neighbours; the forest must be the one the full
    ripple (charm_forest_balance, every leaf every pass) gives: refine the
    leaf at a point four times in a row (ripples of several passes)."""
    case = small_case("sod", "HLLC", "BJ", level=2)
    fa, fb = Forest(case), Forest(case)
    for r in range(4):
        mesh = fa.flatten()
        d = np.abs(mesh.center - 0.37).max(axis=0)
        i = int(np.argmin(d))
        grad = np.zeros((3, mesh.n_elem))
        grad[0, i] = 1.0e9
        u = np.ones((case.n_var, 4, mesh.n_elem))
        fa.adapt_state(grad, 0.01, 9, 9, case.n_comp, u)   # minlevel 9: nothing coarsens
        flags = np.zeros(mesh.n_elem, np.int8)
        flags[i] = 1
        fb.adapt(flags, 9, 9)
        qa, la = fa.leaves()
        qb, lb = fb.leaves()
        assert len(fa) == len(fb) and (qa == qb).all() and (la == lb).all(), f"adapt {r}"
    assert int(la.max()) - int(la.min()) >= 4


def test_adapt_plan_matches_adapt_state_on_large_meshes():
    """Meshes of 30-190 k leaves (the refine and coarsen passes run in blocks
    of 4096 leaves on several threads, families straddle block edges): a
    spherical front of refine flags moving outward, so every adapt refines,
    coarsens and ripples; plan and state forms agree bit for bit."""
    from charm_3d_gb300 import synthetic
    case = synthetic("blast")
    fa, fb = Forest(case), Forest(case)
    mesh = fa.flatten()
    rng = np.random.default_rng(5)
    u = rng.standard_normal((case.n_var, 4, mesh.n_elem)) * 0.1
    u[4, 0] += 1.0
    coarsened = 0
    for it in range(5):
        r = np.sqrt(((mesh.center - 0.5) ** 2).sum(axis=0))
        g = np.zeros((3, mesh.n_elem))
        g[0] = np.where(np.abs(r - 0.1 - 0.01 * it) < 0.03, 50.0, 0.0)
        rho = u[4:, 0].sum(axis=0)
        ua = fa.adapt_state(g, case.max_err, case.min_level, case.max_level, case.n_comp, u)
        n, plan = fb.adapt_plan(g, rho, case.max_err, case.min_level, case.max_level)
        qa, la = fa.leaves()
        qb, lb = fb.leaves()
        assert n == len(fa) and (qa == qb).all() and (la == lb).all()
        assert np.array_equal(apply_plan(plan, u), ua), f"adapt {it}"
        for p in range(plan.n_pass):
            m = np.ctypeslib.as_array(plan.map[p], (2 * plan.n_out[p],))
            coarsened += int((m[1::2] == 8).sum())
        mesh = fa.flatten()
        u = ua
    assert mesh.n_elem > 4 * 4096 and coarsened > 0


@pytest.mark.parametrize("seed", [0, 1])
def test_plan_driven_by_flags_is_the_flag_adapt(seed):
    """charm_host_forest_adapt_plan_flags (refine +1, coarsen families of -1,
    balance) gives the forest of charm_host_forest_adapt with the same
    flags, and its plan carries the mass of a state (the p1 projections
    keep it up to rounding)."""
    case = small_case("random", "HLLC", "BJ", level=3)
    rng = np.random.default_rng(seed)
    pre = (rng.uniform(size=8 ** 3) < 0.3).astype(np.int8)
    a, b = Forest(case), Forest(case)
    a.adapt(pre, 2, 5)   # a mesh with mortars
    b.adapt(pre, 2, 5)
    n = len(a)
    lv0 = a.leaves()[1]
    flags = rng.choice(np.array([-1, 0, 1], np.int8), size=n, p=[0.6, 0.3, 0.1])
    u = case.initial_state(a.flatten().center)
    a.adapt(flags, 2, 5)
    n_new, plan = b.adapt_plan_flags(flags, 2, 5)
    qa, la = a.leaves()
    qb, lb = b.leaves()
    assert n_new == len(a) and np.array_equal(qa, qb) and np.array_equal(la, lb)
    assert plan.n_in == n and n_new != n
    w = apply_plan(plan, u)

    def mass(x, lv):
        return float((x[4, 0] * 8.0 ** (-lv.astype(np.float64))).sum())

    assert abs(mass(w, lb) - mass(u, lv0)) < 1e-13 * mass(u, lv0)
