"""Pointwise derivatives of the adjoint (charm_3d_gb300/csrc/adjoint_math.h),
built for the host, against central differences of the oracle's fluxes.

For every flux (LF, CD, HLLC), boundary type (inlet, outlet, slip and no-slip
wall) and the volume flux, the vector-Jacobian product (dq/dU)^T qb is
compared column by column with (q(U + h e_j) - q(U - h e_j)) / 2h of the
oracle, on random states that visit every HLLC case (both supersonic sides,
both star states, shocks and rarefactions)."""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np
import pytest

from charm_3d_gb300.case import GAS_R, Component
from charm_3d_gb300.solver import Forest
from oracle.port import Port

from .common import small_case

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "native"))
import build_native  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_native.build())
        P = C.c_void_p
        _lib.adj_point.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P]
        _lib.adj_bpoint.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P, P, P, P]
        _lib.adj_vpoint.argtypes = [C.c_int, P, P, P, P]
    return _lib


FLUX_ID = {"LF": 0, "HLLC": 2, "CD": 3}


def ptr(a):
    return a.ctypes.data


def make(kind="random", flux="HLLC", n_comp=1):
    case = small_case(kind, flux, "NONE", level=1)
    if n_comp == 2:
        case.components = [Component("A", m=0.02869409, cp=(1014.16,)), Component("B", m=0.018, cp=(1850.0,))]
    cfg = case.config()
    port = Port(cfg, Forest(case).flatten())
    c0 = case.components[0]
    cv = c0.cp[0] - GAS_R / c0.m
    gas = np.array([c0.cp[0] / cv, 1.0 / cv, c0.m, GAS_R, 1e-12])
    return case, port, gas


def random_states(case, rng, n, spread=1.0):
    """Conserved states with velocities from subsonic to supersonic either way."""
    V = case.n_var
    out = np.zeros((n, V))
    for i in range(n):
        rho = rng.uniform(0.3, 2.0)
        p = rng.uniform(0.2, 3.0)
        vel = rng.normal(0.0, spread, 3)
        if case.n_comp > 1:
            c = rng.uniform(0.1, 1.0, case.n_comp)
            c /= c.sum()
        else:
            c = None
        U = case.cons_from_prim(np.array([rho]), np.array([vel[0]]), np.array([vel[1]]), np.array([vel[2]]),
                                np.array([p]), None if c is None else c[:, None])
        out[i] = U[:, 0]
    return out


def unit(rng):
    n = rng.normal(size=3)
    return n / np.linalg.norm(n)


def fd_columns(f, x, h_rel=1e-6):
    cols = []
    for j in range(x.size):
        h = h_rel * max(1.0, abs(x[j]))
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        cols.append((f(xp) - f(xm)) / (2 * h))
    return np.stack(cols, axis=1)


def check(J, qb, got, what):
    want = J.T @ qb
    scale = np.abs(J).max() * np.abs(qb).max()
    err = np.abs(got - want).max() / scale
    assert err < 2e-7, f"{what}: {err:.3e}\n{got}\n{want}"


@pytest.mark.parametrize("n_comp", [1, 2])
@pytest.mark.parametrize("flux", ["LF", "CD", "HLLC"])
def test_interior_flux_vjp(flux, n_comp):
    case, port, gas = make("random", flux, n_comp)
    V = case.n_var
    rng = np.random.default_rng(100 + 10 * FLUX_ID[flux] + n_comp)
    for trial in range(60):
        spread = (0.3, 1.5, 4.0)[trial % 3]
        Ua, Ub = random_states(case, rng, 2, spread)
        n = unit(rng) if trial % 2 else np.eye(3)[trial % 3] * (1 if trial % 4 < 2 else -1)
        qb = rng.normal(size=V)
        Uab, Ubb, q = np.zeros(V), np.zeros(V), np.zeros(V)
        lib().adj_point(FLUX_ID[flux], case.n_comp, ptr(gas), ptr(Ua), ptr(Ub), ptr(n), ptr(qb), ptr(Uab), ptr(Ubb),
                        ptr(q))
        want_q = port.point_flux_cons(np.stack([Ua, Ub]), n)
        assert np.abs(q - want_q).max() <= 1e-12 * np.abs(want_q).max()
        x = np.concatenate([Ua, Ub])
        J = fd_columns(lambda x: port.point_flux_cons(x.reshape(2, V), n), x)
        check(J, qb, np.concatenate([Uab, Ubb]), f"{flux} trial {trial}")


def test_hllc_cases_visited():
    """The random states above reach all four HLLC cases and the shock branch."""
    case, port, gas = make("random", "HLLC", 1)
    rng = np.random.default_rng(112)
    seen = set()
    for trial in range(60):
        spread = (0.3, 1.5, 4.0)[trial % 3]
        Ua, Ub = random_states(case, rng, 2, spread)
        n = unit(rng) if trial % 2 else np.eye(3)[trial % 3] * (1 if trial % 4 < 2 else -1)
        # classify with the primitive states
        def pr(U):
            r = U[4:].sum()
            vel = U[:3] / r
            e = U[3] / r - 0.5 * vel @ vel
            p = r * e * (gas[0] - 1)
            return r, vel @ n, p, np.sqrt(gas[0] * p / r)
        ra, ua, pa, ca = pr(Ua)
        rb, ub, pb, cb = pr(Ub)
        ps = max(0.5 * (pa + pb) - 0.5 * (ub - ua) * 0.25 * (ra + rb) * (ca + cb), 0.0)
        g = gas[0]
        ql = 1.0 if ps <= pa else np.sqrt(1 + (g + 1) * (ps / pa - 1) / (2 * g))
        qr = 1.0 if ps <= pb else np.sqrt(1 + (g + 1) * (ps / pb - 1) / (2 * g))
        sl, sr = ua - ca * ql, ub + cb * qr
        sl, sr = min(sl, sr), max(sl, sr)
        ss = (pb - pa + ra * ua * (sl - ua) - rb * ub * (sr - ub)) / (ra * (sl - ua) - rb * (sr - ub))
        ss = min(max(ss, sl), sr)
        seen.add("supA" if sl >= 0 else "supB" if sr <= 0 else "starA" if ss >= 0 else "starB")
        if ps > pa or ps > pb:
            seen.add("shock")
    assert seen == {"supA", "supB", "starA", "starB", "shock"}


@pytest.mark.parametrize("flux", ["LF", "HLLC"])
def test_boundary_flux_vjp(flux):
    case, port, gas = make("walls", flux, 1)
    V = case.n_var
    rng = np.random.default_rng(7 + FLUX_ID[flux])
    types = [b.type for b in case.config().bnd[:case.config().n_bnd]]
    for bid, btype in enumerate(types):
        par = np.array(case.config().bnd[bid].params[:], dtype=np.float64)
        for trial in range(12):
            (U,) = random_states(case, rng, 1, (0.3, 1.0, 2.5)[trial % 3])
            d = trial % 3
            n = np.eye(3)[d] * (1.0 if trial % 2 else -1.0)
            qb = rng.normal(size=V)
            Uab, q = np.zeros(V), np.zeros(V)
            lib().adj_bpoint(FLUX_ID[flux], btype, 1, ptr(par), ptr(gas), ptr(U), ptr(n), ptr(qb), ptr(Uab), ptr(q))
            want_q = port.point_bflux_cons(bid, U, n)
            assert np.abs(q - want_q).max() <= 1e-12 * np.abs(want_q).max()
            J = fd_columns(lambda x: port.point_bflux_cons(bid, x, n), U)
            check(J, qb, Uab, f"{flux} bnd type {btype} trial {trial}")


@pytest.mark.parametrize("n_comp", [1, 2])
def test_volume_flux_vjp(n_comp):
    case, port, gas = make("random", "LF", n_comp)
    V = case.n_var
    rng = np.random.default_rng(31 + n_comp)
    for trial in range(20):
        (U,) = random_states(case, rng, 1, 1.0)
        a = rng.normal(size=(3, V))
        Uab = np.zeros(V)
        lib().adj_vpoint(case.n_comp, ptr(gas), ptr(U), ptr(np.ascontiguousarray(a)), ptr(Uab))
        J = fd_columns(lambda x: port.point_vflux(x).ravel(), U)
        check(J, a.ravel(), Uab, f"volume trial {trial}")
