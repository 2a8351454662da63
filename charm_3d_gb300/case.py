"""Case description: what the reference's task.yaml plus initial data describe.

A ``Case`` holds the selections the reference makes from YAML strings
(flux, limiter, EOS, model, boundary types; reference
src/charm_init_yaml.cpp:333-413), the components and boundary parameters,
the brick mesh, and a seeded initial state.  ``Case.config()`` produces the
``charm_gpu_config_t`` of include/charm_gpu.h.

``synthetic(name, level=...)`` builds the benchmark workloads:
  sod     Euler 3D Sod tube on the unit cube (LF, BJ limiter, outlet BCs)
  vortex  isentropic vortex on the periodic box [0,10]^3 (HLLC, no limiter)
  blast   spherical blast in the unit cube (HLLC, BJ limiter, outlet BCs)
Initial data set coefficient 0 of each cell (as the reference's region
initialisation does, src/charm_init.c:61-68); higher coefficients are 0.
"""
from __future__ import annotations

import dataclasses as dc
import math

import numpy as np

from . import abi

GAS_R = 8.31446261815324          # src/charm_eos.c:8
M_AIR = 0.02869409                # molar mass used by the reference's sample case
CP_AIR = 3.5 * GAS_R / M_AIR      # gamma = 1.4


@dc.dataclass
class Component:
    name: str = "AIR"
    m: float = M_AIR
    cp: tuple = (CP_AIR,)
    cp_type: str = "CONST"
    kp_type: str = "CONST"
    ml_type: str = "CONST"
    ml0: float = 0.0
    kp0: float = 0.0
    t0: float = 273.15
    ts: float = 218.0
    sig: float = 3.512
    ek: float = 139.8
    h0: float = 0.0


@dc.dataclass
class Reaction:
    """One Arrhenius reaction, k = a T^n exp(-e / (T R)); components by index, -1 = none."""
    left: tuple = (0, -1, -1)
    right: tuple = (1, -1, -1)
    a: float = 1.0e9
    e: float = 15000.0 * GAS_R
    n: float = 0.0


@dc.dataclass
class Boundary:
    name: str
    type: str = "BOUND_OUTLET"
    params: tuple = ()


SIDES = ("-x", "+x", "-y", "+y", "-z", "+z")


@dc.dataclass
class Case:
    name: str = "case"
    model: str = "NS"
    flux: str = "LF"
    limiter: str = "BJ"
    eos: str = "IDEAL"
    precision: str = "FP64"
    dt_mode: str = "TAU"
    components: list = dc.field(default_factory=lambda: [Component()])
    boundaries: list = dc.field(default_factory=lambda: [Boundary("ALL")])
    bnd_of_side: tuple = (0, 0, 0, 0, 0, 0)
    grav: tuple = (0.0, 0.0, 0.0)
    tau: float = 1.0e-3
    cfl: float = 0.3
    t_ref: float = 298.15
    brick: tuple = (1, 1, 1)
    periodic: tuple = (0, 0, 0)
    origin: tuple = (0.0, 0.0, 0.0)
    tree_len: tuple = (1.0, 1.0, 1.0)
    level: int = 3
    max_err: float = 0.01
    min_level: int = 0
    max_level: int = 0
    refine_period: int = 0
    steps: int = 10
    seed: int = 0
    init: str = "sod"          # initial-data generator name (see initial_state)
    p_order: int = 1
    use_visc: int = 0
    use_diff: int = 0
    reactions: list = dc.field(default_factory=list)
    init_args: dict = dc.field(default_factory=dict)

    @property
    def n_comp(self) -> int:
        return len(self.components)

    @property
    def n_var(self) -> int:
        return 4 + self.n_comp

    @property
    def n_basis(self) -> int:
        return 10 if self.p_order == 2 else 4

    def config(self) -> abi.Config:
        c = abi.Config()
        c.model = abi.MODEL[self.model]
        c.flux = abi.FLUX[self.flux]
        c.limiter = abi.LIMITER[self.limiter]
        c.eos = abi.EOS[self.eos]
        c.precision = abi.PRECISION[self.precision]
        c.dt_mode = abi.DT_MODE[self.dt_mode]
        c.n_comp = self.n_comp
        for i, comp in enumerate(self.components):
            cc = c.comp[i]
            cc.m, cc.ml0, cc.kp0, cc.t0, cc.ts = comp.m, comp.ml0, comp.kp0, comp.t0, comp.ts
            cc.sig, cc.ek, cc.h0 = comp.sig, comp.ek, comp.h0
            cc.cp_type = abi.CP_TYPE[comp.cp_type]
            cc.kp_type = abi.LAW[comp.kp_type]
            cc.ml_type = abi.LAW[comp.ml_type]
            cc.n_cp = len(comp.cp)
            for k, v in enumerate(comp.cp):
                cc.cp[k] = v
        c.n_bnd = len(self.boundaries)
        for i, b in enumerate(self.boundaries):
            c.bnd[i].type = abi.BND[b.type]
            for k, v in enumerate(b.params):
                c.bnd[i].params[k] = v
        for k in range(3):
            c.grav[k] = self.grav[k]
        c.tau, c.cfl, c.t_ref = self.tau, self.cfl, self.t_ref
        c.use_visc = self.use_visc
        c.use_diff = self.use_diff
        c.n_react = len(self.reactions)
        for i, r in enumerate(self.reactions):
            for k in range(3):
                c.react[i].left[k] = (list(r.left) + [-1, -1, -1])[k]
                c.react[i].right[k] = (list(r.right) + [-1, -1, -1])[k]
            c.react[i].a, c.react[i].e, c.react[i].n = r.a, r.e, r.n
        c.check_every = 0
        c.p_order = self.p_order
        return c

    # ---- thermodynamics for building initial states (reference formulas) ----
    def gas_constants(self) -> tuple[float, float]:
        """(cv, gamma) of a single-species ideal gas as charm_mat_eos_ideal computes them."""
        comp = self.components[0]
        cp = comp.cp[0]
        cv = cp - GAS_R / comp.m
        return cv, cp / cv

    def cons_from_prim(self, rho, u, v, w, p, c=None) -> np.ndarray:
        """Conserved variables [V, E] from primitive fields (single ideal gas or
        a mixture with constant cp): ru, rv, rw, re, rc_i."""
        rho = np.asarray(rho, dtype=np.float64)
        n = rho.shape[0]
        if c is None:
            c = np.zeros((self.n_comp, n))
            c[0] = 1.0
        if self.eos == "IDEAL":
            _, gam = self.gas_constants()
            gam = np.full(n, gam)
        else:
            M_ = sum(c[i] / self.components[i].m for i in range(self.n_comp))
            cp = sum(c[i] * self.components[i].cp[0] for i in range(self.n_comp))
            cv = cp - GAS_R * M_
            gam = cp / cv
        e = p / (rho * (gam - 1.0))
        out = np.empty((self.n_var, n))
        out[0] = rho * u
        out[1] = rho * v
        out[2] = rho * w
        out[3] = rho * (e + 0.5 * (u * u + v * v + w * w))
        for i in range(self.n_comp):
            out[4 + i] = rho * c[i]
        return out

    def initial_state(self, center: np.ndarray) -> np.ndarray:
        """Seeded initial state [V][B][E] for element centres center[3][E]."""
        E = center.shape[1]
        x, y, z = center
        rng = np.random.default_rng(self.seed)
        a = self.init_args
        zeros = np.zeros(E)
        if self.init == "sod":
            left = x < a.get("x0", 0.5)
            rho = np.where(left, 1.0, 0.125)
            p = np.where(left, 1.0, 0.1)
            U = self.cons_from_prim(rho, zeros, zeros, zeros, p)
        elif self.init == "vortex":
            gam = self.gas_constants()[1]
            beta = a.get("strength", 5.0)
            xc, yc = a.get("xc", 5.0), a.get("yc", 5.0)
            u0, v0 = a.get("u0", 1.0), a.get("v0", 1.0)
            dx, dy = x - xc, y - yc
            r2 = dx * dx + dy * dy
            f = np.exp(0.5 * (1.0 - r2))
            du = -beta / (2 * math.pi) * dy * f
            dv = beta / (2 * math.pi) * dx * f
            dT = -(gam - 1.0) * beta * beta / (8.0 * gam * math.pi * math.pi) * np.exp(1.0 - r2)
            rho = (1.0 + dT) ** (1.0 / (gam - 1.0))
            p = rho ** gam
            U = self.cons_from_prim(rho, u0 + du, v0 + dv, zeros, p)
            amp = a.get("noise", 1.0e-3)
            U[4] = U[4] + rng.uniform(-amp, amp, E)
        elif self.init == "blast":
            cx, cy, cz = a.get("center", (0.5, 0.5, 0.5))
            r = np.sqrt((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2)
            p = np.where(r < a.get("radius", 0.1), a.get("p_in", 1.0e3), a.get("p_out", 0.1))
            rho = np.ones(E) * (1.0 + rng.uniform(-a.get("noise", 0.01), a.get("noise", 0.01), E))
            U = self.cons_from_prim(rho, zeros, zeros, zeros, p)
        elif self.init == "flame":
            r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2)
            hot = r < a.get("radius", 0.2)
            T = np.where(hot, a.get("t_in", 1500.0), a.get("t_out", 300.0))
            T = T * (1.0 + rng.uniform(-a.get("noise", 0.01), a.get("noise", 0.01), E))
            c = np.zeros((self.n_comp, E))
            c[0] = np.where(hot, 1.0, 0.0)
            c[1] = 1.0 - c[0]
            M_ = sum(c[i] / self.components[i].m for i in range(self.n_comp))
            p = np.full(E, a.get("p", 1.0e5))
            rho = p / (GAS_R * T * M_)
            U = self.cons_from_prim(rho, zeros, zeros, zeros, p, c)
        elif self.init == "random":
            # smooth-ish random state for unit tests: all 4 coefficients set
            rho = 1.0 + 0.2 * rng.uniform(-1, 1, E)
            p = 1.0 + 0.2 * rng.uniform(-1, 1, E)
            vel = 0.3 * rng.uniform(-1, 1, (3, E))
            c = None
            if self.n_comp > 1:
                c = rng.uniform(0.05, 1.0, (self.n_comp, E))
                c /= c.sum(axis=0)
            U = self.cons_from_prim(rho, vel[0], vel[1], vel[2], p, c)
            out = np.zeros((self.n_var, self.n_basis, E))
            out[:, 0, :] = U
            slope = a.get("slope", 0.05)
            out[:, 1:4, :] = slope * rng.uniform(-1, 1, (self.n_var, 3, E)) * np.abs(U)[:, None, :]
            if self.n_basis == 10:   # second-order coefficients for p2
                out[:, 4:, :] = 0.3 * slope * rng.uniform(-1, 1, (self.n_var, 6, E)) * np.abs(U)[:, None, :]
            return np.ascontiguousarray(out)
        else:
            raise ValueError(f"unknown initial data '{self.init}'")
        out = np.zeros((self.n_var, self.n_basis, E))
        out[:, 0, :] = U
        return np.ascontiguousarray(out)

    def ref_region(self) -> dict:
        """Region parameters for the reference's own initialisation (overwritten later)."""
        cv, gam = self.gas_constants()
        return {"v": (0.0, 0.0, 0.0), "t": 300.0, "p": 1.0e5, "c": tuple([1.0] + [0.0] * (self.n_comp - 1))}


def tau_from_cfl(case: Case, U: np.ndarray, cfl: float) -> float:
    """TAU = cfl * h / max(|u| + c) of the initial state (cell-centre values)."""
    h = min(case.tree_len[d] / 2 ** case.level for d in range(3))
    cv, gam = case.gas_constants()
    rho = U[4:, 0, :].sum(axis=0)
    vel = U[0:3, 0, :] / rho
    e = U[3, 0, :] / rho - 0.5 * (vel ** 2).sum(axis=0)
    p = rho * e * (gam - 1.0)
    c = np.sqrt(gam * p / rho)
    return float(cfl * h / np.max(np.sqrt((vel ** 2).sum(axis=0)) + c))


def synthetic(name: str, level: int | None = None, **kw) -> Case:
    """Benchmark workloads with their default sizes (override with level=...)."""
    if name == "sod":
        c = Case(name="sod", model="NS", flux="LF", limiter="BJ", level=4 if level is None else level,
                 init="sod", steps=100, boundaries=[Boundary("ALL", "BOUND_OUTLET")])
        c.tau = 0.3 * (1.0 / 2 ** c.level) / math.sqrt(1.4)
    elif name == "vortex":
        c = Case(name="vortex", model="NS", flux="HLLC", limiter="NONE", level=7 if level is None else level,
                 init="vortex", steps=50, periodic=(1, 1, 1), tree_len=(10.0, 10.0, 10.0),
                 init_args={"strength": 5.0, "xc": 5.0, "yc": 5.0, "u0": 1.0, "v0": 1.0, "noise": 1.0e-3},
                 boundaries=[Boundary("ALL", "BOUND_OUTLET")])
        # max |u| + c of the freestream-dominated vortex is about 1.41 + 1.18 + vortex speed
        c.tau = 0.3 * (10.0 / 2 ** c.level) / 3.5
    elif name == "blast":
        # pressure ratio 10: at the configuration's 1e4 (p_in = 1e3) the
        # reference's own scheme stops in its first steps (HLLC wave-order
        # check, src/charm_fluxes.c:354-357), at 1e3 too, and at 1e2 right
        # after the first refinement
        c = Case(name="blast", model="NS", flux="HLLC", limiter="BJ", level=5 if level is None else level,
                 init="blast", steps=200, min_level=5, max_level=8, refine_period=10, max_err=0.1,
                 init_args={"radius": 0.1, "p_in": 1.0, "p_out": 0.1, "noise": 0.01},
                 boundaries=[Boundary("ALL", "BOUND_OUTLET")])
        c.tau = 0.2 * (1.0 / 2 ** 8) / math.sqrt(1.4 * 1.0)
    elif name == "flame":
        # reacting 2-species Navier-Stokes: hot fuel kernel (T = 1500 K, Y_A = 1,
        # r < 0.2) in 300 K air (species B), p = 1e5 Pa, unit cube; one-step
        # A -> B, a = 1e9 1/s, Ea/R = 15000 K, heat release h0_A - h0_B = 2e6 J/kg;
        # Sutherland viscosity, conductivity mu*cp/Pr with Pr = 0.72
        mu0, cp = 1.716e-5, 1004.5
        sl = dict(ml_type="SATHERLAND", kp_type="SATHERLAND", ml0=mu0, kp0=mu0 * cp / 0.72, t0=273.15, ts=110.4)
        c = Case(name="flame", model="NS", flux="HLLC", limiter="NONE", level=6 if level is None else level,
                 init="flame", steps=20, eos="MIX", use_visc=1, use_diff=1,
                 components=[Component("A", m=0.02869409, cp=(cp,), h0=2.0e6, sig=3.62, ek=97.0, **sl),
                             Component("B", m=0.02869409, cp=(cp,), h0=0.0, sig=3.62, ek=97.0, **sl)],
                 reactions=[Reaction(left=(0, -1, -1), right=(1, -1, -1), a=1.0e9, e=15000.0 * GAS_R, n=0.0)],
                 init_args={"radius": 0.2, "t_in": 1500.0, "t_out": 300.0, "p": 1.0e5, "noise": 0.01},
                 boundaries=[Boundary("ALL", "BOUND_OUTLET")])
        # acoustic limit of the hot kernel: c = sqrt(1.4 R 1500 / M) ~ 777 m/s
        c.tau = 0.05 * (1.0 / 2 ** c.level) / 777.0
    else:
        raise ValueError(f"unknown synthetic case '{name}'")
    for k, v in kw.items():
        setattr(c, k, v)
    return c
