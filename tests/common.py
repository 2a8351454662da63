"""Shared helpers for the tests: cases, meshes with hanging faces, error norms."""
from __future__ import annotations

import numpy as np

from charm_3d_gb300 import Boundary, Case, Component, Reaction, synthetic
from charm_3d_gb300.case import GAS_R
from charm_3d_gb300.solver import Forest


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def rel_max(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def ref_mass_matrix(nb: int) -> np.ndarray:
    """Mass matrix of the Taylor basis (4 or 10 functions) on the reference
    box [-1/2, 1/2]^3 of volume 1 (3-point Gauss per axis, exact)."""
    g = np.array([-0.5 * np.sqrt(0.6), 0.0, 0.5 * np.sqrt(0.6)])
    w = np.array([5.0, 8.0, 5.0]) / 18.0
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    wt = (w[:, None, None] * w[None, :, None] * w[None, None, :]).ravel()
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    phi = [np.ones_like(x), x, y, z] + ([x * x, y * y, z * z, x * y, x * z, y * z] if nb == 10 else [])
    P = np.stack(phi)
    return (P * wt) @ P.T


def rel_l2_field(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 norm over the domain of the difference of two DG fields
    (arrays [..., B, E] on a uniform mesh): sqrt(sum c^T M c) with the
    reference mass matrix, so that every basis function counts with its
    contribution to the field."""
    nb = a.shape[-2]
    M = ref_mass_matrix(nb)
    d = (a - b).reshape(-1, nb, a.shape[-1])
    r = b.reshape(-1, nb, b.shape[-1])
    num = np.einsum("vke,kl,vle->", d, M, d)
    den = np.einsum("vke,kl,vle->", r, M, r)
    return float(np.sqrt(num / max(den, 1e-300)))


def small_case(kind: str, flux: str = "LF", limiter: str = "BJ", level: int = 3, model: str = "NS") -> Case:
    """Small parity cases."""
    if kind == "sod":
        c = synthetic("sod", level=level)
    elif kind == "vortex":
        c = synthetic("vortex", level=level)
    elif kind == "random":
        c = synthetic("sod", level=level)
        c.init = "random"
        c.seed = 7
    elif kind == "walls":
        # every boundary type of the reference on one box (src/charm_bnd_cond.c)
        c = synthetic("sod", level=level)
        c.init = "random"
        c.seed = 11
        T_in = 1.0 * 0.02869409 / (1.0 * 8.31446261815324)
        c.boundaries = [Boundary("IN", "BOUND_INLET", (0.3, 0.0, 0.0, T_in, 1.0)),
                        Boundary("OUT", "BOUND_OUTLET"),
                        Boundary("SLIP", "BOUND_WALL_SLIP"),
                        Boundary("NOSLIP", "BOUND_WALL_NO_SLIP", (T_in,))]
        c.bnd_of_side = (0, 1, 2, 2, 3, 2)
    elif kind == "massflow":
        # mass-flow boundary (src/charm_bnd_cond.c:96-146) on both x faces with
        # flow direction +x: inflow at -x (total temperature, mass flux,
        # species), outflow at +x.  The state stays subsonic, so the outflow
        # branch only reads its stored pressure param[6] and never writes it
        # back (the write-back is not reproduced on the GPU or in the oracle).
        c = synthetic("sod", level=level)
        c.init = "random"
        c.seed = 29
        T_tot = 1.05 * 0.02869409 / 8.31446261815324
        c.boundaries = [Boundary("MF", "BOUND_MASS_FLOW", (0.3, 1.0, T_tot, 1.0, 0.0, 0.0, 0.95, 1.0)),
                        Boundary("OUT", "BOUND_OUTLET"),
                        Boundary("SLIP", "BOUND_WALL_SLIP")]
        c.bnd_of_side = (0, 0, 2, 2, 1, 2)
    elif kind == "mix2":
        # two species, mixture EOS (src/charm_eos.c:120-148), constant cp
        c = synthetic("sod", level=level)
        c.init = "random"
        c.seed = 5
        c.eos = "MIX"
        c.components = [Component("A", m=0.02869409, cp=(1014.16,)), Component("B", m=0.018, cp=(1850.0,))]
    elif kind in ("visc", "visc_walls", "visc2", "react"):
        # viscous / reacting unit cases on dimensionless states (T ~ 3.5e-3):
        # constant transport laws large enough to matter next to the fluxes
        c = synthetic("sod", level=level)
        c.init = "random"
        c.seed = {"visc": 13, "visc_walls": 17, "visc2": 19, "react": 23}[kind]
        c.use_visc = 1
        if kind == "visc_walls":
            T_in = 1.0 * 0.02869409 / (1.0 * 8.31446261815324)
            c.boundaries = [Boundary("IN", "BOUND_INLET", (0.3, 0.0, 0.0, T_in, 1.0)),
                            Boundary("OUT", "BOUND_OUTLET"),
                            Boundary("SLIP", "BOUND_WALL_SLIP"),
                            Boundary("NOSLIP", "BOUND_WALL_NO_SLIP", (T_in,))]
            c.bnd_of_side = (0, 1, 2, 2, 3, 2)
        if kind in ("visc2", "react"):
            c.eos = "MIX"
            c.components = [Component("A", m=0.02869409, cp=(1014.16,), h0=2.0e6, sig=3.62, ek=97.0),
                            Component("B", m=0.018, cp=(1850.0,), sig=2.64, ek=809.1)]
            c.use_diff = 1
        if kind == "react":
            # rates and heat release scaled to the dimensionless state
            c.t_ref = 0.0
            c.components[0].h0 = 1.0
            c.reactions = [Reaction(left=(0, -1, -1), right=(1, -1, -1), a=4.0, e=2.0e-3 * GAS_R, n=0.5)]
        for comp in c.components:
            comp.ml0, comp.kp0 = 0.02, 0.03
    else:
        raise ValueError(kind)
    c.flux, c.limiter, c.model = flux, limiter, model
    c.steps = 3
    if kind in ("random", "walls", "massflow", "mix2", "visc", "visc_walls", "visc2", "react"):
        # random slopes and no limiter: keep the step well inside p1 DG's CFL limit
        c.tau = 0.1 * (1.0 / 2 ** level) / 1.5
    return c


def hanging_forest(case: Case, frac: float = 0.2, seed: int = 3) -> tuple[Forest, np.ndarray]:
    """Forest of `case` with a random subset of leaves refined once and 2:1 balanced.
    Scales case.tau by 1/4 so that the finer leaves stay well inside the CFL limit."""
    f = Forest(case)
    case.tau *= 0.25
    rng = np.random.default_rng(seed)
    flags = (rng.uniform(size=len(f)) < frac).astype(np.int8)
    f.adapt(flags, case.level, case.level + 1)
    return f, flags


def amr_case(kind: str = "sod", level: int = 2, max_level: int = 4, max_err: float = 0.05, flux: str = "HLLC",
             limiter: str = "BJ") -> Case:
    """A small AMR case: refine / coarsen by the reference's criterion every `refine_period` steps."""
    c = small_case(kind, flux, limiter, level=level)
    c.max_err, c.min_level, c.max_level, c.refine_period = max_err, level, max_level, 2
    c.tau = 0.1 * (1.0 / 2 ** max_level) / 1.5
    return c


def amr_run_oracle(case: Case, steps: int):
    """The AMR time loop of charm_model_ns_timestep_single (src/models/ns/charm_model.c:197-214)
    on the oracle: adapt every refine_period steps (not at step 0), then the step."""
    from oracle.port import Port
    forest = Forest(case)
    mesh = forest.flatten()
    u = case.initial_state(mesh.center)
    for step in range(steps):
        if case.refine_period and step and step % case.refine_period == 0:
            port = Port(case.config(), mesh)
            port.set_state(u)
            u = forest.adapt_state(port.amr_grad(), case.max_err, case.min_level, case.max_level, case.n_comp, u)
            mesh = forest.flatten()
        port = Port(case.config(), mesh)
        port.set_state(u)
        port.step(case.tau)
        u = port.get_state()
    return forest, mesh, u


GAUSS_PHI = 0.28867513459481288225   # 1/(2 sqrt 3): Taylor basis at the 2x2x2 Gauss points


def pressure_box_J(case, mesh, u, lo, hi) -> float:
    """Integral of the pressure over the elements whose centre lies in [lo, hi)
    (8-point Gauss rule), the objective of charm_gpu_objective, in numpy."""
    _, gam = case.gas_constants()
    E = mesh.n_elem
    c = mesh.center
    inside = np.ones(E, bool)
    for d in range(3):
        inside &= (c[d] >= lo[d]) & (c[d] < hi[d])
    h = np.stack([np.asarray(mesh.tree_len[d]) * 2.0 ** (-mesh.level.astype(np.float64)) for d in range(3)])
    w8 = h[0] * h[1] * h[2] * 0.125
    J = 0.0
    for g in range(8):
        phi = [GAUSS_PHI if (g >> d) & 1 else -GAUSS_PHI for d in range(3)]
        U = u[:, 0, :] + phi[0] * u[:, 1, :] + phi[1] * u[:, 2, :] + phi[2] * u[:, 3, :]
        r = U[4:].sum(axis=0)
        vel = U[:3] / r
        e = U[3] / r - 0.5 * (vel * vel).sum(axis=0)
        p = r * e * (gam - 1.0)
        J += float((w8 * p)[inside].sum())
    return J


def face_sets_of_reference(faces):
    """Conforming (lower, upper, axis), hanging (lower, upper, axis, sub) and
    boundary (element, face) records of the reference's face iteration
    (p4est_iterate's face callback sides, one row per face)."""
    conf, hang_set, bnd = set(), set(), set()
    for r in faces:
        ns = r[0]
        if ns == 1:
            bnd.add((int(r[3]), int(r[1])))
            continue
        f0, h0, f1, h1 = r[1], r[2], r[7], r[8]
        assert f0 % 2 == 1 and f1 == f0 - 1, "side 0 must be the lower leaf"
        if not h0 and not h1:
            conf.add((int(r[3]), int(r[9]), int(f0 // 2)))
        elif h1:
            for k in range(4):
                hang_set.add((int(r[3]), int(r[9 + k]), int(f0 // 2), k))
        else:
            for k in range(4):
                hang_set.add((int(r[3 + k]), int(r[9]), int(f0 // 2), k))
    return conf, hang_set, bnd


def face_sets_of_mesh(mesh):
    """The same records from the flattened mesh."""
    got_c, got_h = set(), set()
    for k in range(mesh.n_face):
        a, b = (int(x) for x in mesh.face_elem[:, k])
        info = int(mesh.face_info[k])
        d, kind, sub = info & 3, (info >> 2) & 3, (info >> 4) & 3
        if kind == 0:
            got_c.add((a, b, d))
        else:
            got_h.add((a, b, d, sub))
    got_b = {(int(e), int(f)) for e, f in zip(mesh.bface_elem, mesh.bface_face)}
    return got_c, got_h, got_b
