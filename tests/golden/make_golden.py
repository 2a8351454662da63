"""Generate tests/golden/*.npz from the reference's own code (oracle/_ref).

Run where the reference checkout exists:  python tests/golden/make_golden.py [name ...]
Each fixture holds the initial state, the reference's residual int_* of it,
and the reference's state after `steps` calls of timestep_single_fn, on a
small brick mesh built by the host octree (identical leaves on both sides;
the script checks that).  Mesh and initial data are rebuilt from the case
name by tests/common.py, so only arrays are stored.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from charm_3d_gb300.solver import Forest  # noqa: E402
from oracle.ref import RefSolver  # noqa: E402
from tests.common import amr_case, hanging_forest, pressure_box_J, small_case  # noqa: E402
from tests.golden_cases import HEX_AMR_STEPS, HEX_NAMES, hex_case  # noqa: E402

# name: (kind, flux, limiter, model, level, steps, hanging)
FIXTURES = {
    "sod_lf_bj": ("random", "LF", "BJ", "NS", 3, 3, False),
    "sod_step_lf_bj": ("sod", "LF", "BJ", "NS", 3, 4, False),
    "vortex_hllc": ("vortex", "HLLC", "NONE", "NS", 3, 3, False),
    "walls_hllc_bj": ("walls", "HLLC", "BJ", "NS", 2, 3, False),
    "walls_cd": ("walls", "CD", "NONE", "NS", 2, 1, False),
    "massflow_hllc": ("massflow", "HLLC", "NONE", "NS", 2, 3, False),
    "euler_lf_bj": ("random", "LF", "BJ", "EULER", 3, 2, False),
    "mix2_hllc_bj": ("mix2", "HLLC", "BJ", "NS", 2, 2, False),
    "hanging_hllc_bj": ("random", "HLLC", "BJ", "NS", 2, 2, True),
    "hanging_lf": ("random", "LF", "NONE", "NS", 2, 2, True),
    # viscous terms, species diffusion and Arrhenius chemistry
    # (src/models/ns/charm_model_ns_diff*.c, charm_model_ns_chem.c)
    "visc_hllc_bj": ("visc", "HLLC", "BJ", "NS", 2, 3, False),
    "visc_walls_lf": ("visc_walls", "LF", "NONE", "NS", 2, 3, False),
    "visc2_hllc_hanging": ("visc2", "HLLC", "NONE", "NS", 2, 2, True),
    "react_hllc": ("react", "HLLC", "NONE", "NS", 2, 3, False),
    "react_lf_bj": ("react", "LF", "BJ", "NS", 2, 3, False),
}


def make(name: str) -> dict:
    kind, flux, lim, model, level, steps, hanging = FIXTURES[name]
    case = small_case(kind, flux, lim, level=level, model=model)
    variant = "patched" if hanging else "ref"
    if hanging:
        forest, flags = hanging_forest(case)   # also scales case.tau for the finer leaves
        ref = RefSolver(case, variant)
        n = ref.refine_flags(flags, case.level + 1)
        q, lv = forest.leaves()
        rl = ref.leaves()
        assert n == len(forest), (n, len(forest))
        assert (rl[:, :4] == q).all() and (rl[:, 4] == lv).all(), "reference forest differs from host octree"
    else:
        ref = RefSolver(case, variant)
        forest = Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    ref.set_state(u0)
    res = ref.residual()
    ref.set_state(u0)
    dt = ref.run(steps)
    out = ref.get_state()
    return {"u0": u0, "residual": res, "state": out, "steps": np.array(steps), "dt": np.array(dt),
            "meta": np.array(json.dumps({"kind": kind, "flux": flux, "limiter": lim, "model": model, "level": level,
                                         "steps": steps, "hanging": hanging, "variant": variant}))}


def point_fluxes() -> dict:
    """Reference LF/HLLC/CD fluxes for random state pairs and random unit normals, and its exact Riemann solver."""
    rng = np.random.default_rng(2024)
    n = 64
    prim = np.stack([rng.uniform(0.2, 2.0, n), rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n),
                     rng.uniform(-1.5, 1.5, n), rng.uniform(0.2, 2.0, n)], axis=1)
    prim2 = np.stack([prim, np.roll(prim, 7, axis=0) * rng.uniform(0.8, 1.2, (n, 5))], axis=1)   # [n,2,5]
    normals = rng.normal(size=(n, 3))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    normals[:6] = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float)
    out = {"prim2": prim2, "normals": normals}
    for flux in ("LF", "HLLC", "CD"):
        case = small_case("random", flux, "NONE", level=1)
        ref = RefSolver(case)
        out[flux] = np.stack([ref.point_flux(prim2[i].ravel(), normals[i]) for i in range(n)])
    # Godunov: the reference's flux function is a stub, so the fixture holds
    # its exact solver rim_orig on the same pairs (face frame) and the flux
    # assembled from that solution; plus rim_orig on a wide set of states
    from oracle import ref as ref_mod
    rin = rim_inputs(prim2, normals)
    rout = ref_mod.rim(rin)
    out["GODUNOV"] = np.stack([godunov_from_rim(prim2[i], normals[i], rout[i]) for i in range(n)])
    out["rim_in"] = rim_cases()
    out["rim_out"] = ref_mod.rim(out["rim_in"])
    return out


GAM = 1.4


def _frame(n: np.ndarray) -> np.ndarray:
    """Rows n, t1, t2 of the face frame of charm_calc_flux_hllc (src/charm_fluxes.c:458-488)."""
    nt = np.zeros((3, 3))
    nt[0] = n
    ri = np.hypot(n[0], n[1])
    if ri > 1e-12:
        nt[1] = (-n[1] / ri, n[0] / ri, 0.0)
    else:
        ri = np.hypot(n[1], n[2])
        if ri > 1e-12:
            nt[1] = (0.0, -n[2] / ri, n[1] / ri)
        else:
            ri = np.hypot(n[0], n[2])
            nt[1] = (-n[2] / ri, 0.0, n[0] / ri)
    nt[2] = np.cross(nt[0], nt[1])
    return nt


def godunov_from_rim(prim2: np.ndarray, n: np.ndarray, rim_out: np.ndarray) -> np.ndarray:
    """The Godunov flux (the commented sketch of charm_calc_flux_godunov,
    src/charm_fluxes.c:182-253, one species) assembled from the face-frame
    solution (r e p u v w) of the exact solver."""
    nt = _frame(n)
    ri, ei, pi = rim_out[:3]
    uu = rim_out[3:]
    uv = nt.T @ uu
    qr = ri * uu[0]
    q = np.empty(5)
    q[:3] = qr * uv + pi * n
    q[3] = (ri * (ei + 0.5 * (uv @ uv)) + pi) * uu[0]
    q[4] = qr
    return q


def rim_inputs(prim2: np.ndarray, normals: np.ndarray) -> np.ndarray:
    """Exact-solver inputs (rL pL uL vL wL rR pR uR vR wR gam) of state pairs [n][2][r u v w p] in the face frame."""
    rows = []
    for k in range(prim2.shape[0]):
        nt = _frame(normals[k])
        row = []
        for s in range(2):
            r, u, v, w, p = prim2[k, s]
            row += [r, p] + list(nt @ np.array([u, v, w]))
        rows.append(row + [GAM])
    return np.array(rows)


def rim_cases() -> np.ndarray:
    """Inputs of the exact Riemann solver over a wide range of states (all
    wave patterns: shocks, rarefactions, fans across x/t = 0, supersonic
    flow either way), no vacuum."""
    rng = np.random.default_rng(4242)
    n = 512
    r = np.exp(rng.uniform(np.log(0.1), np.log(10.0), (n, 2)))
    p = np.exp(rng.uniform(np.log(0.01), np.log(100.0), (n, 2)))
    u = rng.uniform(-6.0, 6.0, (n, 2))
    vt = rng.uniform(-1.0, 1.0, (n, 2, 2))
    c = np.sqrt(GAM * p / r)
    keep = (u[:, 1] - u[:, 0]) < 2.0 * (c[:, 0] + c[:, 1]) / (GAM - 1.0) - 1e-3
    rows = np.concatenate([r[:, :1], p[:, :1], u[:, :1], vt[:, 0], r[:, 1:], p[:, 1:], u[:, 1:], vt[:, 1],
                           np.full((n, 1), GAM)], axis=1)
    return rows[keep]


ADJ_EPS = 1e-6
ADJ_STEPS = 10


def adjoint_fd() -> dict:
    """Central differences of J = integral of p over the middle half of the
    box after ADJ_STEPS steps of the reference (vortex, level 3, HLLC, no
    limiter), along 4 seeded directions on the density mean of every element:
    the finite-difference side of the adjoint check, through the reference."""
    case = small_case("vortex", "HLLC", "NONE", level=3)
    ref = RefSolver(case)
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    lo = [o + 0.25 * b * t for o, b, t in zip(case.origin, case.brick, case.tree_len)]
    hi = [o + 0.75 * b * t for o, b, t in zip(case.origin, case.brick, case.tree_len)]
    rng = np.random.default_rng(77)
    dirs = np.zeros((4,) + u0.shape)
    dirs[:, 4, 0, :] = rng.uniform(-1.0, 1.0, (4, mesh.n_elem))

    def J(u):
        ref.set_state(u)
        ref.run(ADJ_STEPS)
        return pressure_box_J(case, mesh, ref.get_state(), lo, hi)

    Jp = np.array([J(u0 + ADJ_EPS * d) for d in dirs])
    Jm = np.array([J(u0 - ADJ_EPS * d) for d in dirs])
    return {"u0": u0, "dirs": dirs, "Jp": Jp, "Jm": Jm, "J0": np.array(J(u0)), "eps": np.array(ADJ_EPS),
            "steps": np.array(ADJ_STEPS), "lo": np.array(lo), "hi": np.array(hi)}


# name: (kind, max_err, minlevel, level): one charm_adapt of the seeded state
AMR_ADAPT = {
    "amr_adapt_sod": ("sod", 0.05, 1, 2),
    "amr_adapt_random": ("random", 0.3, 1, 2),
    "amr_adapt_walls": ("walls", 0.2, 1, 2),
}
AMR_LOOP_STEPS = 7


def amr_adapt(name: str) -> dict:
    """The reference's charm_adapt (src/charm_amr.c:575-610; refine and
    coarsen by the gradient estimate, 2:1 balance, projections; patched
    limiter variant for the hanging faces) on a seeded state: its leaves
    (tree, x, y, z, level) and the projected state."""
    kind, max_err, minl, level = AMR_ADAPT[name]
    case = small_case(kind, "HLLC", "BJ", level=level)
    case.max_err, case.min_level, case.max_level = max_err, minl, level + 2
    ref = RefSolver(case, "patched")
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    ref.set_state(u0)
    ref.adapt()
    return {"u0": u0, "leaves": ref.leaves(), "state": ref.get_state(),
            "meta": np.array(json.dumps({"kind": kind, "max_err": max_err, "min_level": minl, "level": level}))}


def amr_loop() -> dict:
    """AMR_LOOP_STEPS steps of the reference's time loop with an adapt every
    2 steps (charm_model_ns_timestep_single, src/models/ns/charm_model.c:197-214)
    on the small Sod AMR case: final leaves and state."""
    case = amr_case("sod", level=2, max_level=4, max_err=0.05)
    ref = RefSolver(case, "patched")
    m0 = Forest(case).flatten()
    u0 = case.initial_state(m0.center)
    ref.set_state(u0)
    ref.run(AMR_LOOP_STEPS)
    return {"u0": u0, "leaves": ref.leaves(), "state": ref.get_state(), "steps": np.array(AMR_LOOP_STEPS)}


def mesh_faces() -> dict:
    """The reference's face iteration (p4est_iterate face callback sides) on
    the level-2 brick, uniform and with the seeded hanging refinement."""
    case = small_case("random", "LF", "NONE", level=2)
    uniform = RefSolver(case).faces()
    forest, flags = hanging_forest(case)
    ref = RefSolver(case, "patched")
    assert ref.refine_flags(flags, case.level + 1) == len(forest)
    return {"faces_uniform": uniform, "faces_hanging": ref.faces()}


def cell_fields() -> dict:
    """The reference's output fields (src/charm_output.c:10-52) of the seeded
    states of three small cases: one species, two species (MIX EOS), the
    vortex after two steps."""
    out = {}
    for key, (kind, steps) in {"random": ("random", 0), "mix2": ("mix2", 0), "vortex": ("vortex", 2)}.items():
        case = small_case(kind, "HLLC", "NONE", level=2)
        ref = RefSolver(case)
        mesh = Forest(case).flatten()
        u0 = case.initial_state(mesh.center)
        ref.set_state(u0)
        if steps:
            ref.run(steps)
        out[key + "_u"] = ref.get_state()
        out[key + "_fields"] = ref.cell_fields()
    return out


def hex_fixture(name: str) -> dict:
    """The reference's own code on general hexahedra (its connectivity of
    one tree per hexahedron, the trilinear geometry of src/charm_geom.c):
    residual and steps of tests/golden_cases.HEX_NAMES, or (hex_ramp_amr)
    HEX_AMR_STEPS steps of its AMR time loop on the ramp with the sample
    case's controls (MAX_ERROR 0.01, MAX_LEVEL 1, REFINE_PERIOD 10)."""
    case, forest, mesh, u0, (vert, t2v, tb) = hex_case(name)
    if name == "hex_ramp_amr":
        case.max_err, case.min_level, case.max_level, case.refine_period = 0.01, 0, 1, 10
        ref = RefSolver(case, "patched", hexmesh=(vert, t2v, tb))
        ref.set_state(u0)
        ref.run(HEX_AMR_STEPS)
        return {"u0": u0, "leaves": ref.leaves(), "state": ref.get_state(), "steps": np.array(HEX_AMR_STEPS)}
    geo, kind, flux, lim, model, level, steps, refine = HEX_NAMES[name]
    ref = RefSolver(case, "patched" if refine else "ref", hexmesh=(vert, t2v, tb))
    if refine:
        rng = np.random.default_rng(5)
        flags = (rng.uniform(size=int(ref.n_elem)) < 0.3).astype(np.int8)
        assert ref.refine_flags(flags, level + 1) == len(forest)
    q, lv = forest.leaves()
    rl = ref.leaves()
    assert (rl[:, :4] == q).all() and (rl[:, 4] == lv).all(), "reference forest differs from host octree"
    ref.set_state(u0)
    res = ref.residual()
    ref.set_state(u0)
    dt = ref.run(steps)
    return {"u0": u0, "residual": res, "state": ref.get_state(), "steps": np.array(steps), "dt": np.array(dt)}


def main(names: list[str]) -> None:
    """All fixtures, or only the ones named on the command line."""
    for name in FIXTURES:
        if names and name not in names:
            continue
        d = make(name)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, d["u0"].shape, "dt", float(d["dt"]))
    if not names or "point_fluxes" in names:
        np.savez_compressed(os.path.join(HERE, "point_fluxes.npz"), **point_fluxes())
        print("point_fluxes")
    for name in AMR_ADAPT:
        if not names or name in names:
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **amr_adapt(name))
            print(name)
    if not names or "mesh_faces" in names:
        np.savez_compressed(os.path.join(HERE, "mesh_faces.npz"), **mesh_faces())
        print("mesh_faces")
    if not names or "amr_loop_sod" in names:
        np.savez_compressed(os.path.join(HERE, "amr_loop_sod.npz"), **amr_loop())
        print("amr_loop_sod")
    if not names or "cell_fields" in names:
        np.savez_compressed(os.path.join(HERE, "cell_fields.npz"), **cell_fields())
        print("cell_fields")
    for name in list(HEX_NAMES) + ["hex_ramp_amr"]:
        if not names or name in names:
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **hex_fixture(name))
            print(name)
    if not names or "adjoint_fd_vortex" in names:
        np.savez_compressed(os.path.join(HERE, "adjoint_fd_vortex.npz"), **adjoint_fd())
        print("adjoint_fd_vortex")


if __name__ == "__main__":
    main(sys.argv[1:])
