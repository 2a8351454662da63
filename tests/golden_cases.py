"""Rebuild the mesh and inputs of a tests/golden fixture (shared by CPU and GPU tests)."""
from __future__ import annotations

import json
import os

import numpy as np

from charm_3d_gb300.solver import Forest

from .common import hanging_forest, small_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["sod_lf_bj", "sod_step_lf_bj", "vortex_hllc", "walls_hllc_bj", "walls_cd", "massflow_hllc", "euler_lf_bj",
         "mix2_hllc_bj", "hanging_hllc_bj", "hanging_lf"]
# viscous / reacting Navier-Stokes (the reference's diffusion and chemistry)
VISC_NAMES = ["visc_hllc_bj", "visc_walls_lf", "visc2_hllc_hanging", "react_hllc", "react_lf_bj"]


def load(name: str):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["meta"]))
    case = small_case(meta["kind"], meta["flux"], meta["limiter"], level=meta["level"], model=meta["model"])
    forest = hanging_forest(case)[0] if meta["hanging"] else Forest(case)
    mesh = forest.flatten()
    return case, forest, mesh, d, meta


# Fixtures on general hexahedra: the sample case's ramp geometry
# (charm_3d_gb300.hexmesh.ramp_channel: 3 x 3 / 3 x 3 / 18 x 3 blocks, trees
# in random orientations) and a keystone block with every boundary type;
# name -> (mesh, case kind, flux, limiter, model, level, steps, refine)
HEX_NAMES = {
    "hex_ramp_hllc_bj": ("ramp", None, "HLLC", "BJ", "EULER", 0, 5, False),
    "hex_ramp_hanging": ("ramp", None, "HLLC", "BJ", "EULER", 0, 3, True),
    "hex_block_walls": ("block", "walls", "HLLC", "BJ", "NS", 1, 3, False),
    "hex_block_mix2_lf": ("block", "mix2", "LF", "NONE", "NS", 1, 3, False),
}
HEX_AMR_STEPS = 30


def hex_case(name: str):
    """(case, forest, mesh, u0, (vertices, tree corners, tree-face boundaries))
    of a general-hexahedron fixture, rebuilt from its name."""
    from charm_3d_gb300.hexmesh import WEDGE_PATCHES, ramp_channel, wedge_mesh

    from .hexmesh import SIDE_PATCHES, block_mesh, keystone
    if name == "hex_ramp_amr":
        geo, kind, flux, lim, model, level, refine = "ramp", None, "HLLC", "BJ", "EULER", 0, False
    else:
        geo, kind, flux, lim, model, level, _, refine = HEX_NAMES[name]
    if geo == "ramp":
        case, forest, _, _ = ramp_channel(level, 3, rotate=True, seed=9)
        m = wedge_mesh(3, rotate=True, seed=9)
        tb = m.tree_bnd(WEDGE_PATCHES)
    else:
        case = small_case(kind, flux, lim, model=model)
        m = block_mesh(3, 2, 2, rotate=True, seed=3, shape=keystone)
        tb = m.tree_bnd(SIDE_PATCHES)
        tb = np.where(tb >= 0, np.array(case.bnd_of_side, np.int8)[np.maximum(tb, 0)], -1).astype(np.int8)
        case.level = level
        forest = Forest.from_hex(m.vert, m.trees, tb, level)
    if refine:
        rng = np.random.default_rng(5)
        case.tau *= 0.5
        forest.adapt((rng.uniform(size=len(forest)) < 0.3).astype(np.int8), level, level + 1)
    mesh = forest.flatten()
    if geo == "ramp":
        # the ramp's seeded inflow state, on the (possibly refined) leaves
        rng = np.random.default_rng(4)
        T, P, V = 300.0, 101325.0, 697.7082
        rho = P * case.components[0].m / (8.31446261815324 * T)
        E = mesh.n_elem
        one = np.ones(E)
        u0 = np.zeros((case.n_var, 4, E))
        u0[:, 0, :] = case.cons_from_prim(rho * (1.0 + 0.01 * rng.uniform(-1, 1, E)), V * one, 0 * one, 0 * one,
                                          P * one)
    else:
        u0 = case.initial_state(mesh.center)
    return case, forest, mesh, u0, (m.vert, m.trees, tb)
