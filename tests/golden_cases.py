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
