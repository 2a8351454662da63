"""The GPU model plugin (drop-in timestep_single_fn) against the reference's own types.

charm_3d_gb300/csrc/plugin/charm_model_gpu.c is compiled with the
reference's headers and p4est (the shim), then its flattening through
p4est_iterate and its configuration from charm_ctx_t are compared with the
host octree's flattening and with Case.config().  No GPU calls.
"""
import ctypes as C

import numpy as np
import pytest

from charm_3d_gb300 import abi
from charm_3d_gb300.solver import Forest
from oracle.ref import RefSolver

from .common import hanging_forest, small_case

pytestmark = pytest.mark.reference


def _faces(mesh):
    fe = mesh.face_elem
    return sorted(zip(fe[0].tolist(), fe[1].tolist(), mesh.face_info.tolist()))


@pytest.mark.parametrize("kind,hang", [("random", False), ("walls", False), ("random", True)])
def test_plugin_flatten_matches_host_octree(kind, hang):
    case = small_case(kind, "HLLC", "BJ", level=2)
    if hang:
        forest, flags = hanging_forest(case)
        ref = RefSolver(case, "plugin")
        ref.refine_flags(flags, case.level + 1)
    else:
        forest = Forest(case)
        ref = RefSolver(case, "plugin")
    want = forest.flatten()
    got = ref.plugin_flatten()
    assert got.n_elem == want.n_elem
    assert np.array_equal(got.level, want.level)
    assert np.allclose(got.center, want.center, rtol=0, atol=1e-15)
    assert got.tree_len == want.tree_len
    assert _faces(got) == _faces(want)
    bg = sorted(zip(got.bface_elem.tolist(), got.bface_face.tolist(), got.bface_bnd.tolist()))
    bw = sorted(zip(want.bface_elem.tolist(), want.bface_face.tolist(), want.bface_bnd.tolist()))
    assert bg == bw


@pytest.mark.parametrize("kind,flux,lim", [("walls", "HLLC", "BJ"), ("mix2", "LF", "NONE"), ("random", "CD", "BJ")])
def test_plugin_config_matches_case(kind, flux, lim):
    case = small_case(kind, flux, lim, level=1)
    ref = RefSolver(case, "plugin")
    got = ref.plugin_config(abi.PRECISION["FP64"])
    want = case.config()
    want.model = abi.MODEL["NS"]
    assert bytes(got) == bytes(want)
