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


@pytest.mark.parametrize("kind,flux,lim,model", [("walls", "HLLC", "BJ", "NS"), ("mix2", "LF", "NONE", "NS"),
                                                 ("random", "CD", "BJ", "NS"), ("random", "HLLC", "BJ", "EULER")])
def test_plugin_config_matches_case(kind, flux, lim, model):
    """The model comes from the step the reference's model init registered
    (forward Euler for charm_model_euler_init, SSP-RK3 for the NS model)."""
    case = small_case(kind, flux, lim, level=1, model=model)
    ref = RefSolver(case, "plugin")
    got = ref.plugin_config(abi.PRECISION["FP64"])
    want = case.config()
    assert want.model == abi.MODEL[model]
    if model == "EULER":
        want.t_ref = 0.0   # ctx->model.ns is not the Euler model's member (t_ref is unused on its step)
    assert bytes(got) == bytes(want)


def _hex_faces(mesh):
    fe, ff = mesh.face_elem, mesh.face_face
    kind = (mesh.face_info >> 2) & 3
    return sorted(zip(fe[0].tolist(), fe[1].tolist(), ff[0].tolist(), ff[1].tolist(), kind.tolist()))


@pytest.mark.parametrize("name", ["hex_ramp_hllc_bj", "hex_ramp_hanging", "hex_block_walls"])
def test_plugin_takes_general_hexahedra_from_p4est(name):
    """On the tree-per-hexahedron forest of an unstructured mesh the plugin
    switches to the general-hexahedron form: p4est's face sides (side 0
    gives the normal) with both faces, and every leaf's corners from
    p4est_qcoord_to_vertex; the same records as the host octree's
    flatten, the same corners."""
    from .golden_cases import HEX_NAMES, hex_case
    case, forest, mesh, _, (vert, t2v, tb) = hex_case(name)
    ref = RefSolver(case, "plugin", hexmesh=(vert, t2v, tb))
    if HEX_NAMES[name][7]:
        rng = np.random.default_rng(5)
        ref.refine_flags((rng.uniform(size=int(ref.n_elem)) < 0.3).astype(np.int8), HEX_NAMES[name][5] + 1)
    is_hex, got = ref.plugin_flatten_hex()
    assert is_hex
    assert got.n_elem == mesh.n_elem
    assert np.allclose(got.vertex, mesh.vertex, rtol=1e-14, atol=1e-12)
    assert _hex_faces(got) == _hex_faces(mesh)
    bg = sorted(zip(got.bface_elem.tolist(), got.bface_face.tolist(), got.bface_bnd.tolist()))
    bw = sorted(zip(mesh.bface_elem.tolist(), mesh.bface_face.tolist(), mesh.bface_bnd.tolist()))
    assert bg == bw


def test_plugin_keeps_the_box_form_on_bricks():
    case = small_case("random", "HLLC", "BJ", level=2)
    ref = RefSolver(case, "plugin")
    is_hex, _ = ref.plugin_flatten_hex()
    assert not is_hex


def test_plugin_init_again_and_finish_release_what_it_holds():
    """charm_model_gpu_init a second time releases the flattened arrays of
    the first (no handle exists before a step, so nothing reaches a GPU),
    and charm_model_gpu_finalize releases the rest; the flattening still
    works between them."""
    case = small_case("random", "HLLC", "BJ", level=2)
    ref = RefSolver(case, "plugin")
    first = _faces(ref.plugin_flatten())
    ref.plugin_use_gpu(abi.PRECISION["FP64"])
    again = _faces(ref.plugin_flatten())
    ref.plugin_use_gpu(abi.PRECISION["FP64"])
    assert ref.plugin_finish() == 0
    assert first == again
