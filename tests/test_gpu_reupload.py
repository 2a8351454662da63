"""One handle across meshes of different sizes: the upload keeps the device
buffers that are still large enough and replaces the others.  After each
re-upload the step must equal that of a fresh handle on the same mesh
(bit-identical: same kernels, same data), for the FP64, mixed, viscous and
p2 paths, growing and shrinking."""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver

from .common import small_case

pytestmark = pytest.mark.gpu


def _variant(kind):
    if kind == "p2":
        case = small_case("visc2", "LF", "NONE", level=2)   # as the p2 step parity case
        case.p_order = 2
        case.tau *= 0.5
        return case
    return small_case(kind, "HLLC", "NONE" if kind != "walls" else "BJ", level=2)


def _fresh(case, level):
    case.level = level
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    g = Solver(case)
    g.upload(mesh)
    g.set_state(u0)
    g.run(2, case.tau)
    g.sync()
    u = g.get_state()
    g.close()
    return mesh, u0, u


@pytest.mark.parametrize("kind,prec", [("random", "FP64"), ("random", "MIXED"), ("walls", "FP64"),
                                       ("visc2", "FP64"), ("p2", "FP64"), ("p2", "MIXED")])
def test_reupload_matches_fresh_handle(kind, prec):
    case = _variant(kind)
    case.precision = prec
    shared = Solver(case)
    for level in (2, 3, 2, 3):   # grow, shrink, grow
        mesh, u0, want = _fresh(case, level)
        shared.upload(mesh)
        shared.set_state(u0)
        shared.run(2, case.tau)
        shared.sync()
        got = shared.get_state()
        assert got.shape == want.shape
        assert np.array_equal(got, want), f"level {level}"
    shared.close()
