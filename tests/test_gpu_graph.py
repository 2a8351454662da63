"""Back-to-back steps replayed as a CUDA graph (charm_gpu_run with a fixed
dt): the same states, bit for bit, and the same launch counts as the same
steps launched one by one (the path taken while kernels are timed)."""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver

from .common import hanging_forest, small_case

pytestmark = pytest.mark.gpu


def _two(case, forest=None):
    forest = forest or Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    out = []
    for _ in range(2):
        g = Solver(case)
        g.upload(mesh)
        g.set_state(u0)
        out.append(g)
    return out


@pytest.mark.parametrize("kind,model,lim,prec", [("random", "NS", "BJ", "FP64"), ("random", "EULER", "NONE", "FP64"),
                                                 ("random", "NS", "NONE", "MIXED"), ("random", "NS", "BJ", "DW"),
                                                 ("random", "EULER", "BJ", "FP64")])
def test_graph_replay_matches_launches(kind, model, lim, prec):
    case = small_case(kind, "HLLC", lim, model=model)
    case.precision = prec
    a, b = _two(case)
    b.set_timing(True)          # kernels timed one by one: no graph
    a.reset_stats()
    b.reset_stats()
    a.run(9, case.tau)          # 4 graph launches of two steps, then one step
    b.run(9, case.tau)
    a.sync()
    b.sync()
    assert np.array_equal(a.get_state(), b.get_state())
    assert np.array_equal(a.kernel_stats()[0], b.kernel_stats()[0])
    # the cached graph serves the next run with the same dt
    a.run(4, case.tau)
    b.run(4, case.tau)
    a.sync()
    b.sync()
    assert np.array_equal(a.get_state(), b.get_state())


def test_graph_replay_on_hanging_faces_and_after_reupload():
    case = small_case("random", "HLLC", "BJ")
    forest, _ = hanging_forest(case)
    a, b = _two(case, forest)
    b.set_timing(True)
    a.run(6, case.tau)
    b.run(6, case.tau)
    a.sync()
    b.sync()
    assert np.array_equal(a.get_state(), b.get_state())
    # a new mesh drops the graph: the next run captures one for it
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    for g in (a, b):
        g.upload(mesh)
        g.set_state(u0)
        g.run(6, case.tau)
        g.sync()
    assert np.array_equal(a.get_state(), b.get_state())
