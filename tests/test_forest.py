"""Host octree and flattening: checked against a brute-force geometric face matcher.

Connectivity must be exact: every face of every leaf appears exactly once,
as a conforming face, one of four mortar sub-faces, or a boundary face, with
p4est's side order (side 0 at the lower coordinate).
"""
import itertools

import numpy as np
import pytest

from charm_3d_gb300 import Case
from charm_3d_gb300.solver import Forest

from .common import hanging_forest


def boxes(forest, case):
    q, lv = forest.leaves()
    nt = np.array(case.brick)
    t = q[:, 3]
    ti = np.stack([t % nt[0], (t // nt[0]) % nt[1], t // (nt[0] * nt[1])], axis=1)
    R = 1 << 19
    lo = ti * R + q[:, :3]
    ln = (1 << (19 - lv.astype(np.int64)))
    return lo.astype(np.int64), ln.astype(np.int64), lv


def brute_force_faces(forest, case):
    """All face adjacencies from box geometry (integer coordinates, O(E^2))."""
    lo, ln, lv = boxes(forest, case)
    E = len(ln)
    ext = np.array(case.brick, np.int64) * (1 << 19)
    conf, hang, bnd = set(), set(), set()
    for i in range(E):
        for d in range(3):
            s, t = [a for a in range(3) if a != d]
            # + side of i
            x = lo[i, d] + ln[i]
            wrap = False
            if x == ext[d]:
                if case.periodic[d]:
                    x, wrap = 0, True
                else:
                    bnd.add((i, 2 * d + 1))
            if lo[i, d] == 0 and not case.periodic[d]:
                bnd.add((i, 2 * d))
            if x == ext[d] and not case.periodic[d]:
                continue
            for j in range(E):
                if lo[j, d] != x:
                    continue
                # tangential overlap with positive area
                if lo[j, s] >= lo[i, s] + ln[i] or lo[i, s] >= lo[j, s] + ln[j]:
                    continue
                if lo[j, t] >= lo[i, t] + ln[i] or lo[i, t] >= lo[j, t] + ln[j]:
                    continue
                if ln[i] == ln[j]:
                    conf.add((i, j, d))
                else:
                    hang.add((i, j, d))
    return conf, hang, bnd


def flattened_faces(mesh):
    conf, hang, bnd = set(), set(), set()
    for k in range(mesh.n_face):
        a, b = int(mesh.face_elem[0, k]), int(mesh.face_elem[1, k])
        info = int(mesh.face_info[k])
        d, kind = info & 3, (info >> 2) & 3
        (conf if kind == 0 else hang).add((a, b, d))
    for k in range(mesh.n_bface):
        bnd.add((int(mesh.bface_elem[k]), int(mesh.bface_face[k])))
    return conf, hang, bnd


CASES = [Case(level=2), Case(level=2, periodic=(1, 1, 1)), Case(level=1, brick=(2, 3, 1)),
         Case(level=1, brick=(3, 1, 2), periodic=(1, 0, 1))]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("refine", [False, True])
def test_flatten_matches_brute_force(case, refine):
    forest = hanging_forest(case, frac=0.25, seed=9)[0] if refine else Forest(case)
    mesh = forest.flatten()
    got = flattened_faces(mesh)
    want = brute_force_faces(forest, case)
    assert got[0] == want[0]
    assert got[1] == want[1]
    assert got[2] == want[2]
    # every face record appears once
    assert mesh.n_face == len(got[0]) + len(got[1])
    assert mesh.n_bface == len(got[2])


@pytest.mark.parametrize("level,per", [(3, 0), (3, 1)])
def test_uniform_counts(level, per):
    case = Case(level=level, periodic=(per, per, per))
    mesh = Forest(case).flatten()
    N = 2 ** level
    assert mesh.n_elem == N ** 3
    assert mesh.n_face == (3 * N ** 3 if per else 3 * N * N * (N - 1))
    assert mesh.n_bface == (0 if per else 6 * N * N)
    assert ((mesh.face_info >> 6) & 1).sum() == (3 * N * N if per else 0)


def test_mortar_records_are_consecutive_and_ordered():
    case = Case(level=2)
    mesh = hanging_forest(case, frac=0.3, seed=1)[0].flatten()
    info = mesh.face_info
    kind, sub = (info >> 2) & 3, (info >> 4) & 3
    idx = np.nonzero(kind > 0)[0]
    assert idx.size % 4 == 0 and idx.size > 0
    for k in range(0, idx.size, 4):
        blk = idx[k:k + 4]
        assert (np.diff(blk) == 1).all()
        assert list(sub[blk]) == [0, 1, 2, 3]
        big = [mesh.face_elem[1 if kind[j] == 1 else 0, j] for j in blk]
        assert len(set(big)) == 1


def test_balance_is_two_to_one_after_deep_refinement():
    case = Case(level=1)
    f = Forest(case)
    for _ in range(4):   # keep refining the leaf at the origin corner
        q, lv = f.leaves()
        flags = np.zeros(len(f), np.int8)
        flags[0] = 1
        f.adapt(flags, 0, 10)
    lo, ln, lv = boxes(f, case)
    conf, hang, _ = brute_force_faces(f, case)
    for a, b, _ in hang:
        assert abs(int(lv[a]) - int(lv[b])) == 1
    mesh = f.flatten()   # flatten refuses unbalanced forests
    assert mesh.n_elem == len(f)


def test_watertight_face_areas():
    """Sum of face areas seen from each element = its closed surface."""
    case = Case(level=2, tree_len=(1.0, 2.0, 0.5))
    mesh = hanging_forest(case, frac=0.3, seed=4)[0].flatten()
    E = mesh.n_elem
    h = np.array(case.tree_len)[:, None] / (2.0 ** mesh.level[None, :])
    area = np.zeros(E)
    for k in range(mesh.n_face):
        info = int(mesh.face_info[k])
        d, kind = info & 3, (info >> 2) & 3
        s, t = [a for a in range(3) if a != d]
        a, b = mesh.face_elem[:, k]
        small = a if kind in (0, 1) else b
        ar = h[s, small] * h[t, small]
        area[a] += ar
        area[b] += ar
    for k in range(mesh.n_bface):
        e, fc = mesh.bface_elem[k], mesh.bface_face[k]
        s, t = [a for a in range(3) if a != fc // 2]
        area[e] += h[s, e] * h[t, e]
    surf = 2 * (h[0] * h[1] + h[1] * h[2] + h[0] * h[2])
    assert np.allclose(area, surf, rtol=1e-14)


def test_adapt_coarsens_complete_families_only():
    case = Case(level=2)
    f = Forest(case)
    flags = -np.ones(len(f), np.int8)
    flags[:3] = 0          # first family keeps three non-coarsening members
    n = f.adapt(flags, 0, 5)
    assert n == 8 + 7      # first family stays, the other 7 merge


def vectorized_face_check(forest, case, mesh):
    """Geometric checks of every face record in O(E) (for meshes where the
    brute-force matcher is too slow): conforming sides are same-size boxes
    touching across the face with equal tangential extent, mortar sub-faces
    a half-size box inside the big side's face at its sub position, boundary
    faces on the domain boundary; the records' areas close every element."""
    lo, ln, lv = boxes(forest, case)
    ext = np.array(case.brick, np.int64) * (1 << 19)
    fe, info = mesh.face_elem.astype(np.int64), mesh.face_info.astype(np.int64)
    a, b, d = fe[0], fe[1], info & 3
    kind, sub, wrap = (info >> 2) & 3, (info >> 4) & 3, (info >> 6) & 1
    k = np.arange(mesh.n_face)
    s_ax = np.where(d == 0, 1, 0)
    t_ax = np.where(d == 2, 1, 2)
    # side 0's upper face coordinate meets side 1's lower face (mod period)
    top_a = (lo[a, d] + ln[a]) % ext[d]
    assert (top_a == lo[b, d]).all()
    assert ((lo[a, d] + ln[a] == ext[d]) == (wrap == 1)).all()
    small = np.where(kind == 2, b, a)
    big = np.where(kind == 2, a, b)
    conf = kind == 0
    assert (ln[a[conf]] == ln[b[conf]]).all()
    assert (lo[a[conf], s_ax[conf]] == lo[b[conf], s_ax[conf]]).all()
    assert (lo[a[conf], t_ax[conf]] == lo[b[conf], t_ax[conf]]).all()
    hang = ~conf
    sm, bg, kk = small[hang], big[hang], k[hang]
    assert (2 * ln[sm] == ln[bg]).all()
    off_s = lo[sm, s_ax[kk]] - lo[bg, s_ax[kk]]
    off_t = lo[sm, t_ax[kk]] - lo[bg, t_ax[kk]]
    assert (off_s == (sub[kk] & 1) * ln[sm]).all() and (off_t == ((sub[kk] >> 1) & 1) * ln[sm]).all()
    # boundary records lie on the domain boundary
    be, bf = mesh.bface_elem.astype(np.int64), mesh.bface_face.astype(np.int64)
    bd, up = bf // 2, bf % 2
    x = np.where(up == 1, lo[be, bd] + ln[be], lo[be, bd])
    assert (np.where(up == 1, x == ext[bd], x == 0)).all()
    # closed surfaces: 6 faces of area ln^2 per element (in units of the small side)
    area = np.zeros(len(ln))
    ar = ln[small].astype(np.float64) ** 2
    np.add.at(area, a, ar)
    np.add.at(area, b, ar)
    np.add.at(area, be, ln[be].astype(np.float64) ** 2)
    assert np.array_equal(area, 6.0 * ln.astype(np.float64) ** 2)


@pytest.mark.parametrize("case", [Case(level=5), Case(level=5, brick=(2, 1, 1), periodic=(1, 0, 1))])
def test_flatten_large_meshes(case):
    """Meshes above the size where flatten and balance run their neighbour
    queries on several threads (16384 leaves), refined with hanging faces."""
    forest = hanging_forest(case, frac=0.05, seed=21)[0]
    assert len(forest) > 16384
    vectorized_face_check(forest, case, forest.flatten())


def test_write_vtu_round_trip(tmp_path):
    """The VTK XML writer: one hexahedron per leaf with the leaf's corners,
    level and field arrays as written."""
    import xml.etree.ElementTree as ET
    case = Case(level=1, tree_len=(1.0, 2.0, 0.5))
    forest = hanging_forest(case, frac=0.3, seed=2)[0]
    mesh = forest.flatten()
    E = mesh.n_elem
    fields = np.stack([np.arange(E, dtype=np.float64) * 0.5, -np.linspace(0.0, 1.0, E)])
    path = str(tmp_path / "out.vtu")
    forest.write_vtu(path, fields, ["R", "C_AIR"])
    piece = ET.parse(path).getroot().find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfCells")) == E and int(piece.get("NumberOfPoints")) == 8 * E
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=np.float64) for a in piece.iter("DataArray")}
    assert np.array_equal(arrays["level"], mesh.level.astype(np.float64))
    assert np.array_equal(arrays["R"], fields[0]) and np.array_equal(arrays["C_AIR"], fields[1])
    assert (arrays["types"] == 12).all()
    pts = piece.find("Points/DataArray")
    xyz = np.array(pts.text.split(), dtype=np.float64).reshape(E, 8, 3)
    h = np.array(case.tree_len)[None, :] / (2.0 ** mesh.level[:, None])
    assert np.allclose(xyz.mean(axis=1), mesh.center.T, rtol=0, atol=1e-15)
    assert np.allclose(xyz.max(axis=1) - xyz.min(axis=1), h, rtol=1e-15)


def _records(mesh):
    return (mesh.center.copy(), mesh.level.copy(), mesh.face_elem.copy(), mesh.face_info.copy(),
            mesh.bface_elem.copy(), mesh.bface_face.copy(), mesh.bface_bnd.copy())


def test_parallel_loops_from_two_threads():
    """The host octree's worker pool serves one loop at a time; a loop that
    finds it busy (another thread's flatten) runs on its own thread.  Both
    give the records a lone flatten gives."""
    import threading
    case = Case(level=5, brick=(2, 1, 1), periodic=(1, 0, 1))
    forests = [hanging_forest(case, frac=0.05, seed=21)[0] for _ in range(2)]
    want = _records(forests[0].flatten())
    got = [None, None]

    def run(k):
        for _ in range(3):
            got[k] = _records(forests[k].flatten())

    th = [threading.Thread(target=run, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=120)
    assert not any(t.is_alive() for t in th)
    for g in got:
        assert all(np.array_equal(a, b) for a, b in zip(g, want))


@pytest.mark.filterwarnings("ignore:This process .* is multi-threaded:DeprecationWarning")
def test_parallel_loops_in_forked_child():
    """A child forked after the worker pool started has none of its threads:
    its first parallel loop starts a pool of its own (no wait on a thread
    that does not exist), and its records match the parent's."""
    import os
    import time
    case = Case(level=5)
    forest = hanging_forest(case, frac=0.05, seed=21)[0]
    want = _records(forest.flatten())           # the pool is running now
    pid = os.fork()
    if pid == 0:                                # child: report by exit code only
        code = 1
        try:
            got = _records(forest.flatten())
            code = 0 if all(np.array_equal(a, b) for a, b in zip(got, want)) else 2
        finally:
            os._exit(code)
    deadline = time.time() + 120
    status = None
    while time.time() < deadline:
        done, status = os.waitpid(pid, os.WNOHANG)
        if done:
            break
        time.sleep(0.05)
    else:
        os.kill(pid, 9)
        os.waitpid(pid, 0)
        pytest.fail("forked child did not finish its flatten")
    assert os.WIFEXITED(status) and os.WEXITSTATUS(status) == 0


@pytest.mark.parametrize("hang", [False, True])
def test_flatten_matches_reference_face_fixture(hang):
    """Face and boundary records of flatten against the reference's own face
    iteration recorded in tests/golden/mesh_faces.npz (conforming,
    hanging 1-to-4 and boundary faces; same element indices)."""
    import os
    from .common import face_sets_of_mesh, face_sets_of_reference, small_case
    from .golden_cases import GOLDEN
    d = np.load(os.path.join(GOLDEN, "mesh_faces.npz"))
    case = small_case("random", "LF", "NONE", level=2)
    forest = hanging_forest(case)[0] if hang else Forest(case)
    want = face_sets_of_reference(d["faces_hanging" if hang else "faces_uniform"])
    assert face_sets_of_mesh(forest.flatten()) == want
    if hang:
        assert len(want[1]) > 0
