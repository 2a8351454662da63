"""Unstructured hexahedral meshes on the host (no GPU): the gmsh reader, the
connectivity of trees in every face orientation, flattening with mortars
across tree faces, and the oracle's general-hexahedron geometry.

Reference: src/charm_connectivity.c:315-519 (charm_conn_reader_msh),
src/charm_geom.c (trilinear geometry), p4est_connectivity_complete and
p4est_iterate (face sides across trees).
"""
import os

import numpy as np
import pytest

from charm_3d_gb300 import Boundary, synthetic
from charm_3d_gb300.abi import EINVAL, CharmGpuError
from charm_3d_gb300.solver import Forest
from oracle.port import Port

from .common import rel_max, small_case
from .hexmesh import (FACE_CORNERS, SIDE_PATCHES, WEDGE_PATCHES, block_forest, block_mesh, keystone, wedge_mesh,
                      write_gmsh)

from oracle.build_ref import reference_root  # noqa: E402

REF = reference_root() or ""


def face_center(mesh, e, f):
    return mesh.vertex[FACE_CORNERS[f], :, e].mean(axis=0)


def face_area(mesh, e, f):
    v = mesh.vertex[FACE_CORNERS[f], :, e]
    return 0.5 * (np.linalg.norm(np.cross(v[1] - v[0], v[2] - v[0])) + np.linalg.norm(np.cross(v[1] - v[3], v[2] - v[3])))


def test_gmsh_reader_matches_the_arrays_it_was_written_from(tmp_path):
    m = block_mesh(3, 2, 2, rotate=True, seed=5, shape=keystone)
    path = str(tmp_path / "block.msh")
    write_gmsh(m, path)
    a = Forest.from_hex(m.vert, m.trees, m.tree_bnd(SIDE_PATCHES), 1).flatten()
    b = Forest.from_gmsh(path, 1, SIDE_PATCHES).flatten()
    assert a.n_elem == b.n_elem == 12 * 8
    assert np.array_equal(a.vertex, b.vertex)
    assert np.array_equal(a.face_elem, b.face_elem) and np.array_equal(a.face_face, b.face_face)
    assert np.array_equal(a.bface_elem, b.bface_elem) and np.array_equal(a.bface_bnd, b.bface_bnd)
    f = Forest.from_gmsh(path, 0, SIDE_PATCHES)
    assert (f.tree_regions() == len(SIDE_PATCHES) + 1).all()   # the volume's physical tag


def test_gmsh_reader_errors(tmp_path):
    m = block_mesh(2, 1, 1)
    path = str(tmp_path / "m.msh")
    write_gmsh(m, path)
    with pytest.raises(CharmGpuError) as ei:   # a patch the case does not configure
        Forest.from_gmsh(path, 0, SIDE_PATCHES[:-1])
    assert ei.value.code == EINVAL and "ZMAX" in str(ei.value)
    text = open(path).read().splitlines()
    # drop one boundary quadrangle: that face has no boundary
    i = next(k for k, ln in enumerate(text) if ln.split()[1:2] == ["3"] and len(ln.split()) == 9)
    cnt = text.index("$Elements") + 1
    text[cnt] = str(int(text[cnt]) - 1)
    del text[i]
    open(path, "w").write("\n".join(text))
    with pytest.raises(CharmGpuError) as ei:
        Forest.from_gmsh(path, 0, SIDE_PATCHES)
    assert "without a physical quadrangle" in str(ei.value)
    with pytest.raises(CharmGpuError):
        Forest.from_gmsh(str(tmp_path / "missing.msh"), 0, SIDE_PATCHES)


def test_face_shared_by_three_trees_is_rejected():
    m = block_mesh(2, 1, 1)
    trees = np.vstack([m.trees, m.trees[1:2]])   # a copy of tree 1 on the same vertices
    with pytest.raises(CharmGpuError):
        Forest.from_hex(m.vert, trees, -np.ones((3, 6), np.int8), 0)


@pytest.mark.parametrize("level", [0, 1, 2])
@pytest.mark.parametrize("kind", ["keystone", "distorted", "wedge"])
def test_faces_join_the_same_surface_from_both_sides(kind, level):
    """Every interior record joins two element faces with the same corners
    (trees meet in all 24 orientations), and the records match a brute-force
    search by face centres; boundary faces are the rest."""
    if kind == "wedge":
        m = wedge_mesh(2, rotate=True, seed=2)
        f = Forest.from_hex(m.vert, m.trees, m.tree_bnd(WEDGE_PATCHES), level)
    else:
        m = block_mesh(3, 2, 2, rotate=True, seed=4, shape=keystone if kind == "keystone" else None,
                       distort=0.15 if kind == "distorted" else 0.0)
        f = Forest.from_hex(m.vert, m.trees, m.tree_bnd(SIDE_PATCHES), level)
    mesh = f.flatten()
    E, F = mesh.n_elem, mesh.n_face
    assert E == len(m.trees) * 8 ** level
    for i in range(F):
        a, b = mesh.face_elem[:, i]
        fa, fb = mesh.face_face[:, i]
        va = {tuple(np.round(x, 9)) for x in mesh.vertex[FACE_CORNERS[fa], :, a]}
        vb = {tuple(np.round(x, 9)) for x in mesh.vertex[FACE_CORNERS[fb], :, b]}
        assert va == vb, i
    # brute force: element faces whose centres coincide
    from scipy.spatial import cKDTree
    keys = [(e, g) for e in range(E) for g in range(6)]
    pts = np.array([face_center(mesh, e, g) for e, g in keys])
    tol = 1e-9 * np.abs(pts).max()
    close = cKDTree(pts).query_pairs(tol)
    seen = [0] * len(keys)
    for a, b in close:
        seen[a] += 1
        seen[b] += 1
    assert max(seen) <= 1
    pairs = {tuple(sorted([keys[a], keys[b]])) for a, b in close}
    singles = {keys[k] for k in range(len(keys)) if seen[k] == 0}
    got = {tuple(sorted([(mesh.face_elem[0, i], mesh.face_face[0, i]), (mesh.face_elem[1, i], mesh.face_face[1, i])]))
           for i in range(F)}
    assert got == pairs
    assert {(e, g) for e, g in zip(mesh.bface_elem, mesh.bface_face)} == singles


def test_mortars_across_rotated_trees():
    """Refining leaves next to tree faces of every orientation: the 2:1
    balance reaches across the trees, and the 4 small faces of each mortar
    tile the big face."""
    m = block_mesh(3, 2, 2, rotate=True, seed=6, shape=keystone)
    f = Forest.from_hex(m.vert, m.trees, m.tree_bnd(SIDE_PATCHES), 1)
    rng = np.random.default_rng(1)
    f.adapt((rng.uniform(size=len(f)) < 0.25).astype(np.int8), 0, 3)
    f.adapt((rng.uniform(size=len(f)) < 0.15).astype(np.int8), 0, 3)
    mesh = f.flatten()
    kind = (mesh.face_info >> 2) & 3
    assert (kind > 0).sum() > 0 and (kind > 0).sum() % 4 == 0
    lev = mesh.level
    for i in range(mesh.n_face):
        a, b = mesh.face_elem[:, i]
        assert abs(int(lev[a]) - int(lev[b])) <= 1
        if kind[i] == 0:
            continue
        small, big = (a, b) if kind[i] == 1 else (b, a)
        fs = mesh.face_face[0 if kind[i] == 1 else 1, i]
        fb = mesh.face_face[1 if kind[i] == 1 else 0, i]
        assert lev[small] == lev[big] + 1
        if ((mesh.face_info[i] >> 4) & 3) == 0:
            subs = [mesh.face_elem[0 if kind[i + k] == 1 else 1, i + k] for k in range(4)]
            sfs = [mesh.face_face[0 if kind[i + k] == 1 else 1, i + k] for k in range(4)]
            area = sum(face_area(mesh, s, g) for s, g in zip(subs, sfs))
            assert abs(area - face_area(mesh, big, fb)) < 1e-12 * face_area(mesh, big, fb)
        # the small face's centre lies in the big face's plane
        v = mesh.vertex[FACE_CORNERS[fb], :, big]
        n = np.cross(v[1] - v[0], v[2] - v[0])
        assert abs(np.dot(face_center(mesh, small, fs) - v[0], n)) < 1e-12 * np.linalg.norm(n)


def _uniform_state(case, E):
    u = np.zeros((case.n_var, 4, E))
    one = np.ones(E)
    u[:, 0, :] = case.cons_from_prim(one, 0.3 * one, -0.2 * one, 0.1 * one, one)
    return u


@pytest.mark.parametrize("kind", ["keystone", "wedge"])
def test_oracle_preserves_free_stream_on_non_affine_cells(kind):
    """A uniform state with transmissive boundaries has a zero residual when
    the faces are planar: the triangle rule integrates linear functions on
    them exactly and the trilinear Jacobian is integrated exactly."""
    case = synthetic("sod", level=1)
    if kind == "wedge":
        m = wedge_mesh(3, rotate=True, seed=1)
        case.boundaries = [Boundary(n, "BOUND_OUTLET") for n in WEDGE_PATCHES]
        f = Forest.from_hex(m.vert, m.trees, m.tree_bnd(WEDGE_PATCHES), 1)
    else:
        case.boundaries = [Boundary(n, "BOUND_OUTLET") for n in SIDE_PATCHES]
        f, m = block_forest(case, level=1)
    mesh = f.flatten()
    port = Port(case.config(), mesh)
    u = _uniform_state(case, mesh.n_elem)
    port.set_state(u)
    r = port.residual()
    # scale: flux times face area
    scale = np.abs(u).max() * max(face_area(mesh, e, g) for e in range(mesh.n_elem) for g in range(6))
    assert np.abs(r).max() < 1e-13 * scale


def test_oracle_on_hexahedra_equals_the_box_oracle_on_a_brick():
    """Two unit trees in the identity orientation: the general-hexahedron
    geometry reproduces the box geometry, residual and steps (limiter on)."""
    case = synthetic("sod", level=2)
    case.init, case.seed, case.brick, case.tree_len = "random", 7, (2, 1, 1), (0.5, 1.0, 1.0)
    case.boundaries = [Boundary("ALL", "BOUND_OUTLET")]
    box = Forest(case).flatten()
    m = block_mesh(2, 1, 1)
    hexm = Forest.from_hex(m.vert, m.trees, np.zeros((2, 6), np.int8), 2).flatten()
    order = np.array([np.argmin(((hexm.center.T - c) ** 2).sum(1)) for c in box.center.T])
    assert np.abs(hexm.center[:, order] - box.center).max() < 1e-15
    u0 = case.initial_state(box.center)
    pb, ph = Port(case.config(), box), Port(case.config(), hexm)
    pb.set_state(u0)
    uh = np.empty_like(u0)
    uh[:, :, order] = u0
    ph.set_state(uh)
    assert rel_max(ph.residual()[:, :, order], pb.residual()) < 1e-14
    pb.run(3, case.tau)
    ph.run(3, case.tau)
    assert rel_max(ph.get_state()[:, :, order], pb.get_state()) < 1e-14


def test_oracle_rejects_inverted_hexahedra():
    case = synthetic("sod", level=0)
    case.boundaries = [Boundary(n, "BOUND_OUTLET") for n in SIDE_PATCHES]
    m = block_mesh(2, 1, 1)
    f = Forest.from_hex(m.vert, m.trees, m.tree_bnd(SIDE_PATCHES), 0)
    mesh = f.flatten()
    mesh.vertex = mesh.vertex[[4, 5, 6, 7, 0, 1, 2, 3]]   # mirrored corners: negative Jacobian
    with pytest.raises(MemoryError):
        Port(case.config(), mesh)


@pytest.mark.reference
@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "samples/klin_amr/klin.msh")), reason="no reference checkout")
def test_reference_sample_mesh_reads_with_its_case_file():
    """samples/klin_amr: the 800 hexahedra and the boundary names of its
    task.yaml; every element has a positive Jacobian."""
    from charm_3d_gb300.abi import read_case_yaml
    cf = read_case_yaml(os.path.join(REF, "samples/klin_amr/task.yaml"))
    names = [cf.bnd_name[k].value.decode() for k in range(cf.cfg.n_bnd)]
    f = Forest.from_gmsh(os.path.join(REF, "samples/klin_amr/klin.msh"), 0, names)
    mesh = f.flatten()
    assert mesh.n_elem == 800
    assert set(mesh.bface_bnd.tolist()) == set(range(len(names)))
    port = Port(cf.cfg, mesh)   # raises for a non-positive Jacobian
    assert port.h


@pytest.mark.reference
@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "samples/klin_amr/klin.msh")), reason="no reference checkout")
def test_generated_ramp_channel_is_the_reference_sample_mesh():
    """tests/hexmesh.wedge_mesh(10) has the sample mesh's 800 hexahedra
    (the same corner sets) and the same boundary patch on every boundary
    face, so the GPU tests that run on the generated mesh (the sample is
    not available where they run) run on the sample's geometry."""
    import collections
    names = WEDGE_PATCHES
    sample = Forest.from_gmsh(os.path.join(REF, "samples/klin_amr/klin.msh"), 0, names).flatten()
    m = wedge_mesh(10)
    ours = Forest.from_hex(m.vert, m.trees, m.tree_bnd(names), 0).flatten()

    def corner_sets(mesh):
        return sorted(tuple(sorted(map(tuple, np.round(mesh.vertex[:, :, e], 6).tolist()))) for e in range(mesh.n_elem))

    def patches(mesh):
        return collections.Counter((tuple(np.round(face_center(mesh, e, f), 6)), names[b])
                                   for e, f, b in zip(mesh.bface_elem, mesh.bface_face, mesh.bface_bnd))

    assert sample.n_elem == ours.n_elem == 800
    assert corner_sets(sample) == corner_sets(ours)
    assert patches(sample) == patches(ours)


def _leaf_key(q, lv):
    return (int(q[3]), int(q[0]), int(q[1]), int(q[2]), int(lv))


@pytest.mark.parametrize("mode", ["refine", "coarsen"])
def test_host_adapt_projects_like_the_reference_on_hexahedra(mode):
    """charm_host_forest_adapt_state on an unstructured forest: every new
    leaf's coefficients are the oracle's restatement of charm_replace_quads
    (src/charm_amr.c:206-307, quadrature on the trilinear cells) applied to
    its family, and the refine/coarsen decisions follow the reference's
    criteria with each leaf's own volume."""
    from oracle.port import hex_project
    case = small_case("random", "HLLC", "BJ")
    forest, _ = block_forest(case, level=1, seed=8)
    old = forest.flatten()
    qo, lvo = forest.leaves()
    E = old.n_elem
    u0 = case.initial_state(old.center)
    if mode == "refine":   # a large gradient in tree 0 only: its leaves refine
        grad = np.zeros((3, E))
        grad[0, qo[:, 3] == 0] = 1.0e3
        u1 = forest.adapt_state(grad, 0.01, 0, 2, case.n_comp, u0)
    else:                  # no gradient, equal densities: every family coarsens
        u0[4:, 0, :] = 1.0
        grad = np.zeros((3, E))
        u1 = forest.adapt_state(grad, 10.0, 0, 2, case.n_comp, u0)
    new = forest.flatten()
    qn, lvn = forest.leaves()
    old_at = {_leaf_key(q, l): i for i, (q, l) in enumerate(zip(qo, lvo))}
    cfg = case.config()
    checked = 0
    for k, (q, l) in enumerate(zip(qn, lvn)):
        if _leaf_key(q, l) in old_at:
            assert np.array_equal(u1[:, :, k], u0[:, :, old_at[_leaf_key(q, l)]])
            continue
        if mode == "refine":
            h = 1 << (19 - int(l))
            parent = (int(q[3]), int(q[0]) & ~h, int(q[1]) & ~h, int(q[2]) & ~h, int(l) - 1)
            p = old_at[parent]
            cid = (1 if q[0] & h else 0) | (2 if q[1] & h else 0) | (4 if q[2] & h else 0)
            # the parent's children, in Morton order, are the new leaves k - cid .. k - cid + 7
            kids = np.arange(k - cid, k - cid + 8)
            want = hex_project(cfg, old.vertex[:, :, p], new.vertex[:, :, kids].transpose(2, 0, 1), True,
                               u0[:, :, p])[cid]
        else:
            h = 1 << (19 - int(l) - 1)
            kids = [old_at[(int(q[3]), int(q[0]) + (c & 1) * h, int(q[1]) + ((c >> 1) & 1) * h,
                            int(q[2]) + ((c >> 2) & 1) * h, int(l) + 1)] for c in range(8)]
            want = hex_project(cfg, new.vertex[:, :, k], old.vertex[:, :, kids].transpose(2, 0, 1), False,
                               u0[:, :, kids].transpose(2, 0, 1))
        assert rel_max(u1[:, :, k], want) < 1e-13, k
        checked += 1
    assert checked > 0
    assert new.n_elem == (E + 7 * 8 if mode == "refine" else E // 8)
