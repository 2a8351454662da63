"""Synthetic unstructured hexahedral meshes (the workloads of the tests and
the bench on general hexahedra).

Meshes are built here from structured blocks: vertices on a grid, mapped
through an optional non-affine distortion (so that the hexahedra are
trilinear, not boxes), with each tree's corner numbering optionally turned
by one of the 24 rotations of the cube, so that neighbouring trees meet in
every face orientation.  `write_gmsh` writes a gmsh 2.2 ASCII file of a mesh
with its boundary quadrangles and physical names, the format the library's
reader takes.
"""
from __future__ import annotations

import itertools

import numpy as np

# gmsh hexahedron node order from the p4est corner order (and back)
P4EST_TO_GMSH = [0, 1, 3, 2, 4, 5, 7, 6]
FACE_CORNERS = [[0, 2, 4, 6], [1, 3, 5, 7], [0, 1, 4, 5], [2, 3, 6, 7], [0, 1, 2, 3], [4, 5, 6, 7]]


def _rotations():
    """The 24 proper rotations of the cube as (perm, sign) of the axes."""
    out = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            m = np.zeros((3, 3), int)
            for i in range(3):
                m[i, perm[i]] = signs[i]
            if round(np.linalg.det(m)) == 1:
                out.append(m)
    return out


ROTATIONS = _rotations()


def rotate_tree(corners: np.ndarray, rot: np.ndarray) -> np.ndarray:
    """Relabel the 8 corner vertex ids of one tree by a rotation of its
    reference cube (keeps the orientation, so the Jacobian stays positive)."""
    out = np.empty(8, corners.dtype)
    for k in range(8):
        p = np.array([(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1]) * 2 - 1
        q = rot @ p
        k2 = int((q[0] + 1) // 2) + 2 * int((q[1] + 1) // 2) + 4 * int((q[2] + 1) // 2)
        out[k2] = corners[k]
    return out


class HexMesh:
    """Vertices [n][3], trees [T][8] (p4est corner order), and for every
    boundary tree face (t, f) a patch name."""

    def __init__(self, vert, trees, bnd):
        self.vert = np.asarray(vert, np.float64)
        self.trees = np.asarray(trees, np.int32)
        self.bnd = dict(bnd)   # (tree, face) -> patch name

    def tree_bnd(self, names: list[str]) -> np.ndarray:
        """[T][6] boundary index per tree face (-1 where there is a neighbour)."""
        tb = -np.ones((len(self.trees), 6), np.int8)
        for (t, f), name in self.bnd.items():
            tb[t, f] = names.index(name)
        return tb


def block_mesh(nx, ny, nz, x0=(0.0, 0.0, 0.0), size=(1.0, 1.0, 1.0), distort=0.0, rotate=False, seed=0,
               shape=None) -> HexMesh:
    """nx*ny*nz hexahedra on a grid over the box x0 + [0, size], optionally
    mapped by `shape(x, y, z) -> (x, y, z)` (grid coordinates in [0,1]^3)
    and by a smooth non-affine distortion of relative amplitude `distort`;
    boundary patches XMIN, XMAX, YMIN, YMAX, ZMIN, ZMAX."""
    rng = np.random.default_rng(seed)
    gi = np.arange(nx + 1)[:, None, None] / nx
    gj = np.arange(ny + 1)[None, :, None] / ny
    gk = np.arange(nz + 1)[None, None, :] / nz
    X, Y, Z = np.broadcast_arrays(gi, gj, gk)
    X, Y, Z = X.astype(float), Y.astype(float), Z.astype(float)
    if distort:
        # interior displacement vanishing on the box faces (faces stay planar there)
        bump = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
        X = X + distort * bump * np.sin(2.0 * np.pi * Y + 0.3)
        Y = Y + distort * bump * np.cos(2.0 * np.pi * Z + 0.7)
        Z = Z + distort * bump * np.sin(2.0 * np.pi * X + 1.1)
    if shape is not None:
        X, Y, Z = shape(X, Y, Z)
    else:
        X, Y, Z = x0[0] + size[0] * X, x0[1] + size[1] * Y, x0[2] + size[2] * Z
    vid = np.arange((nx + 1) * (ny + 1) * (nz + 1)).reshape(nx + 1, ny + 1, nz + 1)
    vert = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    trees, bnd = [], {}
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                c = np.array([vid[i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1)] for q in range(8)])
                t = len(trees)
                faces = {0: i == 0, 1: i == nx - 1, 2: j == 0, 3: j == ny - 1, 4: k == 0, 5: k == nz - 1}
                names = {0: "XMIN", 1: "XMAX", 2: "YMIN", 3: "YMAX", 4: "ZMIN", 5: "ZMAX"}
                if rotate:
                    rot = ROTATIONS[int(rng.integers(len(ROTATIONS)))]
                    c2 = rotate_tree(c, rot)
                    # the boundary faces move with the corners: find each by its vertex set
                    for f, on in faces.items():
                        if on:
                            vs = set(c[FACE_CORNERS[f]])
                            g = [g for g in range(6) if set(c2[FACE_CORNERS[g]]) == vs][0]
                            bnd[(t, g)] = names[f]
                    c = c2
                else:
                    for f, on in faces.items():
                        if on:
                            bnd[(t, f)] = names[f]
                trees.append(c)
    return HexMesh(vert, np.array(trees), bnd)


def wedge_mesh(n=4, rotate=False, seed=0, depth=100.0, layers=1) -> HexMesh:
    """A channel with a ramp, in three blocks of n x n, n x n and 6n x n
    hexahedra and `layers` cells deep: [-1000, 0] x [0, 1000], a ramp block
    over [0, 1000] whose floor rises from y = 0 to y = 176.33 (trapezoidal
    cells: trilinear, not affine), and [1000, 6000] x [176.33, 1000]; the
    layout of the reference's sample case samples/klin_amr (n = 10: 800
    hexahedra, one layer 100 deep).  Patches: LEFT (x = -1000), RIGHT
    (x = 6000), BOTTOM (floor and ramp), TOP (y = 1000), FRONT (z = 0),
    BACK (z = depth)."""
    rng = np.random.default_rng(seed)
    ramp = 176.33
    blocks = [(-1000.0, 0.0, lambda s: 0.0 * s, n), (0.0, 1000.0, lambda s: ramp * s, n),
              (1000.0, 6000.0, lambda s: ramp + 0.0 * s, 6 * n)]
    verts, index = [], {}

    def vid(x, y, z):
        key = (round(x, 9), round(y, 9), round(z, 9))
        if key not in index:
            index[key] = len(verts)
            verts.append((x, y, z))
        return index[key]

    trees, bnd = [], {}
    for bi, (xa, xb, floor, nxb) in enumerate(blocks):
        for k in range(layers):
            for j in range(n):
                for i in range(nxb):
                    c = []
                    for q in range(8):
                        s = (i + (q & 1)) / nxb
                        x = xa + (xb - xa) * s
                        y0 = floor(s)
                        y = y0 + (1000.0 - y0) * (j + ((q >> 1) & 1)) / n
                        z = depth * (k + ((q >> 2) & 1)) / layers
                        c.append(vid(x, y, z))
                    c = np.array(c)
                    t = len(trees)
                    faces = {0: bi == 0 and i == 0, 1: bi == 2 and i == nxb - 1, 2: j == 0, 3: j == n - 1,
                             4: k == 0, 5: k == layers - 1}
                    names = {0: "LEFT", 1: "RIGHT", 2: "BOTTOM", 3: "TOP", 4: "BACK", 5: "FRONT"}
                    if rotate:
                        c2 = rotate_tree(c, ROTATIONS[int(rng.integers(len(ROTATIONS)))])
                        for f, on in faces.items():
                            if on:
                                vs = set(c[FACE_CORNERS[f]])
                                g = [g for g in range(6) if set(c2[FACE_CORNERS[g]]) == vs][0]
                                bnd[(t, g)] = names[f]
                        c = c2
                    else:
                        for f, on in faces.items():
                            if on:
                                bnd[(t, f)] = names[f]
                    trees.append(c)
    return HexMesh(np.array(verts), np.array(trees), bnd)


def write_gmsh(mesh: HexMesh, path: str, region: str = "DOMAIN", patches: list[str] | None = None) -> None:
    """gmsh 2.2 ASCII: physical names (patches dim 2, the region dim 3),
    nodes, boundary quadrangles (type 3) and hexahedra (type 5)."""
    names = patches or sorted(set(mesh.bnd.values()))
    tag = {nm: i + 1 for i, nm in enumerate(names)}
    rtag = len(names) + 1
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(names) + 1)]
    lines += [f'2 {tag[nm]} "{nm}"' for nm in names]
    lines += [f'3 {rtag} "{region}"', "$EndPhysicalNames", "$Nodes", str(len(mesh.vert))]
    lines += [f"{i + 1} {float(x):.17g} {float(y):.17g} {float(z):.17g}" for i, (x, y, z) in enumerate(mesh.vert)]
    lines += ["$EndNodes", "$Elements"]
    els = []
    for (t, f), nm in sorted(mesh.bnd.items()):
        c = mesh.trees[t][FACE_CORNERS[f]]
        # a quadrangle's nodes go round its boundary: corners 0, 1, 3, 2 of the face
        els.append(f"3 2 {tag[nm]} {tag[nm]} {c[0] + 1} {c[1] + 1} {c[3] + 1} {c[2] + 1}")
    for t in mesh.trees:
        g = [t[P4EST_TO_GMSH[k]] + 1 for k in range(8)]
        els.append(f"5 2 {rtag} {rtag} " + " ".join(str(v) for v in g))
    lines += [str(len(els))] + [f"{i + 1} {e}" for i, e in enumerate(els)] + ["$EndElements", ""]
    with open(path, "w") as fp:
        fp.write("\n".join(lines))



WEDGE_PATCHES = ["LEFT", "RIGHT", "BOTTOM", "TOP", "FRONT", "BACK"]



def ramp_channel(level: int = 0, n: int = 10, rotate: bool = False, seed: int = 9):
    """The reference's sample case samples/klin_amr on its mesh geometry
    (wedge_mesh(10) has the sample's 800 hexahedra): Euler, HLLC,
    Barth-Jespersen, air at 300 K and 101325 Pa entering at 697.7082 m/s
    through LEFT, outlet RIGHT, slip walls elsewhere (its task.yaml's
    values), the trees refined uniformly to `level`, seeded +-1 % density
    noise, and TAU from CFL 0.1 on the smallest cell edge.  Returns (case,
    forest, mesh, u0)."""
    from .case import Boundary, synthetic
    from .solver import Forest
    case = synthetic("sod", level=level)
    case.name = "ramp"
    case.model, case.flux, case.limiter = "EULER", "HLLC", "BJ"
    T, P, V = 300.0, 101325.0, 697.7082
    case.boundaries = [Boundary("LEFT", "BOUND_INLET", (V, 0.0, 0.0, T, P)), Boundary("RIGHT", "BOUND_OUTLET"),
                       Boundary("BOTTOM", "BOUND_WALL_SLIP"), Boundary("TOP", "BOUND_WALL_SLIP"),
                       Boundary("FRONT", "BOUND_WALL_SLIP"), Boundary("BACK", "BOUND_WALL_SLIP")]
    m = wedge_mesh(n, rotate=rotate, seed=seed)
    forest = Forest.from_hex(m.vert, m.trees, m.tree_bnd(WEDGE_PATCHES), level)
    mesh = forest.flatten()
    rho = P * case.components[0].m / (8.31446261815324 * T)
    E = mesh.n_elem
    rng = np.random.default_rng(4)
    r = rho * (1.0 + 0.01 * rng.uniform(-1, 1, E))
    one = np.ones(E)
    u0 = np.zeros((case.n_var, 4, E))
    u0[:, 0, :] = case.cons_from_prim(r, V * one, 0 * one, 0 * one, P * one)
    # the smallest edge: the depth of the one layer, or a cell of the ramp block
    h = min(100.0, (1000.0 - 176.33) / n) / 2 ** level
    case.tau = 0.1 * h / (V + np.sqrt(1.4 * P / rho))
    return case, forest, mesh, u0
