"""Test helpers on top of the package's synthetic hexahedral meshes."""
from __future__ import annotations

import numpy as np

from charm_3d_gb300.hexmesh import (FACE_CORNERS, P4EST_TO_GMSH, ROTATIONS, WEDGE_PATCHES, HexMesh,  # noqa: F401
                                    block_mesh, rotate_tree, wedge_mesh, write_gmsh)


SIDE_PATCHES = ["XMIN", "XMAX", "YMIN", "YMAX", "ZMIN", "ZMAX"]


def keystone(X, Y, Z):
    """A map of the unit cube whose images of grid planes stay planar but
    whose cells are not parallelepipeds (trapezoids in x-y, sheared in z)."""
    return X, Y * (1.0 + 0.5 * X) + 0.2 * Z, Z


def block_forest(case, n=(3, 2, 2), level=1, rotate=True, seed=3, shape=keystone, distort=0.0):
    """Forest over a block mesh whose side patches take the case's
    boundaries by case.bnd_of_side (-x, +x, -y, +y, -z, +z)."""
    from charm_3d_gb300.solver import Forest
    m = block_mesh(*n, rotate=rotate, seed=seed, shape=shape, distort=distort)
    tb = m.tree_bnd(SIDE_PATCHES)
    tb = np.where(tb >= 0, np.array(case.bnd_of_side, np.int8)[np.maximum(tb, 0)], -1).astype(np.int8)
    return Forest.from_hex(m.vert, m.trees, tb, level), m
