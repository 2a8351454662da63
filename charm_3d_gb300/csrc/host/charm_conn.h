/*
 * Unstructured hexahedral connectivity for the host octree: a forest of
 * trees, one per hexahedron of the mesh, as CHARM_3D builds it for p4est
 * from a gmsh file (reference: src/charm_connectivity.c:315-519,
 * charm_conn_reader_msh, followed by p4est_connectivity_complete).
 *
 * Each tree keeps its 8 corner vertices in p4est order (corner k = ix + 2 iy
 * + 4 iz of the tree's reference cube) and, for each of its 6 faces
 * (p4est numbering -x,+x,-y,+y,-z,+z), the tree across it or -1 on the
 * domain boundary.  Instead of p4est's face orientation codes each tree
 * face carries the integer map of tree coordinates onto the neighbour's:
 * coordinate i of the neighbour tree = sign[i] * (coordinate perm[i] of this
 * tree) + off[i], in the octree's integer quadrant coordinates (a tree edge
 * is CHARM_FOREST_ROOT_LEN), so the map is exact; it is derived from the
 * corner vertices the two trees share.
 */
#ifndef CHARM_CONN_H
#define CHARM_CONN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHARM_CONN_NAME 64

typedef struct charm_conn_patch {
    int32_t dim, tag;
    char name[CHARM_CONN_NAME];
} charm_conn_patch_t;

typedef struct charm_conn {
    int32_t n_tree, n_vert;
    double  *vert;       /* [n_vert][3] */
    int32_t *t2v;        /* [n_tree][8] corner vertices, p4est corner order */
    int32_t *t2t;        /* [n_tree][6] tree across each face, -1 on the boundary */
    int8_t  *t2f;        /* [n_tree][6] the neighbour tree's face */
    int8_t  *xperm;      /* [n_tree][6][3] map onto the neighbour tree (see above) */
    int8_t  *xsign;      /* [n_tree][6][3] */
    int32_t *xoff;       /* [n_tree][6][3] in integer quadrant coordinates */
    int32_t *bnd_tag;    /* [n_tree][6] physical tag of the boundary patch of a face, -1: none */
    int32_t *reg_tag;    /* [n_tree] physical tag of the hexahedron (-1: none) */
    int32_t n_patch;
    charm_conn_patch_t *patch;
} charm_conn_t;

/* corners of each face, lower tangential axis first (p4est's
 * p8est_face_corners, the reference's charm_face_corners) */
extern const int charm_conn_face_corners[6][4];

/* Build from vertex and tree arrays (t2v in p4est corner order) and match
 * the tree faces by their vertex sets.  Returns 0, or -1 with a message in
 * err (a face shared by more than two trees, a face whose corner
 * correspondence is not a symmetry of the square, a repeated vertex). */
int charm_conn_build(charm_conn_t *c, int32_t n_vert, const double *vert, int32_t n_tree, const int32_t *t2v,
                     char *err, int errlen);

/* Read a gmsh 2.x ASCII mesh: $PhysicalNames, $Nodes, and from $Elements
 * the 8-node hexahedra (type 5) as trees and the 4-node quadrangles (type
 * 3) as boundary faces with their physical tag.  Returns 0 or -1 with a
 * message in err. */
int charm_conn_read_gmsh(charm_conn_t *c, const char *path, char *err, int errlen);

void charm_conn_free(charm_conn_t *c);

/* Name of the patch with physical tag `tag` and dimension dim (2 faces, 3
 * volumes), or NULL. */
const char *charm_conn_patch_name(const charm_conn_t *c, int dim, int32_t tag);

/* Point of tree t at reference coordinates (x,y,z) in [0,1]^3: the
 * trilinear map of its corner vertices (p4est_qcoord_to_vertex). */
void charm_conn_point(const charm_conn_t *c, int32_t t, double x, double y, double z, double out[3]);

/* Map the box [p, p + len)^3 of tree t, lying across face f outside the
 * tree, into the neighbour tree: lower corner q (integer coordinates).
 * Returns the neighbour tree or -1 on the boundary. */
int32_t charm_conn_map_box(const charm_conn_t *c, int32_t t, int f, const int32_t p[3], int32_t len, int32_t q[3]);

#ifdef __cplusplus
}
#endif

#endif
