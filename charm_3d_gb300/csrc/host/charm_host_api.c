/*
 * Host side of the boundary: the octree forest exposed through the C ABI of
 * include/charm_gpu.h, and its flattening into the structure-of-arrays mesh
 * that the GPU solver consumes.
 *
 * Flattening follows p4est_iterate's face semantics as CHARM_3D relies on
 * them (reference src/models/ns/charm_model_ns_conv.c:174-356):
 *   - a tree-boundary face with one side is a boundary face (one record);
 *   - a full face has two sides, side 0 at the lower coordinate (face
 *     2*dir+1 of that leaf), side 1 at the upper (face 2*dir);
 *   - a hanging face (2:1) has one full side and one side of 4 small
 *     leaves; it becomes 4 sub-face records ("mortars"), in the small
 *     leaves' z-order on the face (s = lower tangential axis first).
 * Periodic wraps (not supported by the reference's mesh reader,
 * src/charm_connectivity.c:457-466) are full faces with the wrap bit set.
 */
#include "charm_gpu.h"
#include "charm_forest.h"

#include <stdlib.h>
#include <string.h>

struct charm_host_forest_s {
    charm_forest_t f;
    int8_t bnd_of_side[6];
    /* flattened arrays (owned) */
    double  *center;
    int8_t  *level;
    int32_t *face_elem;
    uint8_t *face_info;
    int32_t *bface_elem;
    int8_t  *bface_face;
    int8_t  *bface_bnd;
    int64_t  n_face, n_bface;
};

static void free_flat(struct charm_host_forest_s *h)
{
    free(h->center); free(h->level); free(h->face_elem); free(h->face_info);
    free(h->bface_elem); free(h->bface_face); free(h->bface_bnd);
    h->center = NULL; h->level = NULL; h->face_elem = NULL; h->face_info = NULL;
    h->bface_elem = NULL; h->bface_face = NULL; h->bface_bnd = NULL;
    h->n_face = h->n_bface = 0;
}

int charm_host_forest_new(charm_host_forest_t *out, const int32_t ntree[3], const int32_t periodic[3],
                          const double origin[3], const double tree_len[3], int level)
{
    if (!out || !ntree) return CHARM_GPU_EINVAL;
    struct charm_host_forest_s *h = (struct charm_host_forest_s *) calloc(1, sizeof(*h));
    if (!h) return CHARM_GPU_ENOMEM;
    if (charm_forest_init_uniform(&h->f, ntree, periodic, origin, tree_len, level)) {
        free(h);
        return CHARM_GPU_EINVAL;
    }
    for (int k = 0; k < 6; k++) h->bnd_of_side[k] = 0;
    *out = h;
    return CHARM_GPU_OK;
}

int charm_host_forest_free(charm_host_forest_t h)
{
    if (!h) return CHARM_GPU_EINVAL;
    free_flat(h);
    charm_forest_free(&h->f);
    free(h);
    return CHARM_GPU_OK;
}

int64_t charm_host_forest_count(charm_host_forest_t h) { return h ? h->f.n : -1; }

int charm_host_forest_set_bnd(charm_host_forest_t h, const int8_t bnd_of_side[6])
{
    if (!h || !bnd_of_side) return CHARM_GPU_EINVAL;
    memcpy(h->bnd_of_side, bnd_of_side, 6);
    return CHARM_GPU_OK;
}

int charm_host_forest_leaves(charm_host_forest_t h, int32_t *qcoord, int8_t *level)
{
    if (!h) return CHARM_GPU_EINVAL;
    for (int64_t i = 0; i < h->f.n; i++) {
        const charm_leaf_t *q = &h->f.leaf[i];
        if (qcoord) {
            qcoord[4 * i + 0] = q->x; qcoord[4 * i + 1] = q->y;
            qcoord[4 * i + 2] = q->z; qcoord[4 * i + 3] = q->tree;
        }
        if (level) level[i] = q->level;
    }
    return CHARM_GPU_OK;
}

/* ---- adapt ---------------------------------------------------------------- */

typedef struct { const int8_t *flags; } coarsen_ctx_t;

static int coarsen_all_minus(void *user, const charm_leaf_t *leaves, const int64_t idx[8])
{
    (void) leaves;
    const coarsen_ctx_t *c = (const coarsen_ctx_t *) user;
    for (int k = 0; k < 8; k++)
        if (c->flags[idx[k]] >= 0) return 0;
    return 1;
}

int charm_host_forest_adapt(charm_host_forest_t h, const int8_t *flags, int minlevel, int maxlevel, int64_t *n_new)
{
    if (!h || !flags) return CHARM_GPU_EINVAL;
    int64_t n0 = h->f.n;
    /* coarsening flags must refer to the leaves before refinement: map them */
    int8_t *refine = (int8_t *) malloc((size_t) n0);
    if (!refine) return CHARM_GPU_ENOMEM;
    for (int64_t i = 0; i < n0; i++) refine[i] = flags[i] > 0;
    /* remember which old leaves wanted coarsening; after refinement those
     * leaves are unchanged (a leaf is never both) and keep their order */
    int8_t *coarse_old = (int8_t *) malloc((size_t) n0);
    if (!coarse_old) { free(refine); return CHARM_GPU_ENOMEM; }
    for (int64_t i = 0; i < n0; i++) coarse_old[i] = flags[i] < 0 ? -1 : 0;
    int8_t *old_level = (int8_t *) malloc((size_t) n0);
    if (!old_level) { free(refine); free(coarse_old); return CHARM_GPU_ENOMEM; }
    for (int64_t i = 0; i < n0; i++) old_level[i] = h->f.leaf[i].level;
    if (charm_forest_refine(&h->f, refine, maxlevel, NULL, NULL) < 0) {
        free(refine); free(coarse_old); free(old_level);
        return CHARM_GPU_ENOMEM;
    }
    /* carry coarsen flags over to the refined numbering: a refined old leaf
     * became 8 consecutive new leaves, every other leaf kept its order */
    int8_t *cflag = (int8_t *) calloc((size_t) h->f.n, 1);
    if (!cflag) { free(refine); free(coarse_old); free(old_level); return CHARM_GPU_ENOMEM; }
    {
        int ml = (maxlevel < 0 || maxlevel > CHARM_FOREST_MAXLEVEL - 1) ? CHARM_FOREST_MAXLEVEL - 1 : maxlevel;
        int64_t k = 0;
        for (int64_t i = 0; i < n0; i++) {
            if (refine[i] && old_level[i] < ml) {
                k += 8;
            } else {
                cflag[k] = coarse_old[i];
                k += 1;
            }
        }
    }
    coarsen_ctx_t cc = {cflag};
    if (charm_forest_coarsen(&h->f, minlevel, coarsen_all_minus, NULL, &cc) < 0) {
        free(refine); free(coarse_old); free(cflag); free(old_level);
        return CHARM_GPU_ENOMEM;
    }
    free(refine); free(coarse_old); free(cflag); free(old_level);
    if (charm_forest_balance(&h->f, NULL, NULL) < 0) return CHARM_GPU_ENOMEM;
    free_flat(h);
    if (n_new) *n_new = h->f.n;
    return CHARM_GPU_OK;
}

/* ---- flatten ------------------------------------------------------------- */

int charm_host_forest_flatten(charm_host_forest_t h, charm_gpu_mesh_t *mesh)
{
    if (!h || !mesh) return CHARM_GPU_EINVAL;
    const charm_forest_t *f = &h->f;
    const int64_t E = f->n;
    free_flat(h);
    /* count */
    int64_t nf = 0, nb = 0;
    charm_face_nb_t nbr;
    for (int64_t i = 0; i < E; i++) {
        for (int face = 0; face < 6; face++) {
            charm_forest_face_neighbor(f, i, face, &nbr);
            switch (nbr.kind) {
            case CHARM_NB_BOUNDARY: nb++; break;
            case CHARM_NB_SAME: if (face & 1) nf++; break;
            case CHARM_NB_SMALLER: nf += 4; break;
            case CHARM_NB_BIGGER: break;
            default: return CHARM_GPU_EINVAL;   /* not 2:1 balanced */
            }
        }
    }
    h->center = (double *) malloc((size_t) (3 * E) * sizeof(double));
    h->level = (int8_t *) malloc((size_t) E);
    h->face_elem = (int32_t *) malloc((size_t) (2 * (nf > 0 ? nf : 1)) * sizeof(int32_t));
    h->face_info = (uint8_t *) malloc((size_t) (nf > 0 ? nf : 1));
    h->bface_elem = (int32_t *) malloc((size_t) (nb > 0 ? nb : 1) * sizeof(int32_t));
    h->bface_face = (int8_t *) malloc((size_t) (nb > 0 ? nb : 1));
    h->bface_bnd = (int8_t *) malloc((size_t) (nb > 0 ? nb : 1));
    if (!h->center || !h->level || !h->face_elem || !h->face_info || !h->bface_elem || !h->bface_face ||
        !h->bface_bnd) {
        free_flat(h);
        return CHARM_GPU_ENOMEM;
    }
    for (int64_t i = 0; i < E; i++) {
        double c[3], hh[3];
        charm_forest_leaf_geom(f, i, c, hh);
        h->center[i] = c[0]; h->center[E + i] = c[1]; h->center[2 * E + i] = c[2];
        h->level[i] = f->leaf[i].level;
    }
    /* interior faces grouped by direction, then by leaf order */
    int64_t k = 0;
    for (int d = 0; d < 3; d++) {
        for (int64_t i = 0; i < E; i++) {
            for (int up = 0; up < 2; up++) {
                int face = 2 * d + up;
                charm_forest_face_neighbor(f, i, face, &nbr);
                uint8_t wrap = nbr.wrap ? 0x40 : 0;
                if (nbr.kind == CHARM_NB_SAME && up) {
                    h->face_elem[k] = (int32_t) i;
                    h->face_elem[nf + k] = (int32_t) nbr.idx[0];
                    h->face_info[k] = (uint8_t) (d | wrap);
                    k++;
                } else if (nbr.kind == CHARM_NB_SMALLER) {
                    for (int j = 0; j < 4; j++) {
                        if (up) {   /* big leaf is the lower side */
                            h->face_elem[k] = (int32_t) i;
                            h->face_elem[nf + k] = (int32_t) nbr.idx[j];
                            h->face_info[k] = (uint8_t) (d | (2 << 2) | (j << 4) | wrap);
                        } else {    /* small leaves are the lower side */
                            h->face_elem[k] = (int32_t) nbr.idx[j];
                            h->face_elem[nf + k] = (int32_t) i;
                            h->face_info[k] = (uint8_t) (d | (1 << 2) | (j << 4) | wrap);
                        }
                        k++;
                    }
                }
            }
        }
    }
    int64_t kb = 0;
    for (int64_t i = 0; i < E; i++) {
        for (int face = 0; face < 6; face++) {
            charm_forest_face_neighbor(f, i, face, &nbr);
            if (nbr.kind == CHARM_NB_BOUNDARY) {
                h->bface_elem[kb] = (int32_t) i;
                h->bface_face[kb] = (int8_t) face;
                h->bface_bnd[kb] = h->bnd_of_side[face];
                kb++;
            }
        }
    }
    h->n_face = nf;
    h->n_bface = nb;
    mesh->n_elem = E;
    mesh->center = h->center;
    mesh->level = h->level;
    for (int d = 0; d < 3; d++) mesh->tree_len[d] = f->tree_len[d];
    mesh->n_face = nf;
    mesh->face_elem = h->face_elem;
    mesh->face_info = h->face_info;
    mesh->n_bface = nb;
    mesh->bface_elem = h->bface_elem;
    mesh->bface_face = h->bface_face;
    mesh->bface_bnd = h->bface_bnd;
    return CHARM_GPU_OK;
}
