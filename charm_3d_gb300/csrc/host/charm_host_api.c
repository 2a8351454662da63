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
#include "charm_conn.h"
#include "charm_forest.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void charm_internal_set_error(const char *msg);   /* the library's last-error text (charm_gpu.cu) */

struct charm_host_forest_s {
    charm_forest_t f;
    int8_t bnd_of_side[6];
    double *state;          /* state projected by the last charm_host_forest_adapt_state */
    /* projection plan of the last charm_host_forest_adapt_plan */
    int plan_n, plan_cap;
    int64_t plan_n_in;
    int64_t *plan_nout;
    int32_t **plan_map;
    /* flattened arrays (owned) */
    double  *center;
    int8_t  *level;
    int32_t *face_elem;
    uint8_t *face_info;
    int32_t *bface_elem;
    int8_t  *bface_face;
    int8_t  *bface_bnd;
    int64_t  n_face, n_bface;
    /* unstructured hexahedral mesh: the connectivity the forest points to,
     * the boundary index of every tree face, and the flattened geometry */
    charm_conn_t *conn;
    int8_t  *tree_bnd;      /* [n_tree][6], -1 where a tree face has a neighbour */
    double  *hex_vertex;    /* [8][3][E] */
    int8_t  *hex_face_face; /* [2][n_face] */
    /* flatten's scratch (keys, face-neighbour records, counts), kept between
     * flattens: an adapt loop reuses touched pages instead of faulting in
     * ~290 B per leaf each time */
    uint64_t *s_keys;
    charm_face_nb_t *s_nbs;
    int64_t *s_cnt;
    int64_t s_cap;
    /* capacities of the box flatten's arrays (leaves, faces, boundary faces),
     * which keep their memory from one flatten to the next */
    int64_t cap_e, cap_f, cap_b;
};

static void free_scratch(struct charm_host_forest_s *h)
{
    free(h->s_keys); free(h->s_nbs); free(h->s_cnt);
    h->s_keys = NULL; h->s_nbs = NULL; h->s_cnt = NULL;
    h->s_cap = 0;
}

/* scratch for E leaves (grown by a quarter when it grows) */
static int ensure_scratch(struct charm_host_forest_s *h, int64_t E)
{
    if (E <= h->s_cap && h->s_keys) return 0;
    free_scratch(h);
    const int64_t cap = (E > 0 ? E : 1) + (E >> 2);
    h->s_keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) cap);
    h->s_nbs = (charm_face_nb_t *) malloc(sizeof(charm_face_nb_t) * (size_t) (6 * cap));
    h->s_cnt = (int64_t *) malloc(sizeof(int64_t) * (size_t) (4 * cap));
    if (!h->s_keys || !h->s_nbs || !h->s_cnt) { free_scratch(h); return -1; }
    h->s_cap = cap;
    return 0;
}

static void free_flat(struct charm_host_forest_s *h)
{
    free(h->center); free(h->level); free(h->face_elem); free(h->face_info);
    free(h->bface_elem); free(h->bface_face); free(h->bface_bnd);
    free(h->hex_vertex); free(h->hex_face_face);
    h->center = NULL; h->level = NULL; h->face_elem = NULL; h->face_info = NULL;
    h->bface_elem = NULL; h->bface_face = NULL; h->bface_bnd = NULL;
    h->hex_vertex = NULL; h->hex_face_face = NULL;
    h->n_face = h->n_bface = 0;
    h->cap_e = h->cap_f = h->cap_b = 0;
}

/* After an adapt: the flattened arrays describe the old forest.  A box
 * forest keeps their memory for the next flatten (which overwrites them);
 * an unstructured one releases them. */
static void stale_flat(struct charm_host_forest_s *h)
{
    if (h->conn) free_flat(h);
    else h->n_face = h->n_bface = 0;
}

/* capacity for n items, grown by a quarter beyond n */
static int64_t grown(int64_t n) { return (n > 0 ? n : 1) + (n >> 2); }

/* realloc that keeps *p on failure; -1 then */
static int re_alloc(void **p, size_t bytes)
{
    void *q = realloc(*p, bytes);
    if (!q) return -1;
    *p = q;
    return 0;
}

/* The box flatten's arrays with room for E leaves, nf faces and nb boundary
 * faces, kept with their pages when they are large enough already. */
static int ensure_flat(struct charm_host_forest_s *h, int64_t E, int64_t nf, int64_t nb)
{
    int bad = 0;
    if (E > h->cap_e || !h->center) {
        const int64_t c = grown(E);
        bad |= re_alloc((void **) &h->center, sizeof(double) * 3 * (size_t) c);
        bad |= re_alloc((void **) &h->level, (size_t) c);
        if (!bad) h->cap_e = c;
    }
    if (nf > h->cap_f || !h->face_elem) {
        const int64_t c = grown(nf);
        bad |= re_alloc((void **) &h->face_elem, sizeof(int32_t) * 2 * (size_t) c);
        bad |= re_alloc((void **) &h->face_info, (size_t) c);
        if (!bad) h->cap_f = c;
    }
    if (nb > h->cap_b || !h->bface_elem) {
        const int64_t c = grown(nb);
        bad |= re_alloc((void **) &h->bface_elem, sizeof(int32_t) * (size_t) c);
        bad |= re_alloc((void **) &h->bface_face, (size_t) c);
        bad |= re_alloc((void **) &h->bface_bnd, (size_t) c);
        if (!bad) h->cap_b = c;
    }
    return bad ? -1 : 0;
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

static void free_plan(struct charm_host_forest_s *h)
{
    for (int p = 0; p < h->plan_n; p++) free(h->plan_map[p]);
    h->plan_n = 0;
}

int charm_host_forest_free(charm_host_forest_t h)
{
    if (!h) return CHARM_GPU_EINVAL;
    free_flat(h);
    free_plan(h);
    free(h->plan_map);
    free(h->plan_nout);
    free(h->state);
    free_scratch(h);
    charm_forest_free(&h->f);
    if (h->conn) { charm_conn_free(h->conn); free(h->conn); }
    free(h->tree_bnd);
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

/* ---- output (charm_write_solution, reference src/charm_output.c:55-120,
 * through p4est's VTK writer: cell-centre fields, level and rank per cell) -- */

int charm_host_forest_write_vtu(charm_host_forest_t h, const char *path, int n_fields, const char *const *names,
                                const double *fields)
{
    if (!h || !path || n_fields < 0 || (n_fields > 0 && (!names || !fields))) return CHARM_GPU_EINVAL;
    if (h->conn) return CHARM_GPU_ENOTSUP;
    const charm_forest_t *f = &h->f;
    const int64_t E = f->n;
    FILE *fp = fopen(path, "w");
    if (!fp) return CHARM_GPU_EINVAL;
    fprintf(fp, "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" "
                "byte_order=\"LittleEndian\">\n<UnstructuredGrid>\n"
                "<Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n",
            (long long) (8 * E), (long long) E);
    /* the 8 corners of every leaf, in VTK_HEXAHEDRON order (bottom face
     * counter-clockwise, then the top face) */
    static const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    fprintf(fp, "<Points>\n<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n");
    for (int64_t i = 0; i < E; i++) {
        double c[3], hh[3];
        charm_forest_leaf_geom(f, i, c, hh);
        for (int k = 0; k < 8; k++)
            fprintf(fp, "%.17g %.17g %.17g\n", c[0] + (corner[k][0] - 0.5) * hh[0], c[1] + (corner[k][1] - 0.5) * hh[1],
                    c[2] + (corner[k][2] - 0.5) * hh[2]);
    }
    fprintf(fp, "</DataArray>\n</Points>\n<Cells>\n<DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n");
    for (int64_t i = 0; i < E; i++)
        fprintf(fp, "%lld %lld %lld %lld %lld %lld %lld %lld\n", (long long) (8 * i), (long long) (8 * i + 1),
                (long long) (8 * i + 2), (long long) (8 * i + 3), (long long) (8 * i + 4), (long long) (8 * i + 5),
                (long long) (8 * i + 6), (long long) (8 * i + 7));
    fprintf(fp, "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n");
    for (int64_t i = 0; i < E; i++) fprintf(fp, "%lld\n", (long long) (8 * (i + 1)));
    fprintf(fp, "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
    for (int64_t i = 0; i < E; i++) fprintf(fp, "12\n");
    fprintf(fp, "</DataArray>\n</Cells>\n<CellData Scalars=\"level\">\n"
                "<DataArray type=\"Int32\" Name=\"level\" format=\"ascii\">\n");
    for (int64_t i = 0; i < E; i++) fprintf(fp, "%d\n", (int) f->leaf[i].level);
    fprintf(fp, "</DataArray>\n<DataArray type=\"Int32\" Name=\"mpirank\" format=\"ascii\">\n");
    for (int64_t i = 0; i < E; i++) fprintf(fp, "0\n");
    fprintf(fp, "</DataArray>\n");
    for (int k = 0; k < n_fields; k++) {
        fprintf(fp, "<DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n", names[k]);
        for (int64_t i = 0; i < E; i++) fprintf(fp, "%.17g\n", fields[(int64_t) k * E + i]);
        fprintf(fp, "</DataArray>\n");
    }
    fprintf(fp, "</CellData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
    const int bad = ferror(fp);
    if (fclose(fp) != 0 || bad) return CHARM_GPU_EINVAL;
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
    stale_flat(h);
    if (n_new) *n_new = h->f.n;
    return CHARM_GPU_OK;
}

/* ---- flatten ------------------------------------------------------------- */

typedef struct { const charm_forest_t *f; const uint64_t *keys; charm_face_nb_t *nbs; } nbs_ctx_t;

static void nbs_range(void *c, int64_t lo, int64_t hi)
{
    const nbs_ctx_t *n = (const nbs_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++)
        for (int face = 0; face < 6; face++) charm_forest_face_neighbor_k(n->f, n->keys, i, face, &n->nbs[6 * i + face]);
}

/* flatten, per-leaf passes (run on several threads; every leaf writes only
 * its own records, at offsets from prefix sums, so the records come out in
 * the serial order: interior faces grouped by direction, then by leaf, then
 * lower/upper face; boundary faces by leaf, then face) */
typedef struct {
    struct charm_host_forest_s *h;
    const charm_face_nb_t *nbs;
    int64_t E, nf;
    int64_t *cnt;        /* [4][E]: records per direction, boundary records; then offsets */
} flat_ctx_t;

static void flat_count_range(void *c, int64_t lo, int64_t hi)
{
    const flat_ctx_t *x = (const flat_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) {
        int64_t n[4] = {0, 0, 0, 0};
        for (int face = 0; face < 6; face++) {
            const charm_face_nb_t *nbr = &x->nbs[6 * i + face];
            switch (nbr->kind) {
            case CHARM_NB_BOUNDARY: n[3]++; break;
            case CHARM_NB_SAME: if (face & 1) n[face / 2]++; break;
            case CHARM_NB_SMALLER: n[face / 2] += 4; break;
            case CHARM_NB_BIGGER: break;
            default: n[3] = -1000000; break;   /* not 2:1 balanced */
            }
        }
        for (int d = 0; d < 4; d++) x->cnt[(int64_t) d * x->E + i] = n[d];
    }
}

static void flat_emit_range(void *c, int64_t lo, int64_t hi)
{
    const flat_ctx_t *x = (const flat_ctx_t *) c;
    struct charm_host_forest_s *h = x->h;
    const int64_t E = x->E, nf = x->nf;
    for (int64_t i = lo; i < hi; i++) {
        double cc[3], hh[3];
        charm_forest_leaf_geom(&h->f, i, cc, hh);
        h->center[i] = cc[0]; h->center[E + i] = cc[1]; h->center[2 * E + i] = cc[2];
        h->level[i] = h->f.leaf[i].level;
        for (int d = 0; d < 3; d++) {
            int64_t k = x->cnt[(int64_t) d * E + i];
            for (int up = 0; up < 2; up++) {
                const int face = 2 * d + up;
                const charm_face_nb_t *nbr = &x->nbs[6 * i + face];
                const uint8_t wrap = nbr->wrap ? 0x40 : 0;
                if (nbr->kind == CHARM_NB_SAME && up) {
                    h->face_elem[k] = (int32_t) i;
                    h->face_elem[nf + k] = (int32_t) nbr->idx[0];
                    h->face_info[k] = (uint8_t) (d | wrap);
                    k++;
                } else if (nbr->kind == CHARM_NB_SMALLER) {
                    for (int j = 0; j < 4; j++) {
                        if (up) {   /* big leaf is the lower side */
                            h->face_elem[k] = (int32_t) i;
                            h->face_elem[nf + k] = (int32_t) nbr->idx[j];
                            h->face_info[k] = (uint8_t) (d | (2 << 2) | (j << 4) | wrap);
                        } else {    /* small leaves are the lower side */
                            h->face_elem[k] = (int32_t) nbr->idx[j];
                            h->face_elem[nf + k] = (int32_t) i;
                            h->face_info[k] = (uint8_t) (d | (1 << 2) | (j << 4) | wrap);
                        }
                        k++;
                    }
                }
            }
        }
        int64_t kb = x->cnt[3 * E + i];
        for (int face = 0; face < 6; face++) {
            if (x->nbs[6 * i + face].kind == CHARM_NB_BOUNDARY) {
                h->bface_elem[kb] = (int32_t) i;
                h->bface_face[kb] = (int8_t) face;
                h->bface_bnd[kb] = h->bnd_of_side[face];
                kb++;
            }
        }
    }
}

int charm_host_forest_flatten(charm_host_forest_t h, charm_gpu_mesh_t *mesh)
{
    if (!h || !mesh) return CHARM_GPU_EINVAL;
    if (h->conn) return CHARM_GPU_ENOTSUP;   /* charm_host_forest_flatten_hex */
    const charm_forest_t *f = &h->f;
    const int64_t E = f->n;
    /* every leaf's six face-neighbour relations, found once (binary searches
     * on precomputed Morton keys) and read by the passes below */
    if (ensure_scratch(h, E)) return CHARM_GPU_ENOMEM;
    uint64_t *keys = h->s_keys;
    charm_face_nb_t *nbs = h->s_nbs;
    int64_t *cnt = h->s_cnt;
    charm_forest_keys(f, keys);
    nbs_ctx_t nc = {f, keys, nbs};
    charm_forest_parallel_for_min(E, 256, nbs_range, &nc);
    /* count, then turn the counts into offsets */
    flat_ctx_t fc = {h, nbs, E, 0, cnt};
    charm_forest_parallel_for(E, flat_count_range, &fc);
    int64_t nf = 0, nb = 0;
    for (int d = 0; d < 3; d++)
        for (int64_t i = 0; i < E; i++) {
            const int64_t n = cnt[(int64_t) d * E + i];
            cnt[(int64_t) d * E + i] = nf;
            nf += n;
        }
    for (int64_t i = 0; i < E; i++) {
        const int64_t n = cnt[3 * E + i];
        if (n < 0) return CHARM_GPU_EINVAL;   /* not 2:1 balanced */
        cnt[3 * E + i] = nb;
        nb += n;
    }
    /* the arrays keep their memory between flattens (the mesh pointers of
     * the previous flatten are invalid from here on, as before) */
    if (ensure_flat(h, E, nf, nb)) {
        free_flat(h);
        return CHARM_GPU_ENOMEM;
    }
    fc.nf = nf;
    charm_forest_parallel_for(E, flat_emit_range, &fc);
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

/* ---- adapt with the state (charm_adapt, reference src/charm_amr.c:575-610) ---- */

#include <math.h>

static void leaf_h(const charm_forest_t *f, int level, double h[3])
{
    for (int d = 0; d < 3; d++) h[d] = ldexp(f->tree_len[d], -level);
}

/* vol^(5/3) as charm_error_sqr_estimate computes it, exp(log(vol) * 5 / 3),
 * for the box volume of every level (the same value for all leaves of a
 * level, so computed once per level instead of once per leaf) */
static void level_vpow(const charm_forest_t *f, double vpow[CHARM_FOREST_MAXLEVEL + 1])
{
    for (int l = 0; l <= CHARM_FOREST_MAXLEVEL; l++) {
        double h[3];
        leaf_h(f, l, h);
        vpow[l] = exp(log(h[0] * h[1] * h[2]) * 5. / 3.);
    }
}

/* charm_error_sqr_estimate (src/charm_amr.c:12-30); vpow = vol^(5/3) */
static double err_sqr(const double *grad, int64_t E, int64_t i, double vpow)
{
    double diff2 = 0.;
    for (int k = 0; k < 3; k++) diff2 += grad[k * E + i] * grad[k * E + i];
    return diff2 * (1. / 12.) * vpow;
}

/* p1 L2 projection parent -> child for boxes (charm_replace_quads,
 * src/charm_amr.c:268-305): the child keeps the parent's linear function. */
static void project_down(const double *u, int64_t E, int64_t p, double *w, int64_t En, int64_t c, int cid, int V)
{
    const double o[3] = {(cid & 1) ? 0.25 : -0.25, (cid & 2) ? 0.25 : -0.25, (cid & 4) ? 0.25 : -0.25};
    for (int v = 0; v < V; v++) {
        const double *P = u + (int64_t) v * 4 * E;
        double *C = w + (int64_t) v * 4 * En;
        C[c] = P[p] + o[0] * P[E + p] + o[1] * P[2 * E + p] + o[2] * P[3 * E + p];
        for (int k = 1; k < 4; k++) C[(int64_t) k * En + c] = 0.5 * P[(int64_t) k * E + p];
    }
}

/* p1 L2 projection of 8 children onto their parent (charm_replace_quads,
 * src/charm_amr.c:218-266) for boxes: mean of the means, and slopes from the
 * children's means and slopes. */
static void project_up(const double *u, int64_t E, const int64_t ch[8], const int cid[8], double *w, int64_t En,
                       int64_t p, int V)
{
    for (int v = 0; v < V; v++) {
        const double *C = u + (int64_t) v * 4 * E;
        double *P = w + (int64_t) v * 4 * En;
        double m = 0., s[3] = {0., 0., 0.};
        for (int i = 0; i < 8; i++) {
            m += C[ch[i]];
            for (int k = 0; k < 3; k++) {
                const double sg = (cid[i] >> k) & 1 ? 0.375 : -0.375;
                s[k] += sg * C[ch[i]] + C[(int64_t) (k + 1) * E + ch[i]] * (1. / 16.);
            }
        }
        P[p] = m * 0.125;
        for (int k = 0; k < 3; k++) P[(int64_t) (k + 1) * En + p] = s[k];
    }
}

/* ---- general hexahedra: leaf geometry and the quadrature projections ---- */

/* Geometry of a leaf of an unstructured forest (charm_geom_quad_calc,
 * src/charm_geom.c:40-172, 496-530): corners through the tree's trilinear
 * map, the 8 Gauss points of the leaf's own trilinear map with their
 * Jacobian determinants (gw = 1), dh = the corners' bounding box, the
 * centre, the volume and the inverse of the 4x4 mass matrix. */
typedef struct {
    double c[3], dh[3], vol;
    double xq[8][3], wq[8];
    double ainv[4][4];
} hexg_t;

static void hex_leaf_geom(const charm_conn_t *conn, const charm_leaf_t *q, hexg_t *g)
{
    const double inv = 1.0 / (double) CHARM_FOREST_ROOT_LEN;
    const int32_t len = CHARM_FOREST_QLEN(q->level);
    double v[8][3];
    for (int k = 0; k < 8; k++)
        charm_conn_point(conn, q->tree, (double) (q->x + ((k & 1) ? len : 0)) * inv,
                         (double) (q->y + ((k & 2) ? len : 0)) * inv, (double) (q->z + ((k & 4) ? len : 0)) * inv, v[k]);
    const double s3 = 0.57735026918962576451;
    for (int q8 = -1; q8 < 8; q8++) {
        const double r[3] = {q8 < 0 ? 0.0 : ((q8 & 1) ? s3 : -s3), q8 < 0 ? 0.0 : ((q8 & 2) ? s3 : -s3),
                             q8 < 0 ? 0.0 : ((q8 & 4) ? s3 : -s3)};
        double x[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int k = 0; k < 8; k++) {
            const double sx = (k & 1) ? 1.0 : -1.0, sy = (k & 2) ? 1.0 : -1.0, sz = (k & 4) ? 1.0 : -1.0;
            const double wx = 1.0 + sx * r[0], wy = 1.0 + sy * r[1], wz = 1.0 + sz * r[2];
            for (int d = 0; d < 3; d++) {
                x[d] += wz * wy * wx * 0.125 * v[k][d];
                J[d][0] += wz * wy * sx * 0.125 * v[k][d];
                J[d][1] += wz * wx * sy * 0.125 * v[k][d];
                J[d][2] += wy * wx * sz * 0.125 * v[k][d];
            }
        }
        if (q8 < 0) { memcpy(g->c, x, sizeof(x)); continue; }
        memcpy(g->xq[q8], x, sizeof(x));
        g->wq[q8] = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                    J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    }
    for (int d = 0; d < 3; d++) {
        double lo = v[0][d], hi = v[0][d];
        for (int k = 1; k < 8; k++) {
            if (lo > v[k][d]) lo = v[k][d];
            if (hi < v[k][d]) hi = v[k][d];
        }
        g->dh[d] = hi - lo;
    }
    g->vol = 0.0;
    for (int q8 = 0; q8 < 8; q8++) g->vol += g->wq[q8];
    double a[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double acc = 0.0;
            for (int q8 = 0; q8 < 8; q8++) {
                const double pi = i ? (g->xq[q8][i - 1] - g->c[i - 1]) / g->dh[i - 1] : 1.0;
                const double pj = j ? (g->xq[q8][j - 1] - g->c[j - 1]) / g->dh[j - 1] : 1.0;
                acc += g->wq[q8] * pi * pj;
            }
            a[i][j] = acc;
            g->ainv[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int i = 0; i < 4; i++) {   /* Gauss-Jordan with partial pivoting (charm_matr_inv) */
        int p = i;
        for (int r = i + 1; r < 4; r++)
            if (fabs(a[r][i]) > fabs(a[p][i])) p = r;
        for (int j = 0; p != i && j < 4; j++) {
            double t = a[i][j]; a[i][j] = a[p][j]; a[p][j] = t;
            t = g->ainv[i][j]; g->ainv[i][j] = g->ainv[p][j]; g->ainv[p][j] = t;
        }
        const double piv = a[i][i];
        for (int j = 0; j < 4; j++) { a[i][j] /= piv; g->ainv[i][j] /= piv; }
        for (int r = 0; r < 4; r++) {
            if (r == i) continue;
            const double fct = a[r][i];
            for (int j = 0; j < 4; j++) { a[r][j] -= fct * a[i][j]; g->ainv[r][j] -= fct * g->ainv[i][j]; }
        }
    }
}

static double hex_phi(const hexg_t *g, const double x[3], int k)
{   /* charm_base_func, src/charm_base_func.c:8-20 */
    return k ? (x[k - 1] - g->c[k - 1]) / g->dh[k - 1] : 1.0;
}

/* charm_replace_quads (src/charm_amr.c:206-307) on general hexahedra: the
 * L2 projection of the source leaves' fields onto the target leaf's basis,
 * by the quadrature of the target (refine: one child from its parent) or
 * of each source (coarsen: the parent from its 8 children):
 * w_t = A_t^-1 sum_q gw gj phi_t(x_q) u_s(x_q). */
static void hex_project_down(const hexg_t *P, const hexg_t *C, const double *u, int64_t E, int64_t p, double *w,
                             int64_t En, int64_t c, int V)
{
    for (int v = 0; v < V; v++) {
        double rhs[4] = {0, 0, 0, 0};
        for (int q = 0; q < 8; q++) {
            double up = 0.0;
            for (int n = 0; n < 4; n++) up += u[((int64_t) v * 4 + n) * E + p] * hex_phi(P, C->xq[q], n);
            for (int m = 0; m < 4; m++) rhs[m] += C->wq[q] * hex_phi(C, C->xq[q], m) * up;
        }
        for (int k = 0; k < 4; k++)
            w[((int64_t) v * 4 + k) * En + c] =
                C->ainv[k][0] * rhs[0] + C->ainv[k][1] * rhs[1] + C->ainv[k][2] * rhs[2] + C->ainv[k][3] * rhs[3];
    }
}

static void hex_project_up(const hexg_t *P, const hexg_t C[8], const double *u, int64_t E, int64_t i0, double *w,
                           int64_t En, int64_t k, int V)
{
    for (int v = 0; v < V; v++) {
        double rhs[4] = {0, 0, 0, 0};
        for (int i = 0; i < 8; i++)
            for (int q = 0; q < 8; q++) {
                double uc = 0.0;
                for (int n = 0; n < 4; n++) uc += u[((int64_t) v * 4 + n) * E + i0 + i] * hex_phi(&C[i], C[i].xq[q], n);
                for (int m = 0; m < 4; m++) rhs[m] += C[i].wq[q] * hex_phi(P, C[i].xq[q], m) * uc;
            }
        for (int b = 0; b < 4; b++)
            w[((int64_t) v * 4 + b) * En + k] =
                P->ainv[b][0] * rhs[0] + P->ainv[b][1] * rhs[1] + P->ainv[b][2] * rhs[2] + P->ainv[b][3] * rhs[3];
    }
}

static double hex_leaf_vol(const charm_conn_t *conn, const charm_leaf_t *q)
{
    hexg_t g;
    hex_leaf_geom(conn, q, &g);
    return g.vol;
}

static void parent_of(const charm_leaf_t *c, charm_leaf_t *p)
{
    const int32_t len = CHARM_FOREST_QLEN(c->level);
    p->x = c->x & ~len; p->y = c->y & ~len; p->z = c->z & ~len;
    p->tree = c->tree;
    p->level = (int8_t) (c->level - 1);
}

static void child_leaf(const charm_leaf_t *p, int cid, charm_leaf_t *c)
{
    const int32_t h = CHARM_FOREST_QLEN(p->level + 1);
    c->x = p->x + ((cid & 1) ? h : 0); c->y = p->y + ((cid & 2) ? h : 0); c->z = p->z + ((cid & 4) ? h : 0);
    c->tree = p->tree;
    c->level = (int8_t) (p->level + 1);
}

/* refine flagged leaves one level (charm_forest_refine_map); o2n[E] gets
 * each old leaf's first new index (the identity when nothing is refined) */
static int refine_o2n(charm_forest_t *f, const int8_t *fl, int64_t **o2n)
{
    const int64_t E = f->n;
    int64_t *m = (int64_t *) malloc(sizeof(int64_t) * (size_t) (E + 1));
    if (!m) return CHARM_GPU_ENOMEM;
    const int64_t r = charm_forest_refine_map(f, fl, -1, NULL, NULL, m);
    if (r < 0) { free(m); return CHARM_GPU_ENOMEM; }
    if (r == 0)
        for (int64_t i = 0; i < E; i++) m[i] = i;
    m[E] = f->n;   /* end of the last old leaf's outputs */
    *o2n = m;
    return CHARM_GPU_OK;
}

typedef struct {
    const charm_forest_t *f;   /* refined */
    const int64_t *o2n;        /* [E + 1] */
    int64_t E, En;
    int V;
    const double *u;           /* state (refine_state) or densities (refine_plan) before */
    double *w;                 /* after */
    int32_t *map;              /* plan pass (refine_plan) */
} refine_pass_ctx_t;

static void refine_state_range(void *c, int64_t lo, int64_t hi)
{
    const refine_pass_ctx_t *x = (const refine_pass_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) {
        const int64_t k = x->o2n[i];
        if (x->o2n[i + 1] - k == 8 && x->f->conn) {
            charm_leaf_t pl;
            hexg_t P, C;
            parent_of(&x->f->leaf[k], &pl);
            hex_leaf_geom(x->f->conn, &pl, &P);
            for (int ch = 0; ch < 8; ch++) {
                hex_leaf_geom(x->f->conn, &x->f->leaf[k + ch], &C);
                hex_project_down(&P, &C, x->u, x->E, i, x->w, x->En, k + ch, x->V);
            }
        } else if (x->o2n[i + 1] - k == 8) {
            for (int ch = 0; ch < 8; ch++)
                project_down(x->u, x->E, i, x->w, x->En, k + ch, charm_leaf_child_id(&x->f->leaf[k + ch]), x->V);
        } else {
            for (int v = 0; v < x->V; v++)
                for (int b = 0; b < 4; b++)
                    x->w[((int64_t) v * 4 + b) * x->En + k] = x->u[((int64_t) v * 4 + b) * x->E + i];
        }
    }
}

/* refine flagged leaves one level, projecting the state */
static int refine_state(charm_forest_t *f, const int8_t *fl, int V, double **u, int64_t **o2n_out)
{
    const int64_t E = f->n;
    int64_t *o2n = NULL;
    int rc = refine_o2n(f, fl, &o2n);
    if (rc) return rc;
    const int64_t En = f->n;
    double *w = (double *) malloc(sizeof(double) * (size_t) V * 4 * (size_t) En);
    if (!w) { free(o2n); return CHARM_GPU_ENOMEM; }
    refine_pass_ctx_t x = {f, o2n, E, En, V, *u, w, NULL};
    charm_forest_parallel_for(E, refine_state_range, &x);
    if (o2n_out) *o2n_out = o2n;
    else free(o2n);
    free(*u);
    *u = w;
    return CHARM_GPU_OK;
}

/* Append a pass to the plan (takes ownership of map). */
static int plan_push(struct charm_host_forest_s *h, int64_t n_out, int32_t *map)
{
    if (h->plan_n == h->plan_cap) {
        const int cap = h->plan_cap ? 2 * h->plan_cap : 8;
        int64_t *no = (int64_t *) realloc(h->plan_nout, sizeof(int64_t) * (size_t) cap);
        if (!no) return CHARM_GPU_ENOMEM;
        h->plan_nout = no;
        int32_t **nm = (int32_t **) realloc(h->plan_map, sizeof(int32_t *) * (size_t) cap);
        if (!nm) return CHARM_GPU_ENOMEM;
        h->plan_map = nm;
        h->plan_cap = cap;
    }
    h->plan_nout[h->plan_n] = n_out;
    h->plan_map[h->plan_n] = map;
    h->plan_n++;
    return CHARM_GPU_OK;
}

/* refine flagged leaves one level and record the pass: output leaf k is a
 * copy of old leaf i (op -1) or child cid of old leaf i (op cid); the
 * centre densities *rho follow (children: NaN, never read: families made in
 * this adapt are not coarsened) */
static void refine_plan_range(void *c, int64_t lo, int64_t hi)
{
    const refine_pass_ctx_t *x = (const refine_pass_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) {
        const int64_t k = x->o2n[i];
        if (x->o2n[i + 1] - k == 8) {
            for (int ch = 0; ch < 8; ch++) {
                x->map[2 * (k + ch)] = (int32_t) i;
                x->map[2 * (k + ch) + 1] = charm_leaf_child_id(&x->f->leaf[k + ch]);
                x->w[k + ch] = NAN;
            }
        } else {
            x->map[2 * k] = (int32_t) i;
            x->map[2 * k + 1] = -1;
            x->w[k] = x->u[i];
        }
    }
}

static int refine_plan(struct charm_host_forest_s *h, const int8_t *fl, double **rho, int64_t **o2n_out)
{
    charm_forest_t *f = &h->f;
    const int64_t E = f->n;
    int64_t *o2n = NULL;
    int rc = refine_o2n(f, fl, &o2n);
    if (rc) return rc;
    const int64_t En = f->n;
    int32_t *map = (int32_t *) malloc(sizeof(int32_t) * 2 * (size_t) (En > 0 ? En : 1));
    double *r = (double *) malloc(sizeof(double) * (size_t) (En > 0 ? En : 1));
    if (!map || !r) { free(o2n); free(map); free(r); return CHARM_GPU_ENOMEM; }
    refine_pass_ctx_t x = {f, o2n, E, En, 1, *rho, r, map};
    charm_forest_parallel_for(E, refine_plan_range, &x);
    if (o2n_out) *o2n_out = o2n;
    else free(o2n);
    free(*rho);
    *rho = r;
    rc = plan_push(h, En, map);
    if (rc) free(map);
    return rc;
}

typedef struct {
    const charm_forest_t *f;
    const double *grad;        /* per current leaf, NaN for leaves new in this adapt */
    const double *rho;         /* centre densities per current leaf (plan mode), else NULL */
    const double *u;
    int64_t E;
    int nc, minlevel;
    double err2_max;
    const double *vpow;        /* vol^(5/3) per level */
    const int8_t *xflags;      /* caller's flags per current leaf (0 for new leaves), or NULL */
} coarsen_state_ctx_t;

/* charm_coarsen_err_estimate (src/charm_amr.c:90-142) */
static int coarsen_family(void *user, const charm_leaf_t *leaves, const int64_t idx[8])
{
    const coarsen_state_ctx_t *c = (const coarsen_state_ctx_t *) user;
    if (leaves[idx[0]].level <= c->minlevel) return 0;
    if (c->xflags) {   /* the caller's criterion: every child flagged -1 */
        for (int i = 0; i < 8; i++)
            if (c->xflags[idx[i]] != -1) return 0;
        return 1;
    }
    double h[3];
    leaf_h(c->f, leaves[idx[0]].level, h);
    /* the first child's volume stands for every child (as the reference's
     * "the quadrant's volume is also its volume fraction"); each child's
     * own estimate uses its own volume */
    const double vol = c->f->conn ? hex_leaf_vol(c->f->conn, &leaves[idx[0]]) : h[0] * h[1] * h[2];
    double r[8], parentu = 0.;
    for (int i = 0; i < 8; i++) {
        double ri = 0.;   /* prim.r at the centre: sum of the partial-density means, eos flag 4 clamp */
        if (c->rho) ri = c->rho[idx[i]];
        else
            for (int s = 0; s < c->nc; s++) ri += c->u[((int64_t) (4 + s) * 4) * c->E + idx[i]];
        if (ri < 1.e-12) ri = 1.e-12;
        r[i] = ri;
        parentu += ri / 8;
    }
    double err2 = 0.;
    for (int i = 0; i < 8; i++) {
        const double vp = c->f->conn ? exp(log(hex_leaf_vol(c->f->conn, &leaves[idx[i]])) * 5. / 3.)
                                     : c->vpow[leaves[idx[0]].level];
        const double childerr2 = err_sqr(c->grad, c->E, idx[i], vp);
        if (childerr2 > c->err2_max * vol) return 0;
        err2 += childerr2;
        const double diff = (parentu - r[i]) * (parentu - r[i]);
        err2 += diff * vol;
    }
    return err2 < c->err2_max * (vol * 8) ? 1 : 0;
}

typedef struct {
    const charm_forest_t *f;
    const double *grad;
    int64_t E;
    int ml;
    double err2_max;
    const double *vpow;
    double vol[CHARM_FOREST_MAXLEVEL + 1];   /* box volume per level */
    int8_t *fl;
} refine_flags_ctx_t;

/* charm_refine_err_estimate's test per leaf (src/charm_amr.c:32-47) */
static void refine_flags_range(void *c, int64_t lo, int64_t hi)
{
    const refine_flags_ctx_t *x = (const refine_flags_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) {
        const int l = x->f->leaf[i].level;
        if (l >= x->ml) continue;
        if (x->f->conn) {   /* each leaf's own volume */
            const double vol = hex_leaf_vol(x->f->conn, &x->f->leaf[i]);
            x->fl[i] = err_sqr(x->grad, x->E, i, exp(log(vol) * 5. / 3.)) > x->err2_max * vol;
        } else {
            x->fl[i] = err_sqr(x->grad, x->E, i, x->vpow[l]) > x->err2_max * x->vol[l];
        }
    }
}

/* the coarsen pass after charm_forest_coarsen_map: new leaf k is old leaf
 * n2o[k] (op -1) or the parent of the family n2o[k] .. n2o[k] + 7, child
 * ids 0..7 in Morton order (op 8); the state is projected (state mode) or
 * the pass recorded (plan mode), and the new-leaf marks follow */
typedef struct {
    const charm_forest_t *f;   /* coarsened */
    const int64_t *n2o;        /* [En + 1] */
    int64_t E, En;
    int V;
    const double *u;           /* state before (state mode) */
    double *w;                 /* state after (state mode) */
    int32_t *map;              /* plan pass (plan mode) */
    const int8_t *isnew;       /* [E] */
    int8_t *isnew2;            /* [En] */
} coarsen_pass_ctx_t;

static void coarsen_pass_range(void *c, int64_t lo, int64_t hi)
{
    const coarsen_pass_ctx_t *x = (const coarsen_pass_ctx_t *) c;
    static const int cid[8] = {0, 1, 2, 3, 4, 5, 6, 7};
    for (int64_t k = lo; k < hi; k++) {
        const int64_t i = x->n2o[k];
        const int merged = (x->n2o[k + 1] - i == 8);
        x->isnew2[k] = merged ? 1 : x->isnew[i];
        if (x->map) {
            x->map[2 * k] = (int32_t) i;
            x->map[2 * k + 1] = merged ? 8 : -1;
        } else if (merged && x->f->conn) {
            hexg_t P, C[8];
            hex_leaf_geom(x->f->conn, &x->f->leaf[k], &P);
            for (int j = 0; j < 8; j++) {
                charm_leaf_t cl;
                child_leaf(&x->f->leaf[k], j, &cl);
                hex_leaf_geom(x->f->conn, &cl, &C[j]);
            }
            hex_project_up(&P, C, x->u, x->E, i, x->w, x->En, k, x->V);
        } else if (merged) {
            int64_t ch[8];
            for (int j = 0; j < 8; j++) ch[j] = i + j;
            project_up(x->u, x->E, ch, cid, x->w, x->En, k, x->V);
        } else {
            for (int v = 0; v < x->V; v++)
                for (int b = 0; b < 4; b++)
                    x->w[((int64_t) v * 4 + b) * x->En + k] = x->u[((int64_t) v * 4 + b) * x->E + i];
        }
    }
}

/* the refine's old-to-new map o2n [E0 + 1] carries each old leaf's
 * gradient to its new index, NaN for the children of a refined leaf */
typedef struct {
    const int64_t *o2n;
    const double *grad;        /* [3][E0] */
    int64_t E0, E1;
    double *g1;                /* [3][E1] */
    int8_t *isnew;             /* [E1] */
    const int8_t *xf;          /* caller's flags [E0], or NULL */
    int8_t *xf1;               /* [E1]: carried over, 0 for new leaves */
} grad_fill_ctx_t;

static void grad_fill_range(void *c, int64_t lo, int64_t hi)
{
    const grad_fill_ctx_t *x = (const grad_fill_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) {
        const int64_t k = x->o2n[i], n = x->o2n[i + 1] - k;
        for (int64_t j = k; j < k + n; j++) {
            for (int d = 0; d < 3; d++) x->g1[(int64_t) d * x->E1 + j] = (n == 8) ? NAN : x->grad[(int64_t) d * x->E0 + i];
            x->isnew[j] = (int8_t) (n == 8);
            if (x->xf) x->xf1[j] = (n == 8) ? (int8_t) 0 : x->xf[i];
        }
    }
}

/* The adapt of charm_adapt.  State mode (u_in): the state [V][4][E] is
 * projected along, into h->state.  Plan mode (rho_in): only the centre
 * densities [E] that the coarsening criterion reads are carried, and every
 * projection is recorded as a pass of h's plan instead. */
static int adapt_core(struct charm_host_forest_s *h, const double *grad, double max_err, int minlevel, int maxlevel,
                      int n_comp, const double *u_in, const double *rho_in, const int8_t *xflags, int64_t *n_new)
{
    charm_forest_t *f = &h->f;
    const int V = 4 + n_comp;
    const int64_t E0 = f->n;
    const double err2_max = max_err * max_err;
    const int ml = (maxlevel < 0 || maxlevel > CHARM_FOREST_MAXLEVEL - 1) ? CHARM_FOREST_MAXLEVEL - 1 : maxlevel;
    const int plan = (u_in == NULL);
    double *u = NULL, *rho = NULL;
    if (plan) {
        free_plan(h);
        h->plan_n_in = E0;
        rho = (double *) malloc(sizeof(double) * (size_t) (E0 > 0 ? E0 : 1));
        if (!rho) return CHARM_GPU_ENOMEM;
        memcpy(rho, rho_in, sizeof(double) * (size_t) E0);
    } else {
        u = (double *) malloc(sizeof(double) * (size_t) V * 4 * (size_t) E0);
        if (!u) return CHARM_GPU_ENOMEM;
        memcpy(u, u_in, sizeof(double) * (size_t) V * 4 * (size_t) E0);
    }
    int8_t *fl = (int8_t *) calloc((size_t) E0 + 1, 1);
    if (!fl) { free(u); free(rho); return CHARM_GPU_ENOMEM; }
    double vpow[CHARM_FOREST_MAXLEVEL + 1];
    level_vpow(f, vpow);
    /* 1. refine (charm_refine_err_estimate, non-recursive, maxlevel; or the
     * caller's flags) */
    if (xflags) {
        for (int64_t i = 0; i < E0; i++) fl[i] = (xflags[i] == 1 && f->leaf[i].level < ml) ? 1 : 0;
    } else {
        refine_flags_ctx_t rc1 = {f, grad, E0, ml, err2_max, vpow, {0}, fl};
        for (int l = 0; l <= CHARM_FOREST_MAXLEVEL; l++) {
            double hh[3];
            leaf_h(f, l, hh);
            rc1.vol[l] = hh[0] * hh[1] * hh[2];
        }
        charm_forest_parallel_for(E0, refine_flags_range, &rc1);
    }
    int64_t *o2n = NULL;
    int rc = plan ? refine_plan(h, fl, &rho, &o2n) : refine_state(f, fl, V, &u, &o2n);
    free(fl);
    if (rc) { free(u); free(rho); free(o2n); return rc; }
    /* the gradient of the leaves after refinement: unchanged leaves keep theirs,
     * new children get NaN, so their family is never coarsened in this adapt;
     * and the leaves that did not exist before this adapt (children made by
     * the refine, then parents made by the coarsen), in the current numbering */
    const int64_t E1 = f->n;
    double *g1 = (double *) malloc(sizeof(double) * 3 * (size_t) E1);
    int8_t *isnew = (int8_t *) malloc((size_t) E1 + 1);
    int8_t *xf1 = xflags ? (int8_t *) malloc((size_t) E1 + 1) : NULL;
    if (!g1 || !isnew || (xflags && !xf1)) {
        free(u); free(rho); free(g1); free(isnew); free(o2n); free(xf1);
        return CHARM_GPU_ENOMEM;
    }
    {
        grad_fill_ctx_t gf = {o2n, grad, E0, E1, g1, isnew, xflags, xf1};
        charm_forest_parallel_for(E0, grad_fill_range, &gf);
    }
    free(o2n);
    /* 2. coarsen complete families (charm_coarsen_err_estimate, non-recursive) */
    {
        const int64_t E = f->n;
        int64_t *n2o = (int64_t *) malloc(sizeof(int64_t) * (size_t) (E + 1));
        if (!n2o) { free(u); free(rho); free(g1); free(isnew); return CHARM_GPU_ENOMEM; }
        coarsen_state_ctx_t cc = {f, g1, rho, u, E, n_comp, minlevel, err2_max, vpow, xf1};
        int64_t nm = charm_forest_coarsen_map(f, minlevel, coarsen_family, &cc, n2o);
        if (nm < 0) { free(n2o); free(u); free(rho); free(g1); free(isnew); return CHARM_GPU_ENOMEM; }
        if (nm > 0) {
            const int64_t En = f->n;
            double *w = plan ? NULL : (double *) malloc(sizeof(double) * (size_t) V * 4 * (size_t) En);
            int32_t *map = plan ? (int32_t *) malloc(sizeof(int32_t) * 2 * (size_t) En) : NULL;
            int8_t *isnew2 = (int8_t *) malloc((size_t) En + 1);
            if ((plan ? !map : !w) || !isnew2) {
                free(w); free(map); free(isnew2); free(n2o); free(u); free(rho); free(g1); free(isnew);
                return CHARM_GPU_ENOMEM;
            }
            coarsen_pass_ctx_t cp = {f, n2o, E, En, V, u, w, map, isnew, isnew2};
            charm_forest_parallel_for(En, coarsen_pass_range, &cp);
            free(isnew);
            isnew = isnew2;
            if (plan) {
                if ((rc = plan_push(h, En, map))) { free(map); free(n2o); free(rho); free(g1); free(isnew); return rc; }
            } else {
                free(u);
                u = w;
            }
        }
        free(n2o);
    }
    free(g1);
    free(xf1);
    free(rho);   /* the balance passes do not read densities */
    rho = NULL;
    /* 3. 2:1 face balance, one level per pass (p4est_balance_ext with
     * charm_replace_quads).  The forest was balanced before this adapt (every
     * call that changes it ends balanced), and a pair of leaves that both
     * existed before keeps its face relation; so a pass only checks the
     * leaves made since the last balanced forest (by the refine and coarsen
     * above, then by the previous pass) and their face neighbours. */
    int64_t *cand = NULL, n_cand = -1;   /* -1: every leaf */
    {
        int64_t nfr = 0;
        for (int64_t k = 0; k < f->n; k++) nfr += isnew[k];
        if (4 * nfr <= f->n) {           /* else most leaves are new: check them all */
            int64_t *list = (int64_t *) malloc(sizeof(int64_t) * (size_t) (nfr + 1));
            cand = (int64_t *) malloc(sizeof(int64_t) * (size_t) (f->n + 1));
            if (!list || !cand) { free(list); free(cand); free(isnew); free(u); return CHARM_GPU_ENOMEM; }
            nfr = 0;
            for (int64_t k = 0; k < f->n; k++)
                if (isnew[k]) list[nfr++] = k;
            n_cand = charm_forest_fresh_neighbourhood(f, list, nfr, cand);
            free(list);
            if (n_cand < 0) { free(cand); free(isnew); free(u); return CHARM_GPU_ENOMEM; }
        }
        free(isnew);
    }
    for (;;) {
        const int64_t nold = f->n;
        int8_t *bf = (int8_t *) calloc((size_t) nold + 1, 1);
        int8_t *lv = (int8_t *) malloc((size_t) nold + 1);
        if (!bf || !lv) { free(bf); free(lv); free(cand); free(u); return CHARM_GPU_ENOMEM; }
        for (int64_t i = 0; i < nold; i++) lv[i] = f->leaf[i].level;
        const int64_t marks = (n_cand < 0) ? charm_forest_balance_marks(f, bf)
                                           : charm_forest_balance_marks_at(f, cand, n_cand, bf);
        free(cand);
        cand = NULL;
        if (marks) {
            if (plan) {
                double *dummy = (double *) calloc((size_t) nold + 1, sizeof(double));
                rc = dummy ? refine_plan(h, bf, &dummy, NULL) : CHARM_GPU_ENOMEM;
                free(dummy);
            } else {
                rc = refine_state(f, bf, V, &u, NULL);
            }
            if (!rc) {
                /* the children made by this pass, at their new indices */
                int64_t *fresh = (int64_t *) malloc(sizeof(int64_t) * (size_t) (8 * marks + 1));
                cand = (int64_t *) malloc(sizeof(int64_t) * (size_t) (f->n + 1));
                if (!fresh || !cand) {
                    rc = CHARM_GPU_ENOMEM;
                } else {
                    int64_t nf = 0, k = 0;
                    for (int64_t i = 0; i < nold; i++) {
                        if (bf[i] && lv[i] < CHARM_FOREST_MAXLEVEL - 1) {
                            for (int c = 0; c < 8; c++) fresh[nf++] = k + c;
                            k += 8;
                        } else {
                            k++;
                        }
                    }
                    n_cand = charm_forest_fresh_neighbourhood(f, fresh, nf, cand);
                    if (n_cand < 0) rc = CHARM_GPU_ENOMEM;
                }
                free(fresh);
            }
        }
        free(bf);
        free(lv);
        if (rc) { free(cand); free(u); return rc; }
        if (!marks) break;
    }
    free(cand);
    if (!plan) {
        free(h->state);
        h->state = u;
    }
    stale_flat(h);
    if (n_new) *n_new = f->n;
    return CHARM_GPU_OK;
}

int charm_host_forest_adapt_state(charm_host_forest_t h, const double *grad, double max_err, int minlevel, int maxlevel,
                                  int n_comp, const double *u_in, int64_t *n_new)
{
    if (!h || !grad || !u_in || n_comp < 1 || n_comp > CHARM_GPU_MAX_COMP) return CHARM_GPU_EINVAL;
    return adapt_core(h, grad, max_err, minlevel, maxlevel, n_comp, u_in, NULL, NULL, n_new);
}

int charm_host_forest_adapt_plan(charm_host_forest_t h, const double *grad, const double *rho, double max_err,
                                 int minlevel, int maxlevel, int64_t *n_new, charm_gpu_adapt_plan_t *plan)
{
    if (!h || !grad || !rho) return CHARM_GPU_EINVAL;
    if (h->conn) return CHARM_GPU_ENOTSUP;   /* the device projection is the box form */
    int rc = adapt_core(h, grad, max_err, minlevel, maxlevel, 1, NULL, rho, NULL, n_new);
    if (rc) return rc;
    if (plan) {
        plan->n_pass = h->plan_n;
        plan->n_in = h->plan_n_in;
        plan->n_out = h->plan_nout;
        plan->map = (const int32_t *const *) h->plan_map;
    }
    return CHARM_GPU_OK;
}

int charm_host_forest_adapt_plan_flags(charm_host_forest_t h, const int8_t *flags, int minlevel, int maxlevel,
                                       int64_t *n_new, charm_gpu_adapt_plan_t *plan)
{
    if (!h || !flags) return CHARM_GPU_EINVAL;
    if (h->conn) return CHARM_GPU_ENOTSUP;   /* the device projection is the box form */
    const int64_t E = h->f.n;
    /* the criteria are not evaluated: a zero gradient and unit densities
     * only fill the arrays the adapt carries */
    double *zg = (double *) calloc((size_t) 3 * (size_t) (E > 0 ? E : 1), sizeof(double));
    double *one = (double *) malloc(sizeof(double) * (size_t) (E > 0 ? E : 1));
    if (!zg || !one) { free(zg); free(one); return CHARM_GPU_ENOMEM; }
    for (int64_t i = 0; i < E; i++) one[i] = 1.0;
    int rc = adapt_core(h, zg, 0.0, minlevel, maxlevel, 1, NULL, one, flags, n_new);
    free(zg);
    free(one);
    if (rc) return rc;
    if (plan) {
        plan->n_pass = h->plan_n;
        plan->n_in = h->plan_n_in;
        plan->n_out = h->plan_nout;
        plan->map = (const int32_t *const *) h->plan_map;
    }
    return CHARM_GPU_OK;
}

int charm_host_forest_state(charm_host_forest_t h, const double **u_out)
{
    if (!h || !u_out) return CHARM_GPU_EINVAL;
    if (!h->state) return CHARM_GPU_ESTATE;
    *u_out = h->state;
    return CHARM_GPU_OK;
}

/* ---- unstructured hexahedral meshes ------------------------------------------ */

static int new_conn_forest(charm_host_forest_t *out, charm_conn_t *conn, int8_t *tree_bnd, int level)
{
    struct charm_host_forest_s *h = (struct charm_host_forest_s *) calloc(1, sizeof(*h));
    if (!h) { charm_conn_free(conn); free(conn); free(tree_bnd); return CHARM_GPU_ENOMEM; }
    h->conn = conn;
    h->tree_bnd = tree_bnd;
    if (charm_forest_init_conn(&h->f, conn, level)) { charm_host_forest_free(h); return CHARM_GPU_EINVAL; }
    *out = h;
    return CHARM_GPU_OK;
}

int charm_host_forest_new_hex(charm_host_forest_t *out, int32_t n_vert, const double *vert, int32_t n_tree,
                              const int32_t *t2v, const int8_t *tree_bnd, int level)
{
    if (!out || !vert || !t2v || !tree_bnd || n_vert <= 0 || n_tree <= 0) return CHARM_GPU_EINVAL;
    charm_conn_t *c = (charm_conn_t *) calloc(1, sizeof(*c));
    int8_t *tb = (int8_t *) malloc(6 * (size_t) n_tree);
    if (!c || !tb) { free(c); free(tb); return CHARM_GPU_ENOMEM; }
    char err[256];
    if (charm_conn_build(c, n_vert, vert, n_tree, t2v, err, (int) sizeof(err))) {
        free(c); free(tb);
        charm_internal_set_error(err);
        return CHARM_GPU_EINVAL;
    }
    for (size_t k = 0; k < 6 * (size_t) n_tree; k++) {
        tb[k] = (c->t2t[k] < 0) ? tree_bnd[k] : (int8_t) -1;
        if (c->t2t[k] < 0 && tb[k] < 0) {
            charm_conn_free(c); free(c); free(tb);
            charm_internal_set_error("boundary tree face without a boundary index");
            return CHARM_GPU_EINVAL;
        }
    }
    return new_conn_forest(out, c, tb, level);
}

int charm_host_forest_new_gmsh(charm_host_forest_t *out, const char *path, int level, int n_bnd,
                               const char *const *bnd_names)
{
    if (!out || !path || n_bnd < 0 || (n_bnd > 0 && !bnd_names)) return CHARM_GPU_EINVAL;
    charm_conn_t *c = (charm_conn_t *) calloc(1, sizeof(*c));
    if (!c) return CHARM_GPU_ENOMEM;
    char err[512];
    if (charm_conn_read_gmsh(c, path, err, (int) sizeof(err))) {
        free(c);
        charm_internal_set_error(err);
        return CHARM_GPU_EINVAL;
    }
    int8_t *tb = (int8_t *) malloc(6 * (size_t) c->n_tree);
    if (!tb) { charm_conn_free(c); free(c); return CHARM_GPU_ENOMEM; }
    /* a boundary face takes the configured boundary of its patch's physical
     * name (charm_conn_bnd_find_by_id, src/charm_connectivity.c:176-203) */
    for (size_t k = 0; k < 6 * (size_t) c->n_tree; k++) {
        tb[k] = -1;
        if (c->t2t[k] >= 0) continue;
        const char *name = (c->bnd_tag[k] >= 0) ? charm_conn_patch_name(c, 2, c->bnd_tag[k]) : NULL;
        for (int b = 0; name && b < n_bnd; b++)
            if (bnd_names[b] && !strcmp(bnd_names[b], name)) { tb[k] = (int8_t) b; break; }
        if (tb[k] < 0) {
            snprintf(err, sizeof(err), "%s: tree %lld face %d: %s%s%s", path, (long long) (k / 6), (int) (k % 6),
                     name ? "patch '" : "boundary face without a physical quadrangle",
                     name ? name : "", name ? "' is not a configured boundary" : "");
            charm_conn_free(c); free(c); free(tb);
            charm_internal_set_error(err);
            return CHARM_GPU_EINVAL;
        }
    }
    return new_conn_forest(out, c, tb, level);
}

int charm_host_forest_tree_count(charm_host_forest_t h)
{
    if (!h) return -1;
    return h->conn ? h->conn->n_tree : h->f.ntree[0] * h->f.ntree[1] * h->f.ntree[2];
}

int charm_host_forest_tree_region(charm_host_forest_t h, int32_t *reg_tag)
{
    if (!h || !reg_tag) return CHARM_GPU_EINVAL;
    if (!h->conn) return CHARM_GPU_ENOTSUP;
    memcpy(reg_tag, h->conn->reg_tag, sizeof(int32_t) * (size_t) h->conn->n_tree);
    return CHARM_GPU_OK;
}

/* Side 0 of a face between two leaves: inside a tree the leaf at the lower
 * coordinate (its face is odd), across a tree face the leaf of the lower
 * tree, as p4est_iterate visits a tree face from its lower tree. */
static int is_side0(const charm_forest_t *f, int64_t i, int face, int64_t j)
{
    const int32_t ti = f->leaf[i].tree, tj = f->leaf[j].tree;
    if (ti != tj) return ti < tj;
    return face & 1;
}

typedef struct {
    struct charm_host_forest_s *h;
    const charm_face_nb_t *nbs;
    int64_t E, nf;
    int64_t *cnt;        /* [2][E]: interior records, boundary records; then offsets */
} hex_ctx_t;

static void hex_count_range(void *c, int64_t lo, int64_t hi)
{
    const hex_ctx_t *x = (const hex_ctx_t *) c;
    const charm_forest_t *f = &x->h->f;
    for (int64_t i = lo; i < hi; i++) {
        int64_t ni = 0, nb = 0;
        for (int face = 0; face < 6; face++) {
            const charm_face_nb_t *n = &x->nbs[6 * i + face];
            switch (n->kind) {
            case CHARM_NB_BOUNDARY: nb++; break;
            case CHARM_NB_SAME: if (is_side0(f, i, face, n->idx[0])) ni++; break;
            case CHARM_NB_SMALLER: ni += 4; break;
            case CHARM_NB_BIGGER: break;
            default: nb = -1000000; break;
            }
        }
        x->cnt[i] = ni;
        x->cnt[x->E + i] = nb;
    }
}

static void hex_emit_range(void *c, int64_t lo, int64_t hi)
{
    const hex_ctx_t *x = (const hex_ctx_t *) c;
    struct charm_host_forest_s *h = x->h;
    const charm_forest_t *f = &h->f;
    const int64_t E = x->E, nf = x->nf;
    const double inv = 1.0 / (double) CHARM_FOREST_ROOT_LEN;
    for (int64_t i = lo; i < hi; i++) {
        const charm_leaf_t *q = &f->leaf[i];
        const int32_t len = CHARM_FOREST_QLEN(q->level);
        /* corners by the tree's trilinear map (charm_quad_get_vertices,
         * src/charm_geom.c:12-31), centre at the quadrant's middle
         * (_charm_quad_calc_center, :33-37) */
        for (int k = 0; k < 8; k++) {
            double v[3];
            charm_conn_point(h->conn, q->tree, (double) (q->x + ((k & 1) ? len : 0)) * inv,
                             (double) (q->y + ((k & 2) ? len : 0)) * inv, (double) (q->z + ((k & 4) ? len : 0)) * inv, v);
            for (int d = 0; d < 3; d++) h->hex_vertex[(int64_t) (3 * k + d) * E + i] = v[d];
        }
        double cc[3];
        charm_conn_point(h->conn, q->tree, ((double) q->x + 0.5 * len) * inv, ((double) q->y + 0.5 * len) * inv,
                         ((double) q->z + 0.5 * len) * inv, cc);
        h->center[i] = cc[0]; h->center[E + i] = cc[1]; h->center[2 * E + i] = cc[2];
        h->level[i] = q->level;
        int64_t k = x->cnt[i];
        for (int face = 0; face < 6; face++) {
            const charm_face_nb_t *n = &x->nbs[6 * i + face];
            if (n->kind == CHARM_NB_SAME && is_side0(f, i, face, n->idx[0])) {
                h->face_elem[k] = (int32_t) i;
                h->face_elem[nf + k] = (int32_t) n->idx[0];
                h->face_info[k] = (uint8_t) (face / 2);
                h->hex_face_face[k] = (int8_t) face;
                h->hex_face_face[nf + k] = (int8_t) n->nface;
                k++;
            } else if (n->kind == CHARM_NB_SMALLER) {
                const int big0 = is_side0(f, i, face, n->idx[0]);
                for (int j = 0; j < 4; j++) {
                    const int32_t a = big0 ? (int32_t) i : (int32_t) n->idx[j];
                    const int32_t b = big0 ? (int32_t) n->idx[j] : (int32_t) i;
                    h->face_elem[k] = a;
                    h->face_elem[nf + k] = b;
                    h->face_info[k] = (uint8_t) (((big0 ? face : n->nface) / 2) | ((big0 ? 2 : 1) << 2) | (j << 4));
                    h->hex_face_face[k] = (int8_t) (big0 ? face : n->nface);
                    h->hex_face_face[nf + k] = (int8_t) (big0 ? n->nface : face);
                    k++;
                }
            }
        }
        int64_t kb = x->cnt[E + i];
        for (int face = 0; face < 6; face++) {
            if (x->nbs[6 * i + face].kind == CHARM_NB_BOUNDARY) {
                h->bface_elem[kb] = (int32_t) i;
                h->bface_face[kb] = (int8_t) face;
                h->bface_bnd[kb] = h->tree_bnd[6 * (int64_t) q->tree + face];
                kb++;
            }
        }
    }
}

int charm_host_forest_flatten_hex(charm_host_forest_t h, charm_gpu_mesh_t *mesh, charm_gpu_hex_t *hex)
{
    if (!h || !mesh || !hex) return CHARM_GPU_EINVAL;
    if (!h->conn) return CHARM_GPU_ENOTSUP;
    const charm_forest_t *f = &h->f;
    const int64_t E = f->n;
    free_flat(h);
    uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (E > 0 ? E : 1));
    charm_face_nb_t *nbs = (charm_face_nb_t *) malloc(sizeof(charm_face_nb_t) * (size_t) (6 * (E > 0 ? E : 1)));
    int64_t *cnt = (int64_t *) malloc(sizeof(int64_t) * (size_t) (2 * (E > 0 ? E : 1)));
    if (!keys || !nbs || !cnt) { free(keys); free(nbs); free(cnt); return CHARM_GPU_ENOMEM; }
    charm_forest_keys(f, keys);
    nbs_ctx_t nc = {f, keys, nbs};
    charm_forest_parallel_for_min(E, 256, nbs_range, &nc);
    free(keys);
    hex_ctx_t hc = {h, nbs, E, 0, cnt};
    charm_forest_parallel_for(E, hex_count_range, &hc);
    int64_t nf = 0, nb = 0;
    for (int64_t i = 0; i < E; i++) {
        const int64_t a = cnt[i], b = cnt[E + i];
        if (b < 0) { free(nbs); free(cnt); return CHARM_GPU_EINVAL; }   /* not 2:1 balanced */
        cnt[i] = nf; nf += a;
        cnt[E + i] = nb; nb += b;
    }
    h->center = (double *) malloc((size_t) (3 * (E > 0 ? E : 1)) * sizeof(double));
    h->level = (int8_t *) malloc((size_t) (E > 0 ? E : 1));
    h->face_elem = (int32_t *) malloc((size_t) (2 * (nf > 0 ? nf : 1)) * sizeof(int32_t));
    h->face_info = (uint8_t *) malloc((size_t) (nf > 0 ? nf : 1));
    h->bface_elem = (int32_t *) malloc((size_t) (nb > 0 ? nb : 1) * sizeof(int32_t));
    h->bface_face = (int8_t *) malloc((size_t) (nb > 0 ? nb : 1));
    h->bface_bnd = (int8_t *) malloc((size_t) (nb > 0 ? nb : 1));
    h->hex_vertex = (double *) malloc((size_t) (24 * (E > 0 ? E : 1)) * sizeof(double));
    h->hex_face_face = (int8_t *) malloc((size_t) (2 * (nf > 0 ? nf : 1)));
    if (!h->center || !h->level || !h->face_elem || !h->face_info || !h->bface_elem || !h->bface_face ||
        !h->bface_bnd || !h->hex_vertex || !h->hex_face_face) {
        free_flat(h);
        free(nbs);
        free(cnt);
        return CHARM_GPU_ENOMEM;
    }
    hc.nf = nf;
    charm_forest_parallel_for(E, hex_emit_range, &hc);
    free(nbs);
    free(cnt);
    h->n_face = nf;
    h->n_bface = nb;
    mesh->n_elem = E;
    mesh->center = h->center;
    mesh->level = h->level;
    for (int d = 0; d < 3; d++) mesh->tree_len[d] = 1.0;
    mesh->n_face = nf;
    mesh->face_elem = h->face_elem;
    mesh->face_info = h->face_info;
    mesh->n_bface = nb;
    mesh->bface_elem = h->bface_elem;
    mesh->bface_face = h->bface_face;
    mesh->bface_bnd = h->bface_bnd;
    hex->vertex = h->hex_vertex;
    hex->face_face = h->hex_face_face;
    return CHARM_GPU_OK;
}
