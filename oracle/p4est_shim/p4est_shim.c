/*
 * p4est-subset shim: implementation (oracle build only, see p4est_to_p8est.h).
 *
 * One rank, a brick of trees or an unstructured hexahedral connectivity
 * (one tree per hexahedron, trees in any face orientation), leaves held by
 * the host octree of the GPU library (charm_3d_gb300/csrc/host/charm_forest.c,
 * charm_conn.c).  Behaviour kept from p4est because CHARM_3D's arithmetic
 * depends on it:
 *   - p4est_iterate face sides: side 0 at the lower coordinate (its face
 *     2*dir+1), side 1 at the upper inside a tree and in a brick; across
 *     the faces of an unstructured connectivity side 0 is the leaf of the
 *     lower tree, as p4est visits a tree face from its lower tree; a hanging
 *     side lists its 4 small quadrants in z-order on the face; boundary
 *     faces have one side;
 *   - p4est_qcoord_to_vertex: trilinear map of the tree's 8 vertices;
 *   - refine/coarsen/balance call init_fn for new quadrants and replace_fn
 *     with (outgoing, incoming) families; balance refines one level at a
 *     time, so replace_fn always sees 1 -> 8 there.
 * Two departures, both documented where the oracle is described:
 *   - periodic faces: p4est would hand both real quadrants to the face
 *     callback, which CHARM_3D's basis evaluation cannot handle (the two
 *     centres are a period apart).  The shim instead presents each wrap face
 *     twice, once per side, with the far quadrant as a ghost whose geometry
 *     is shifted by the period; ghost sides receive no contribution
 *     (reference src/models/euler/charm_model.c:357).
 *   - user data of quadrants created by refine/coarsen/balance is filled
 *     with NaN bytes instead of p4est's recycled memory, so reads of fields
 *     the reference never initialised are NaN rather than stale values.
 */
#include "p4est_to_p8est.h"
#include "charm_conn.h"
#include "charm_forest.h"

#include <stdarg.h>
#include <time.h>

/* ---- libsc subset ---------------------------------------------------------- */

static int shim_verbose(void)
{
    static int v = -1;
    if (v < 0) v = getenv("CHARM_SHIM_VERBOSE") != NULL;
    return v;
}

void sc_shim_log(int priority, const char *s)
{
    if (shim_verbose() || priority >= SC_LP_ERROR) fputs(s, stderr);
}

void sc_shim_logf(int priority, const char *fmt, ...)
{
    if (!(shim_verbose() || priority >= SC_LP_ERROR)) return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
}

double sc_MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

int sc_MPI_Allreduce(void *send, void *recv, int count, int type, int op, sc_MPI_Comm comm)
{
    (void) op; (void) comm;
    memcpy(recv, send, (size_t) count * (type == sc_MPI_DOUBLE ? sizeof(double) : sizeof(int)));
    return 0;
}

int MPI_Finalize(void) { return 0; }
void sc_finalize(void) {}

void sc_array_init(sc_array_t *a, size_t elem_size)
{
    a->elem_size = elem_size;
    a->elem_count = 0;
    a->byte_alloc = 0;
    a->array = NULL;
}

sc_array_t *sc_array_new(size_t elem_size)
{
    sc_array_t *a = (sc_array_t *) malloc(sizeof(sc_array_t));
    sc_array_init(a, elem_size);
    return a;
}

void sc_array_resize(sc_array_t *a, size_t n)
{
    size_t need = n * a->elem_size;
    if ((ssize_t) need > a->byte_alloc) {
        size_t cap = a->byte_alloc > 0 ? (size_t) a->byte_alloc : 64;
        while (cap < need) cap *= 2;
        a->array = (char *) realloc(a->array, cap);
        a->byte_alloc = (ssize_t) cap;
    }
    a->elem_count = n;
}

sc_array_t *sc_array_new_size(size_t elem_size, size_t n)
{
    sc_array_t *a = sc_array_new(elem_size);
    sc_array_resize(a, n);
    return a;
}

void sc_array_reset(sc_array_t *a)
{
    free(a->array);
    sc_array_init(a, a->elem_size);
}

void sc_array_destroy(sc_array_t *a)
{
    if (!a) return;
    free(a->array);
    free(a);
}

void *sc_array_push(sc_array_t *a)
{
    sc_array_resize(a, a->elem_count + 1);
    return sc_array_index(a, a->elem_count - 1);
}

/* ---- forest state ---------------------------------------------------------- */

struct charm_shim_state {
    charm_forest_t f;
    p4est_quadrant_t *q;   /* one per leaf, in leaf order */
};

/* Hook set by ref_driver.c: shift the geometry of a ghost copy by `shift`. */
void (*charm_shim_ghost_shift)(void *data, const double shift[3]) = NULL;

static void *new_data(p4est_t *p, int nan_fill)
{
    void *d = malloc(p->data_size > 0 ? p->data_size : 1);
    memset(d, nan_fill ? 0xff : 0, p->data_size);
    return d;
}

/* Counts and the per-tree views p4est keeps: tree t's quadrants are the
 * leaves [quadrants_offset, quadrants_offset + count) of the global order. */
static void sync_counts(p4est_t *p)
{
    struct charm_shim_state *s = p->shim;
    p->local_num_quadrants = (p4est_locidx_t) s->f.n;
    p->global_num_quadrants = s->f.n;
    if (!p->trees) p->trees = sc_array_new(sizeof(p4est_tree_t));
    sc_array_resize(p->trees, (size_t) p->connectivity->num_trees);
    int64_t i = 0;
    for (p4est_topidx_t t = 0; t < p->connectivity->num_trees; t++) {
        p4est_tree_t *tr = p4est_tree_array_index(p->trees, t);
        int64_t start = i;
        int8_t ml = 0;
        while (i < s->f.n && s->f.leaf[i].tree == t) {
            if (s->f.leaf[i].level > ml) ml = s->f.leaf[i].level;
            i++;
        }
        tr->quadrants.elem_size = sizeof(p4est_quadrant_t);
        tr->quadrants.elem_count = (size_t) (i - start);
        tr->quadrants.byte_alloc = -1;
        tr->quadrants.array = (char *) (s->q + start);
        tr->quadrants_offset = (p4est_locidx_t) start;
        tr->maxlevel = ml;
    }
}

/* index of a local leaf within its tree, as p4est reports quadid */
static p4est_locidx_t tree_local(p4est_t *p, int64_t i)
{
    return (p4est_locidx_t) (i - p4est_tree_array_index(p->trees, p->shim->f.leaf[i].tree)->quadrants_offset);
}

p4est_connectivity_t *charm_shim_conn_brick(int nx, int ny, int nz, const int periodic[3], const double origin[3],
                                            const double tree_len[3], size_t attr_bytes)
{
    p4est_connectivity_t *c = (p4est_connectivity_t *) calloc(1, sizeof(*c));
    c->brick[0] = nx; c->brick[1] = ny; c->brick[2] = nz;
    for (int d = 0; d < 3; d++) {
        c->periodic[d] = periodic ? periodic[d] : 0;
        c->origin[d] = origin ? origin[d] : 0.0;
        c->tree_len[d] = tree_len ? tree_len[d] : 1.0;
    }
    c->num_trees = nx * ny * nz;
    c->num_vertices = (nx + 1) * (ny + 1) * (nz + 1);
    c->vertices = (double *) malloc(sizeof(double) * 3 * (size_t) c->num_vertices);
    for (int k = 0; k <= nz; k++)
        for (int j = 0; j <= ny; j++)
            for (int i = 0; i <= nx; i++) {
                int v = i + (nx + 1) * (j + (ny + 1) * k);
                c->vertices[3 * v + 0] = c->origin[0] + c->tree_len[0] * i;
                c->vertices[3 * v + 1] = c->origin[1] + c->tree_len[1] * j;
                c->vertices[3 * v + 2] = c->origin[2] + c->tree_len[2] * k;
            }
    c->tree_to_vertex = (p4est_topidx_t *) malloc(sizeof(p4est_topidx_t) * 8 * (size_t) c->num_trees);
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int t = i + nx * (j + ny * k);
                for (int cc = 0; cc < 8; cc++) {
                    int ii = i + (cc & 1), jj = j + ((cc >> 1) & 1), kk = k + ((cc >> 2) & 1);
                    c->tree_to_vertex[8 * t + cc] = ii + (nx + 1) * (jj + (ny + 1) * kk);
                }
            }
    c->tree_attr_bytes = attr_bytes;
    c->tree_to_attr = (char *) calloc((size_t) c->num_trees, attr_bytes > 0 ? attr_bytes : 1);
    return c;
}

/* Unstructured connectivity: n_tree hexahedra with their corner vertices in
 * p4est order; tree faces matched by their vertex sets (the role of
 * p4est_connectivity_complete).  NULL when the faces do not match. */
p4est_connectivity_t *charm_shim_conn_hex(int32_t n_vert, const double *vert, int32_t n_tree, const int32_t *t2v,
                                          size_t attr_bytes)
{
    charm_conn_t *hc = (charm_conn_t *) calloc(1, sizeof(charm_conn_t));
    char err[256];
    if (!hc || charm_conn_build(hc, n_vert, vert, n_tree, t2v, err, (int) sizeof(err))) {
        fprintf(stderr, "p4est shim: %s\n", hc ? err : "out of memory");
        free(hc);
        return NULL;
    }
    p4est_connectivity_t *c = (p4est_connectivity_t *) calloc(1, sizeof(*c));
    c->num_trees = n_tree;
    c->num_vertices = n_vert;
    c->vertices = (double *) malloc(sizeof(double) * 3 * (size_t) n_vert);
    memcpy(c->vertices, vert, sizeof(double) * 3 * (size_t) n_vert);
    c->tree_to_vertex = (p4est_topidx_t *) malloc(sizeof(p4est_topidx_t) * 8 * (size_t) n_tree);
    for (int64_t k = 0; k < 8 * (int64_t) n_tree; k++) c->tree_to_vertex[k] = t2v[k];
    c->brick[0] = n_tree; c->brick[1] = 1; c->brick[2] = 1;
    for (int d = 0; d < 3; d++) c->tree_len[d] = 1.0;
    c->tree_attr_bytes = attr_bytes;
    c->tree_to_attr = (char *) calloc((size_t) n_tree, attr_bytes > 0 ? attr_bytes : 1);
    c->hexconn = hc;
    return c;
}

void charm_shim_conn_destroy(p4est_connectivity_t *c)
{
    if (!c) return;
    if (c->hexconn) { charm_conn_free((charm_conn_t *) c->hexconn); free(c->hexconn); }
    free(c->vertices); free(c->tree_to_vertex); free(c->tree_to_attr); free(c);
}

void p4est_qcoord_to_vertex(p4est_connectivity_t *conn, p4est_topidx_t treeid, p4est_qcoord_t x, p4est_qcoord_t y,
                            p4est_qcoord_t z, double vxyz[3])
{
    const double *vert = conn->vertices;
    const p4est_topidx_t *vi = conn->tree_to_vertex + 8 * treeid;
    double wx[2], wy[2], wz[2];
    wx[1] = (double) x / (double) P4EST_ROOT_LEN; wx[0] = 1. - wx[1];
    wy[1] = (double) y / (double) P4EST_ROOT_LEN; wy[0] = 1. - wy[1];
    wz[1] = (double) z / (double) P4EST_ROOT_LEN; wz[0] = 1. - wz[1];
    vxyz[0] = vxyz[1] = vxyz[2] = 0.;
    int k = 0;
    for (int zi = 0; zi < 2; zi++)
        for (int yi = 0; yi < 2; yi++) {
            double yf = wz[zi] * wy[yi];
            for (int xi = 0; xi < 2; xi++) {
                double xf = yf * wx[xi];
                const double *v = vert + 3 * vi[k++];
                vxyz[0] += xf * v[0];
                vxyz[1] += xf * v[1];
                vxyz[2] += xf * v[2];
            }
        }
}

static void fill_quad(p4est_quadrant_t *q, const charm_leaf_t *l)
{
    q->x = l->x; q->y = l->y; q->z = l->z;
    q->level = l->level; q->pad8 = 0; q->pad16 = 0;
}

p4est_t *p4est_new_ext(sc_MPI_Comm mpicomm, p4est_connectivity_t *conn, p4est_locidx_t min_quadrants, int min_level,
                       int fill_uniform, size_t data_size, p4est_init_t init_fn, void *user_pointer)
{
    (void) min_quadrants; (void) fill_uniform;
    p4est_t *p = (p4est_t *) calloc(1, sizeof(p4est_t));
    p->mpicomm = mpicomm;
    p->mpisize = 1;
    p->mpirank = 0;
    p->data_size = data_size;
    p->user_pointer = user_pointer;
    p->connectivity = conn;
    p->first_local_tree = 0;
    p->last_local_tree = conn->num_trees - 1;
    p->shim = (struct charm_shim_state *) calloc(1, sizeof(struct charm_shim_state));
    if (conn->hexconn) charm_forest_init_conn(&p->shim->f, (const charm_conn_t *) conn->hexconn, min_level);
    else charm_forest_init_uniform(&p->shim->f, conn->brick, conn->periodic, conn->origin, conn->tree_len, min_level);
    int64_t n = p->shim->f.n;
    p->shim->q = (p4est_quadrant_t *) calloc((size_t) n, sizeof(p4est_quadrant_t));
    for (int64_t i = 0; i < n; i++) {
        fill_quad(&p->shim->q[i], &p->shim->f.leaf[i]);
        p->shim->q[i].p.user_data = new_data(p, 0);
    }
    sync_counts(p);
    if (init_fn)
        for (int64_t i = 0; i < n; i++) init_fn(p, p->shim->f.leaf[i].tree, &p->shim->q[i]);
    return p;
}

void p4est_destroy(p4est_t *p)
{
    if (!p) return;
    sc_array_destroy(p->trees);
    for (int64_t i = 0; i < p->shim->f.n; i++) free(p->shim->q[i].p.user_data);
    free(p->shim->q);
    charm_forest_free(&p->shim->f);
    free(p->shim);
    free(p);
}

/* Shim accessors used by the oracle driver. */
int64_t charm_shim_count(p4est_t *p) { return p->shim->f.n; }
p4est_quadrant_t *charm_shim_quad(p4est_t *p, int64_t i) { return &p->shim->q[i]; }
int32_t charm_shim_tree(p4est_t *p, int64_t i) { return p->shim->f.leaf[i].tree; }
const charm_forest_t *charm_shim_forest(p4est_t *p) { return &p->shim->f; }

/* ---- refine / coarsen / balance --------------------------------------------- */

/* Split every flagged leaf into 8 children (one level), keeping user data of
 * the others; init_fn on each child, then replace_fn(parent -> children). */
static int64_t refine_flagged(p4est_t *p, const int8_t *flag, int maxlevel, p4est_init_t init_fn,
                              p4est_replace_t replace_fn, int8_t **is_new)
{
    struct charm_shim_state *s = p->shim;
    const int64_t n0 = s->f.n;
    int ml = (maxlevel < 0 || maxlevel > P4EST_QMAXLEVEL) ? P4EST_QMAXLEVEL : maxlevel;
    int8_t *fl = (int8_t *) calloc((size_t) n0 + 1, 1);
    int64_t nref = 0;
    for (int64_t i = 0; i < n0; i++) {
        fl[i] = flag[i] && s->f.leaf[i].level < ml;
        nref += fl[i];
    }
    if (nref == 0) {
        free(fl);
        if (is_new) *is_new = (int8_t *) calloc((size_t) n0 + 1, 1);
        return 0;
    }
    p4est_quadrant_t *oldq = s->q;
    charm_forest_refine(&s->f, fl, -1, NULL, NULL);
    const int64_t n1 = s->f.n;
    p4est_quadrant_t *nq = (p4est_quadrant_t *) calloc((size_t) n1, sizeof(p4est_quadrant_t));
    int8_t *nw = (int8_t *) calloc((size_t) n1 + 1, 1);
    int64_t k = 0;
    for (int64_t i = 0; i < n0; i++) {
        if (fl[i]) {
            for (int c = 0; c < 8; c++) {
                fill_quad(&nq[k + c], &s->f.leaf[k + c]);
                nq[k + c].p.user_data = new_data(p, 1);
                nw[k + c] = 1;
            }
            k += 8;
        } else {
            nq[k] = oldq[i];
            k++;
        }
    }
    s->q = nq;
    sync_counts(p);
    k = 0;
    for (int64_t i = 0; i < n0; i++) {
        if (fl[i]) {
            p4est_quadrant_t *out[1] = {&oldq[i]};
            p4est_quadrant_t *in[8];
            for (int c = 0; c < 8; c++) {
                in[c] = &nq[k + c];
                if (init_fn) init_fn(p, s->f.leaf[k + c].tree, in[c]);
            }
            if (replace_fn) replace_fn(p, s->f.leaf[k].tree, 1, out, 8, in);
            free(oldq[i].p.user_data);
            k += 8;
        } else {
            k++;
        }
    }
    free(oldq);
    free(fl);
    if (is_new) *is_new = nw; else free(nw);
    return nref;
}

void p4est_refine_ext(p4est_t *p, int refine_recursive, int maxlevel, p4est_refine_t refine_fn, p4est_init_t init_fn,
                      p4est_replace_t replace_fn)
{
    struct charm_shim_state *s = p->shim;
    int ml = (maxlevel < 0 || maxlevel > P4EST_QMAXLEVEL) ? P4EST_QMAXLEVEL : maxlevel;
    int8_t *check = (int8_t *) malloc((size_t) s->f.n + 1);
    memset(check, 1, (size_t) s->f.n + 1);
    for (;;) {
        const int64_t n = s->f.n;
        int8_t *flag = (int8_t *) calloc((size_t) n + 1, 1);
        int64_t cnt = 0;
        for (int64_t i = 0; i < n; i++) {
            if (check[i] && s->f.leaf[i].level < ml && refine_fn(p, s->f.leaf[i].tree, &s->q[i])) {
                flag[i] = 1;
                cnt++;
            }
        }
        int8_t *nw = NULL;
        if (cnt) refine_flagged(p, flag, ml, init_fn, replace_fn, &nw);
        free(flag);
        free(check);
        if (!cnt || !refine_recursive) { free(nw); break; }
        check = nw;
    }
}

void p4est_refine(p4est_t *p, int refine_recursive, p4est_refine_t refine_fn, p4est_init_t init_fn)
{
    p4est_refine_ext(p, refine_recursive, -1, refine_fn, init_fn, NULL);
}

typedef struct {
    p4est_t *p;
    p4est_coarsen_t fn;
} coarsen_ud_t;

static int coarsen_pred(void *user, const charm_leaf_t *leaves, const int64_t idx[8])
{
    coarsen_ud_t *u = (coarsen_ud_t *) user;
    p4est_quadrant_t *fam[8];
    for (int c = 0; c < 8; c++) fam[c] = &u->p->shim->q[idx[c]];
    return u->fn(u->p, leaves[idx[0]].tree, fam);
}

static int64_t coarsen_once(p4est_t *p, p4est_coarsen_t coarsen_fn, p4est_init_t init_fn, p4est_replace_t replace_fn)
{
    struct charm_shim_state *s = p->shim;
    const int64_t n0 = s->f.n;
    charm_leaf_t *old_leaves = (charm_leaf_t *) malloc(sizeof(charm_leaf_t) * (size_t) (n0 + 1));
    memcpy(old_leaves, s->f.leaf, sizeof(charm_leaf_t) * (size_t) n0);
    p4est_quadrant_t *oldq = s->q;
    coarsen_ud_t ud = {p, coarsen_fn};
    int64_t nm = charm_forest_coarsen(&s->f, -1, coarsen_pred, NULL, &ud);
    if (nm <= 0) { free(old_leaves); return 0; }
    const int64_t n1 = s->f.n;
    p4est_quadrant_t *nq = (p4est_quadrant_t *) calloc((size_t) n1, sizeof(p4est_quadrant_t));
    /* walk old and new leaf arrays together */
    int64_t i = 0;
    for (int64_t k = 0; k < n1; k++) {
        const charm_leaf_t *nl = &s->f.leaf[k];
        const charm_leaf_t *ol = &old_leaves[i];
        if (ol->level == nl->level && ol->x == nl->x && ol->y == nl->y && ol->z == nl->z && ol->tree == nl->tree) {
            nq[k] = oldq[i];
            i++;
        } else {
            fill_quad(&nq[k], nl);
            nq[k].p.user_data = new_data(p, 1);
            if (init_fn) init_fn(p, nl->tree, &nq[k]);
            p4est_quadrant_t *out[8];
            for (int c = 0; c < 8; c++) out[c] = &oldq[i + c];
            p4est_quadrant_t *in[1] = {&nq[k]};
            s->q = nq;
            if (replace_fn) replace_fn(p, nl->tree, 8, out, 1, in);
            for (int c = 0; c < 8; c++) free(oldq[i + c].p.user_data);
            i += 8;
        }
    }
    s->q = nq;
    sync_counts(p);
    free(oldq);
    free(old_leaves);
    return nm;
}

void p4est_coarsen_ext(p4est_t *p, int coarsen_recursive, int callback_orphans, p4est_coarsen_t coarsen_fn,
                       p4est_init_t init_fn, p4est_replace_t replace_fn)
{
    (void) callback_orphans;
    while (coarsen_once(p, coarsen_fn, init_fn, replace_fn) > 0 && coarsen_recursive) {
    }
}

void p4est_coarsen(p4est_t *p, int coarsen_recursive, p4est_coarsen_t coarsen_fn, p4est_init_t init_fn)
{
    p4est_coarsen_ext(p, coarsen_recursive, 0, coarsen_fn, init_fn, NULL);
}

void p4est_balance_ext(p4est_t *p, p4est_connect_type_t btype, p4est_init_t init_fn, p4est_replace_t replace_fn)
{
    (void) btype;   /* CHARM_3D balances with CHARM_CONNECT_FACE only */
    struct charm_shim_state *s = p->shim;
    for (;;) {
        int8_t *flag = (int8_t *) calloc((size_t) s->f.n + 1, 1);
        int64_t m = charm_forest_balance_marks(&s->f, flag);
        if (m) refine_flagged(p, flag, -1, init_fn, replace_fn, NULL);
        free(flag);
        if (!m) break;
    }
}

void p4est_balance(p4est_t *p, p4est_connect_type_t btype, p4est_init_t init_fn)
{
    p4est_balance_ext(p, btype, init_fn, NULL);
}

p4est_gloidx_t p4est_partition(p4est_t *p, int allow_for_coarsening, p4est_weight_t weight_fn)
{
    (void) p; (void) allow_for_coarsening; (void) weight_fn;
    return 0;
}

/* ---- ghosts (periodic emulation) -------------------------------------------- */

static double domain_len(const p4est_connectivity_t *c, int d) { return c->tree_len[d] * c->brick[d]; }

/* find or add the ghost (src, shift along d by sign*period) */
static int64_t ghost_lookup(p4est_ghost_t *g, int64_t src, int d, int sign, int add, p4est_t *p)
{
    for (size_t k = 0; k < g->ghosts.elem_count; k++) {
        if (g->src[k] != src) continue;
        double want[3] = {0, 0, 0};
        want[d] = sign * domain_len(p->connectivity, d);
        if (g->shift[3 * k] == want[0] && g->shift[3 * k + 1] == want[1] && g->shift[3 * k + 2] == want[2])
            return (int64_t) k;
    }
    if (!add) return -1;
    size_t k = g->ghosts.elem_count;
    p4est_quadrant_t *gq = (p4est_quadrant_t *) sc_array_push(&g->ghosts);
    *gq = p->shim->q[src];
    gq->p.user_data = NULL;
    g->src = (int64_t *) realloc(g->src, sizeof(int64_t) * (k + 1));
    g->shift = (double *) realloc(g->shift, sizeof(double) * 3 * (k + 1));
    g->src[k] = src;
    g->shift[3 * k] = g->shift[3 * k + 1] = g->shift[3 * k + 2] = 0.0;
    g->shift[3 * k + d] = sign * domain_len(p->connectivity, d);
    return (int64_t) k;
}

p4est_ghost_t *p4est_ghost_new(p4est_t *p, p4est_connect_type_t btype)
{
    p4est_ghost_t *g = (p4est_ghost_t *) calloc(1, sizeof(p4est_ghost_t));
    g->mpisize = 1;
    g->num_trees = p->connectivity->num_trees;
    g->btype = btype;
    sc_array_init(&g->ghosts, sizeof(p4est_quadrant_t));
    const charm_forest_t *f = &p->shim->f;
    charm_face_nb_t nb;
    for (int64_t i = 0; i < f->n; i++)
        for (int face = 0; face < 6; face++) {
            charm_forest_face_neighbor(f, i, face, &nb);
            if (!nb.wrap) continue;
            int cnt = (nb.kind == CHARM_NB_SMALLER) ? 4 : 1;
            for (int k = 0; k < cnt; k++) ghost_lookup(g, nb.idx[k], face / 2, nb.wrap, 1, p);
        }
    return g;
}

void p4est_ghost_destroy(p4est_ghost_t *g)
{
    if (!g) return;
    sc_array_reset(&g->ghosts);
    free(g->src);
    free(g->shift);
    free(g);
}

void p4est_ghost_exchange_data(p4est_t *p, p4est_ghost_t *g, void *ghost_data)
{
    if (!g || !ghost_data) return;
    char *dst = (char *) ghost_data;
    for (size_t k = 0; k < g->ghosts.elem_count; k++) {
        memcpy(dst + k * p->data_size, p->shim->q[g->src[k]].p.user_data, p->data_size);
        if (charm_shim_ghost_shift) charm_shim_ghost_shift(dst + k * p->data_size, &g->shift[3 * k]);
    }
}

/* ---- iterate ------------------------------------------------------------------ */

static void side_full(p4est_iter_face_side_t *sd, int32_t tree, int face, p4est_quadrant_t *q, int ghost,
                      p4est_locidx_t id)
{
    memset(sd, 0, sizeof(*sd));
    sd->treeid = tree;
    sd->face = (int8_t) face;
    sd->is_hanging = 0;
    sd->is.full.is_ghost = (int8_t) ghost;
    sd->is.full.quad = q;
    sd->is.full.quadid = id;
}

static void side_hanging(p4est_iter_face_side_t *sd, int32_t tree, int face, p4est_quadrant_t *q[4],
                         const int8_t ghost[4], const p4est_locidx_t id[4])
{
    memset(sd, 0, sizeof(*sd));
    sd->treeid = tree;
    sd->face = (int8_t) face;
    sd->is_hanging = 1;
    for (int k = 0; k < 4; k++) {
        sd->is.hanging.is_ghost[k] = ghost[k];
        sd->is.hanging.quad[k] = q[k];
        sd->is.hanging.quadid[k] = id[k];
    }
}

static void call_face(p4est_t *p, p4est_ghost_t *g, void *ud, p4est_iter_face_t fn, int nsides,
                      p4est_iter_face_side_t sides[2], int tree_boundary)
{
    p4est_iter_face_info_t info;
    info.p4est = p;
    info.ghost_layer = g;
    info.orientation = 0;
    info.tree_boundary = (int8_t) tree_boundary;
    sc_array_init(&info.sides, sizeof(p4est_iter_face_side_t));
    sc_array_resize(&info.sides, (size_t) nsides);
    memcpy(info.sides.array, sides, sizeof(p4est_iter_face_side_t) * (size_t) nsides);
    fn(&info, ud);
    sc_array_reset(&info.sides);
}

static int64_t ghost_id(p4est_t *p, p4est_ghost_t *g, int64_t src, int d, int sign)
{
    int64_t k = g ? ghost_lookup(g, src, d, sign, 0, p) : -1;
    if (k < 0) {
        fprintf(stderr, "p4est shim: periodic face iterated without its ghost layer\n");
        abort();
    }
    return k;
}

void p4est_iterate(p4est_t *p, p4est_ghost_t *g, void *ud, p4est_iter_volume_t vol_fn, p4est_iter_face_t face_fn,
                   void *edge_fn, void *corner_fn)
{
    (void) edge_fn; (void) corner_fn;
    struct charm_shim_state *s = p->shim;
    const charm_forest_t *f = &s->f;
    if (vol_fn) {
        for (int64_t i = 0; i < f->n; i++) {
            p4est_iter_volume_info_t info;
            info.p4est = p;
            info.ghost_layer = g;
            info.quad = &s->q[i];
            info.quadid = tree_local(p, i);
            info.treeid = f->leaf[i].tree;
            vol_fn(&info, ud);
        }
    }
    if (!face_fn) return;
    p4est_quadrant_t *ghq = g ? (p4est_quadrant_t *) g->ghosts.array : NULL;
    charm_face_nb_t nb;
    p4est_iter_face_side_t sides[2];
    if (f->conn) {   /* unstructured connectivity: no periodic wrap, faces of any orientation */
        for (int64_t i = 0; i < f->n; i++) {
            const int32_t ti = f->leaf[i].tree;
            for (int face = 0; face < 6; face++) {
                charm_forest_face_neighbor(f, i, face, &nb);
                if (nb.kind == CHARM_NB_BOUNDARY) {
                    side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                    call_face(p, g, ud, face_fn, 1, sides, 1);
                    continue;
                }
                if (nb.kind == CHARM_NB_BIGGER) continue;   /* presented from the big side */
                if (nb.kind != CHARM_NB_SAME && nb.kind != CHARM_NB_SMALLER) {
                    fprintf(stderr, "p4est shim: forest is not 2:1 face balanced\n");
                    abort();
                }
                const int32_t tj = f->leaf[nb.idx[0]].tree;
                const int lower = (ti != tj) ? (ti < tj) : (face & 1);   /* this leaf is side 0 */
                if (nb.kind == CHARM_NB_SAME) {
                    if (!lower) continue;
                    const int64_t j = nb.idx[0];
                    side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                    side_full(&sides[1], tj, nb.nface, &s->q[j], 0, tree_local(p, j));
                    call_face(p, g, ud, face_fn, 2, sides, ti != tj);
                    continue;
                }
                p4est_quadrant_t *hq[4];
                int8_t hg[4] = {0, 0, 0, 0};
                p4est_locidx_t hid[4];
                for (int k = 0; k < 4; k++) { hq[k] = &s->q[nb.idx[k]]; hid[k] = tree_local(p, nb.idx[k]); }
                if (lower) {
                    side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                    side_hanging(&sides[1], tj, nb.nface, hq, hg, hid);
                } else {
                    side_hanging(&sides[0], tj, nb.nface, hq, hg, hid);
                    side_full(&sides[1], ti, face, &s->q[i], 0, tree_local(p, i));
                }
                call_face(p, g, ud, face_fn, 2, sides, ti != tj);
            }
        }
        return;
    }
    for (int64_t i = 0; i < f->n; i++) {
        const int32_t ti = f->leaf[i].tree;
        for (int face = 0; face < 6; face++) {
            const int d = face / 2, up = face & 1;
            charm_forest_face_neighbor(f, i, face, &nb);
            switch (nb.kind) {
            case CHARM_NB_BOUNDARY:
                side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                call_face(p, g, ud, face_fn, 1, sides, 1);
                break;
            case CHARM_NB_SAME: {
                const int64_t j = nb.idx[0];
                const int32_t tj = f->leaf[j].tree;
                if (!nb.wrap) {
                    if (!up) break;
                    side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                    side_full(&sides[1], tj, face ^ 1, &s->q[j], 0, tree_local(p, j));
                    call_face(p, g, ud, face_fn, 2, sides, ti != tj);
                } else {
                    const int64_t gk = ghost_id(p, g, j, d, nb.wrap);
                    if (up) {
                        side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                        side_full(&sides[1], tj, face ^ 1, &ghq[gk], 1, (p4est_locidx_t) gk);
                    } else {
                        side_full(&sides[0], tj, face ^ 1, &ghq[gk], 1, (p4est_locidx_t) gk);
                        side_full(&sides[1], ti, face, &s->q[i], 0, tree_local(p, i));
                    }
                    call_face(p, g, ud, face_fn, 2, sides, 1);
                }
                break;
            }
            case CHARM_NB_SMALLER: {
                p4est_quadrant_t *hq[4];
                int8_t hg[4];
                p4est_locidx_t hid[4];
                const int32_t tj = f->leaf[nb.idx[0]].tree;
                for (int k = 0; k < 4; k++) {
                    if (nb.wrap) {
                        const int64_t gk = ghost_id(p, g, nb.idx[k], d, nb.wrap);
                        hq[k] = &ghq[gk]; hg[k] = 1; hid[k] = (p4est_locidx_t) gk;
                    } else {
                        hq[k] = &s->q[nb.idx[k]]; hg[k] = 0; hid[k] = tree_local(p, nb.idx[k]);
                    }
                }
                if (up) {
                    side_full(&sides[0], ti, face, &s->q[i], 0, tree_local(p, i));
                    side_hanging(&sides[1], tj, face ^ 1, hq, hg, hid);
                } else {
                    side_hanging(&sides[0], tj, face ^ 1, hq, hg, hid);
                    side_full(&sides[1], ti, face, &s->q[i], 0, tree_local(p, i));
                }
                call_face(p, g, ud, face_fn, 2, sides, ti != tj || nb.wrap);
                break;
            }
            case CHARM_NB_BIGGER: {
                if (!nb.wrap) break;   /* presented from the big side */
                /* across a wrap: present once, from sub-face 0 of the big face */
                const int64_t big = nb.idx[0];
                charm_face_nb_t back;
                charm_forest_face_neighbor(f, big, face ^ 1, &back);
                if (back.idx[0] != i) break;
                const int64_t gk = ghost_id(p, g, big, d, nb.wrap);
                p4est_quadrant_t *hq[4];
                int8_t hg[4] = {0, 0, 0, 0};
                p4est_locidx_t hid[4];
                for (int k = 0; k < 4; k++) { hq[k] = &s->q[back.idx[k]]; hid[k] = tree_local(p, back.idx[k]); }
                const int32_t tb = f->leaf[big].tree;
                if (up) {
                    side_hanging(&sides[0], ti, face, hq, hg, hid);
                    side_full(&sides[1], tb, face ^ 1, &ghq[gk], 1, (p4est_locidx_t) gk);
                } else {
                    side_full(&sides[0], tb, face ^ 1, &ghq[gk], 1, (p4est_locidx_t) gk);
                    side_hanging(&sides[1], ti, face, hq, hg, hid);
                }
                call_face(p, g, ud, face_fn, 2, sides, 1);
                break;
            }
            default:
                fprintf(stderr, "p4est shim: forest is not 2:1 face balanced\n");
                abort();
            }
        }
    }
}
