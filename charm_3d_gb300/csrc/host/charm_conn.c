/*
 * Unstructured hexahedral connectivity: see charm_conn.h.
 *
 * The gmsh reader follows the reference's charm_conn_reader_msh
 * (src/charm_connectivity.c:315-519): hexahedra (element type 5) become
 * trees with their nodes reordered from gmsh's order (bottom and top faces
 * counter-clockwise) to p4est's corner order, quadrangles (type 3) bind
 * boundary patches to tree faces through their vertex sets, and physical
 * names come from $PhysicalNames.  Where the reference then calls
 * p4est_connectivity_complete, this file matches tree faces by their sorted
 * vertex quadruples and derives the integer coordinate map across each
 * shared face from the corner correspondence.
 */
#define _POSIX_C_SOURCE 200809L
#include "charm_conn.h"
#include "charm_forest.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

const int charm_conn_face_corners[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5},
                                           {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};

static int fail(char *err, int errlen, const char *fmt, ...)
{
    if (err && errlen > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t) errlen, fmt, ap);
        va_end(ap);
    }
    return -1;
}

void charm_conn_free(charm_conn_t *c)
{
    if (!c) return;
    free(c->vert); free(c->t2v); free(c->t2t); free(c->t2f); free(c->xperm); free(c->xsign); free(c->xoff);
    free(c->bnd_tag); free(c->reg_tag); free(c->patch);
    memset(c, 0, sizeof(*c));
}

/* ---- face matching ------------------------------------------------------------ */

typedef struct {
    int32_t key[4];   /* sorted vertex ids */
    int32_t tree;
    int8_t face;
} face_key_t;

static void sort4(int32_t a[4])
{
    for (int i = 1; i < 4; i++)
        for (int j = i; j > 0 && a[j - 1] > a[j]; j--) { int32_t t = a[j]; a[j] = a[j - 1]; a[j - 1] = t; }
}

static int key_cmp(const void *pa, const void *pb)
{
    const face_key_t *a = (const face_key_t *) pa, *b = (const face_key_t *) pb;
    for (int k = 0; k < 4; k++)
        if (a->key[k] != b->key[k]) return a->key[k] < b->key[k] ? -1 : 1;
    if (a->tree != b->tree) return a->tree < b->tree ? -1 : 1;
    return a->face - b->face;
}

static void corner_pos(int k, int32_t p[3])
{
    p[0] = (k & 1) ? CHARM_FOREST_ROOT_LEN : 0;
    p[1] = (k & 2) ? CHARM_FOREST_ROOT_LEN : 0;
    p[2] = (k & 4) ? CHARM_FOREST_ROOT_LEN : 0;
}

/* Integer map from tree t (face f) onto tree u (face g): the linear part is
 * a signed permutation fixed by where two tangential edges of the face go
 * and by the outward normal of f turning into the inward normal of g; the
 * offset puts corner 0 of the face onto its image.  Checked on all 4
 * corners. */
static int face_map(const charm_conn_t *c, int32_t t, int f, int32_t u, int g, int8_t perm[3], int8_t sign[3],
                    int32_t off[3])
{
    const int32_t R = CHARM_FOREST_ROOT_LEN;
    int32_t P[4][3], Q[4][3];
    for (int k = 0; k < 4; k++) {
        const int ck = charm_conn_face_corners[f][k];
        const int32_t gv = c->t2v[8 * t + ck];
        int found = -1;
        for (int m = 0; m < 4; m++)
            if (c->t2v[8 * u + charm_conn_face_corners[g][m]] == gv) found = charm_conn_face_corners[g][m];
        if (found < 0) return -1;
        corner_pos(ck, P[k]);
        corner_pos(found, Q[k]);
    }
    const int a0 = f / 2, a1 = (a0 == 0) ? 1 : 0, a2 = (a0 == 2) ? 1 : 2;
    int M[3][3] = {{0}};
    /* columns a1, a2: images of the tangential edges 0->1 and 0->2 */
    const int src[2] = {a1, a2}, kk[2] = {1, 2};
    for (int s = 0; s < 2; s++) {
        int nz = 0;
        for (int i = 0; i < 3; i++) {
            const int32_t dlt = Q[kk[s]][i] - Q[0][i];
            if (dlt != 0 && dlt != R && dlt != -R) return -1;
            M[i][src[s]] = dlt / R;
            nz += dlt != 0;
        }
        if (nz != 1) return -1;
    }
    /* column a0: outward normal of f -> inward normal of g */
    M[g / 2][a0] = ((f & 1) ? 1 : -1) * ((g & 1) ? -1 : 1);
    for (int i = 0; i < 3; i++) {
        int nz = 0;
        for (int j = 0; j < 3; j++)
            if (M[i][j]) { perm[i] = (int8_t) j; sign[i] = (int8_t) M[i][j]; nz++; }
        if (nz != 1) return -1;
    }
    for (int i = 0; i < 3; i++) off[i] = Q[0][i] - sign[i] * P[0][perm[i]];
    for (int k = 0; k < 4; k++)
        for (int i = 0; i < 3; i++)
            if (sign[i] * P[k][perm[i]] + off[i] != Q[k][i]) return -1;
    return 0;
}

int charm_conn_build(charm_conn_t *c, int32_t n_vert, const double *vert, int32_t n_tree, const int32_t *t2v,
                     char *err, int errlen)
{
    memset(c, 0, sizeof(*c));
    if (n_vert <= 0 || n_tree <= 0 || !vert || !t2v) return fail(err, errlen, "empty connectivity");
    c->n_vert = n_vert;
    c->n_tree = n_tree;
    const size_t T = (size_t) n_tree;
    c->vert = (double *) malloc(sizeof(double) * 3 * (size_t) n_vert);
    c->t2v = (int32_t *) malloc(sizeof(int32_t) * 8 * T);
    c->t2t = (int32_t *) malloc(sizeof(int32_t) * 6 * T);
    c->t2f = (int8_t *) malloc(6 * T);
    c->xperm = (int8_t *) malloc(18 * T);
    c->xsign = (int8_t *) malloc(18 * T);
    c->xoff = (int32_t *) malloc(sizeof(int32_t) * 18 * T);
    c->bnd_tag = (int32_t *) malloc(sizeof(int32_t) * 6 * T);
    c->reg_tag = (int32_t *) malloc(sizeof(int32_t) * T);
    face_key_t *keys = (face_key_t *) malloc(sizeof(face_key_t) * 6 * T);
    if (!c->vert || !c->t2v || !c->t2t || !c->t2f || !c->xperm || !c->xsign || !c->xoff || !c->bnd_tag ||
        !c->reg_tag || !keys) {
        free(keys);
        charm_conn_free(c);
        return fail(err, errlen, "out of memory");
    }
    memcpy(c->vert, vert, sizeof(double) * 3 * (size_t) n_vert);
    memcpy(c->t2v, t2v, sizeof(int32_t) * 8 * T);
    for (size_t k = 0; k < 6 * T; k++) { c->t2t[k] = -1; c->t2f[k] = -1; c->bnd_tag[k] = -1; }
    for (size_t k = 0; k < 18 * T; k++) { c->xperm[k] = 0; c->xsign[k] = 0; c->xoff[k] = 0; }
    for (size_t t = 0; t < T; t++) c->reg_tag[t] = -1;
    for (int32_t t = 0; t < n_tree; t++) {
        for (int a = 0; a < 8; a++) {
            const int32_t v = t2v[8 * t + a];
            if (v < 0 || v >= n_vert) { free(keys); charm_conn_free(c); return fail(err, errlen, "tree %d: vertex out of range", t); }
            for (int b = 0; b < a; b++)
                if (t2v[8 * t + b] == v) { free(keys); charm_conn_free(c); return fail(err, errlen, "tree %d: repeated vertex", t); }
        }
        for (int f = 0; f < 6; f++) {
            face_key_t *k = &keys[6 * t + f];
            for (int m = 0; m < 4; m++) k->key[m] = t2v[8 * t + charm_conn_face_corners[f][m]];
            sort4(k->key);
            k->tree = t;
            k->face = (int8_t) f;
        }
    }
    qsort(keys, 6 * T, sizeof(face_key_t), key_cmp);
    int bad = 0;
    for (size_t i = 0; i < 6 * T && !bad;) {
        size_t j = i + 1;
        while (j < 6 * T && !memcmp(keys[j].key, keys[i].key, sizeof(keys[i].key))) j++;
        if (j - i > 2) {
            bad = fail(err, errlen, "face of tree %d shared by %d trees", keys[i].tree, (int) (j - i));
        } else if (j - i == 2) {
            const face_key_t *A = &keys[i], *B = &keys[i + 1];
            if (A->tree == B->tree) bad = fail(err, errlen, "tree %d is its own face neighbour", A->tree);
            for (int s = 0; s < 2 && !bad; s++) {
                const face_key_t *X = s ? B : A, *Y = s ? A : B;
                const size_t o = 6 * (size_t) X->tree + (size_t) X->face;
                c->t2t[o] = Y->tree;
                c->t2f[o] = Y->face;
                if (face_map(c, X->tree, X->face, Y->tree, Y->face, &c->xperm[3 * o], &c->xsign[3 * o], &c->xoff[3 * o]))
                    bad = fail(err, errlen, "trees %d and %d: shared face is not a square symmetry", X->tree, Y->tree);
            }
        }
        i = j;
    }
    free(keys);
    if (bad) charm_conn_free(c);
    return bad;
}

/* ---- geometry ------------------------------------------------------------------- */

void charm_conn_point(const charm_conn_t *c, int32_t t, double x, double y, double z, double out[3])
{   /* trilinear in the p4est corner order (p4est_qcoord_to_vertex) */
    const int32_t *tv = &c->t2v[8 * t];
    const double w[2][3] = {{1.0 - x, 1.0 - y, 1.0 - z}, {x, y, z}};
    for (int d = 0; d < 3; d++) {
        double s = 0.0;
        for (int k = 0; k < 8; k++)
            s += w[(k >> 2) & 1][2] * (w[(k >> 1) & 1][1] * (w[k & 1][0] * c->vert[3 * tv[k] + d]));
        out[d] = s;
    }
}

int32_t charm_conn_map_box(const charm_conn_t *c, int32_t t, int f, const int32_t p[3], int32_t len, int32_t q[3])
{
    const size_t o = 6 * (size_t) t + (size_t) f;
    const int32_t u = c->t2t[o];
    if (u < 0) return -1;
    const int8_t *perm = &c->xperm[3 * o], *sign = &c->xsign[3 * o];
    const int32_t *off = &c->xoff[3 * o];
    for (int i = 0; i < 3; i++)
        q[i] = (sign[i] > 0) ? p[perm[i]] + off[i] : off[i] - p[perm[i]] - len;
    return u;
}

const char *charm_conn_patch_name(const charm_conn_t *c, int dim, int32_t tag)
{
    for (int32_t i = 0; i < c->n_patch; i++)
        if (c->patch[i].tag == tag && c->patch[i].dim == dim) return c->patch[i].name;
    return NULL;
}

/* ---- gmsh 2.x ASCII --------------------------------------------------------------- */

typedef struct { char *buf; size_t cap; } line_t;

static int read_line(FILE *fp, line_t *l)
{
    ssize_t n = getline(&l->buf, &l->cap, fp);
    if (n < 0) return -1;
    while (n > 0 && (l->buf[n - 1] == '\n' || l->buf[n - 1] == '\r')) l->buf[--n] = 0;
    return 0;
}

static int cmp_i64(const void *a, const void *b)
{
    const int64_t x = ((const int64_t *) a)[0], y = ((const int64_t *) b)[0];
    return (x > y) - (x < y);
}

/* index of node id `id` in the sorted (id, index) table, or -1 */
static int32_t node_index(const int64_t *tab, int64_t n, int64_t id)
{
    int64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (tab[2 * mid] == id) return (int32_t) tab[2 * mid + 1];
        if (tab[2 * mid] < id) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

typedef struct { int32_t key[4]; int32_t tag; } bquad_t;

static int bquad_cmp(const void *pa, const void *pb)
{
    const bquad_t *a = (const bquad_t *) pa, *b = (const bquad_t *) pb;
    for (int k = 0; k < 4; k++)
        if (a->key[k] != b->key[k]) return a->key[k] < b->key[k] ? -1 : 1;
    return 0;
}

int charm_conn_read_gmsh(charm_conn_t *c, const char *path, char *err, int errlen)
{
    memset(c, 0, sizeof(*c));
    FILE *fp = fopen(path, "r");
    if (!fp) return fail(err, errlen, "cannot open %s", path);
    line_t l = {NULL, 0};
    int rc = -1;
    int64_t nn = 0, nh = 0, nq = 0;
    double *vert = NULL;
    int64_t *ids = NULL;             /* (node id, index) pairs, sorted by id */
    int32_t *t2v = NULL, *treg = NULL;
    bquad_t *bq = NULL;
    charm_conn_patch_t *patch = NULL;
    int32_t n_patch = 0;
    int have_nodes = 0, have_elems = 0;
    while (read_line(fp, &l) == 0) {
        if (!strcmp(l.buf, "$MeshFormat")) {
            if (read_line(fp, &l)) { fail(err, errlen, "%s: truncated $MeshFormat", path); goto done; }
            double ver = 0; int ft = -1;
            if (sscanf(l.buf, "%lf %d", &ver, &ft) != 2 || ver < 2.0 || ver >= 3.0 || ft != 0) {
                fail(err, errlen, "%s: only gmsh 2.x ASCII meshes are read (got '%s')", path, l.buf);
                goto done;
            }
        } else if (!strcmp(l.buf, "$PhysicalNames")) {
            if (read_line(fp, &l) || sscanf(l.buf, "%d", &n_patch) != 1 || n_patch < 0) {
                fail(err, errlen, "%s: bad $PhysicalNames", path);
                goto done;
            }
            patch = (charm_conn_patch_t *) calloc((size_t) (n_patch > 0 ? n_patch : 1), sizeof(*patch));
            if (!patch) { fail(err, errlen, "out of memory"); goto done; }
            for (int32_t i = 0; i < n_patch; i++) {
                if (read_line(fp, &l)) { fail(err, errlen, "%s: truncated $PhysicalNames", path); goto done; }
                char *q0 = strchr(l.buf, '"'), *q1 = q0 ? strchr(q0 + 1, '"') : NULL;
                if (sscanf(l.buf, "%d %d", &patch[i].dim, &patch[i].tag) != 2 || !q0 || !q1 ||
                    q1 - q0 - 1 >= CHARM_CONN_NAME) {
                    fail(err, errlen, "%s: bad physical name line '%s'", path, l.buf);
                    goto done;
                }
                memcpy(patch[i].name, q0 + 1, (size_t) (q1 - q0 - 1));
                patch[i].name[q1 - q0 - 1] = 0;
            }
        } else if (!strcmp(l.buf, "$Nodes")) {
            long long n = 0;
            if (read_line(fp, &l) || sscanf(l.buf, "%lld", &n) != 1 || n <= 0 || n >= INT32_MAX) {
                fail(err, errlen, "%s: bad $Nodes", path);
                goto done;
            }
            nn = n;
            vert = (double *) malloc(sizeof(double) * 3 * (size_t) nn);
            ids = (int64_t *) malloc(sizeof(int64_t) * 2 * (size_t) nn);
            if (!vert || !ids) { fail(err, errlen, "out of memory"); goto done; }
            for (int64_t i = 0; i < nn; i++) {
                long long id;
                if (read_line(fp, &l) ||
                    sscanf(l.buf, "%lld %lf %lf %lf", &id, &vert[3 * i], &vert[3 * i + 1], &vert[3 * i + 2]) != 4) {
                    fail(err, errlen, "%s: premature end of $Nodes", path);
                    goto done;
                }
                ids[2 * i] = id;
                ids[2 * i + 1] = i;
            }
            qsort(ids, (size_t) nn, 2 * sizeof(int64_t), cmp_i64);
            for (int64_t i = 1; i < nn; i++)
                if (ids[2 * i] == ids[2 * i - 2]) { fail(err, errlen, "%s: node %lld twice", path, (long long) ids[2 * i]); goto done; }
            have_nodes = 1;
        } else if (!strcmp(l.buf, "$Elements")) {
            long long n = 0;
            if (!have_nodes) { fail(err, errlen, "%s: $Elements before $Nodes", path); goto done; }
            if (read_line(fp, &l) || sscanf(l.buf, "%lld", &n) != 1 || n < 0 || n >= INT32_MAX) {
                fail(err, errlen, "%s: bad $Elements", path);
                goto done;
            }
            t2v = (int32_t *) malloc(sizeof(int32_t) * 8 * (size_t) (n > 0 ? n : 1));
            treg = (int32_t *) malloc(sizeof(int32_t) * (size_t) (n > 0 ? n : 1));
            bq = (bquad_t *) malloc(sizeof(bquad_t) * (size_t) (n > 0 ? n : 1));
            if (!t2v || !treg || !bq) { fail(err, errlen, "out of memory"); goto done; }
            for (long long i = 0; i < n; i++) {
                if (read_line(fp, &l)) { fail(err, errlen, "%s: premature end of $Elements", path); goto done; }
                /* id type ntags tag... nodes... */
                long long f[64];
                int nf = 0, pos = 0, used;
                while (nf < 64 && sscanf(l.buf + pos, "%lld%n", &f[nf], &used) == 1) { nf++; pos += used; }
                if (nf < 3 || f[2] < 0 || 3 + f[2] > nf) { fail(err, errlen, "%s: bad element line '%s'", path, l.buf); goto done; }
                const long long type = f[1], ntag = f[2];
                const int32_t phys = ntag > 0 ? (int32_t) f[3] : -1;
                const long long *nodes = &f[3 + ntag];
                const int nnodes = nf - 3 - (int) ntag;
                if (type == 5) {
                    /* gmsh hexahedron: 0-3 bottom, 4-7 top, counter-clockwise;
                     * p4est corner order swaps 2<->3 and 6<->7 */
                    static const int to_p4est[8] = {0, 1, 3, 2, 4, 5, 7, 6};
                    if (nnodes != 8) { fail(err, errlen, "%s: hexahedron without 8 nodes", path); goto done; }
                    for (int k = 0; k < 8; k++) {
                        const int32_t v = node_index(ids, nn, nodes[k]);
                        if (v < 0) { fail(err, errlen, "%s: unknown node %lld", path, nodes[k]); goto done; }
                        t2v[8 * nh + to_p4est[k]] = v;
                    }
                    treg[nh] = phys;
                    nh++;
                } else if (type == 3) {
                    if (nnodes != 4) { fail(err, errlen, "%s: quadrangle without 4 nodes", path); goto done; }
                    for (int k = 0; k < 4; k++) {
                        const int32_t v = node_index(ids, nn, nodes[k]);
                        if (v < 0) { fail(err, errlen, "%s: unknown node %lld", path, nodes[k]); goto done; }
                        bq[nq].key[k] = v;
                    }
                    sort4(bq[nq].key);
                    bq[nq].tag = phys;
                    nq++;
                }
            }
            have_elems = 1;
        }
    }
    if (!have_nodes || !have_elems || nh == 0) { fail(err, errlen, "%s: no hexahedra", path); goto done; }
    if (charm_conn_build(c, (int32_t) nn, vert, (int32_t) nh, t2v, err, errlen)) goto done;
    memcpy(c->reg_tag, treg, sizeof(int32_t) * (size_t) nh);
    /* boundary patches: a quadrangle names the tree face with its vertex set */
    qsort(bq, (size_t) nq, sizeof(bquad_t), bquad_cmp);
    for (int32_t t = 0; t < c->n_tree; t++)
        for (int f = 0; f < 6; f++) {
            bquad_t k;
            for (int m = 0; m < 4; m++) k.key[m] = c->t2v[8 * t + charm_conn_face_corners[f][m]];
            sort4(k.key);
            const bquad_t *hit = (const bquad_t *) bsearch(&k, bq, (size_t) nq, sizeof(bquad_t), bquad_cmp);
            if (hit) c->bnd_tag[6 * t + f] = hit->tag;
        }
    c->n_patch = n_patch;
    c->patch = patch;
    patch = NULL;
    rc = 0;
done:
    free(l.buf);
    fclose(fp);
    free(vert); free(ids); free(t2v); free(treg); free(bq); free(patch);
    if (rc) charm_conn_free(c);
    return rc;
}
