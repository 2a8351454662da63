/*
 * Host octree forest: see charm_forest.h.
 *
 * The operations mirror what CHARM_3D asks of p4est on its hot path:
 *   - p4est_new_ext at a uniform level (src/charm_3d.c:36),
 *   - face iteration with full / hanging sides (p4est_iterate, used by every
 *     face callback, e.g. src/models/ns/charm_model_ns_conv.c:174-331),
 *   - p4est_refine_ext / p4est_coarsen_ext (non-recursive) and
 *     p4est_balance_ext(CHARM_CONNECT_FACE) with a replace callback
 *     (src/charm_amr.c:601-608).
 */
#define _POSIX_C_SOURCE 200809L
#include "charm_forest.h"
#include "charm_conn.h"

#include <pthread.h>
#include <stdint.h>
#include <sys/types.h>
#include <unistd.h>
#include <stdlib.h>
#include <string.h>

/* ---- Morton keys ------------------------------------------------------- */

static uint64_t spread3(uint32_t v)
{
    /* spread the low 21 bits of v so that bit i moves to bit 3i */
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8))  & 0x100f00f00f00f00full;
    x = (x | (x << 4))  & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2))  & 0x1249249249249249ull;
    return x;
}

static uint64_t morton(int32_t x, int32_t y, int32_t z)
{
    /* x is the least significant coordinate, as in p4est */
    return spread3((uint32_t) x) | (spread3((uint32_t) y) << 1) | (spread3((uint32_t) z) << 2);
}

static int leaf_cmp(const charm_leaf_t *a, const charm_leaf_t *b)
{
    if (a->tree != b->tree) return a->tree < b->tree ? -1 : 1;
    uint64_t ka = morton(a->x, a->y, a->z), kb = morton(b->x, b->y, b->z);
    if (ka != kb) return ka < kb ? -1 : 1;
    if (a->level != b->level) return a->level < b->level ? -1 : 1;
    return 0;
}

int charm_leaf_child_id(const charm_leaf_t *q)
{
    if (q->level == 0) return 0;
    int32_t len = CHARM_FOREST_QLEN(q->level);
    return ((q->x & len) ? 1 : 0) | ((q->y & len) ? 2 : 0) | ((q->z & len) ? 4 : 0);
}

/* ---- storage ------------------------------------------------------------ */

static int reserve(charm_forest_t *f, int64_t n)
{
    if (n <= f->cap) return 0;
    int64_t cap = f->cap ? f->cap : 64;
    while (cap < n) cap *= 2;
    charm_leaf_t *p = (charm_leaf_t *) realloc(f->leaf, (size_t) cap * sizeof(charm_leaf_t));
    if (!p) return -1;
    f->leaf = p;
    f->cap = cap;
    return 0;
}

int charm_forest_init_uniform(charm_forest_t *f, const int32_t ntree[3], const int32_t periodic[3],
                              const double origin[3], const double tree_len[3], int level)
{
    memset(f, 0, sizeof(*f));
    if (level < 0 || level > CHARM_FOREST_MAXLEVEL - 1) return -1;
    for (int d = 0; d < 3; d++) {
        if (ntree[d] < 1) return -1;
        f->ntree[d] = ntree[d];
        f->periodic[d] = periodic ? (periodic[d] != 0) : 0;
        f->origin[d] = origin ? origin[d] : 0.0;
        f->tree_len[d] = tree_len ? tree_len[d] : 1.0;
    }
    int64_t nt = (int64_t) ntree[0] * ntree[1] * ntree[2];
    int64_t per = (int64_t) 1 << (3 * level);
    if (reserve(f, nt * per)) return -1;
    int32_t len = CHARM_FOREST_QLEN(level);
    int64_t k = 0;
    for (int32_t t = 0; t < nt; t++) {
        for (int64_t m = 0; m < per; m++) {
            /* de-interleave m into (i,j,l) at `level` bits each */
            int32_t i = 0, j = 0, l = 0;
            for (int b = 0; b < level; b++) {
                i |= (int32_t) ((m >> (3 * b)) & 1) << b;
                j |= (int32_t) ((m >> (3 * b + 1)) & 1) << b;
                l |= (int32_t) ((m >> (3 * b + 2)) & 1) << b;
            }
            charm_leaf_t *q = &f->leaf[k++];
            q->x = i * len; q->y = j * len; q->z = l * len;
            q->tree = t; q->level = (int8_t) level;
        }
    }
    f->n = k;
    return 0;
}

void charm_forest_free(charm_forest_t *f)
{
    free(f->leaf);
    memset(f, 0, sizeof(*f));
}

int charm_forest_init_conn(charm_forest_t *f, const charm_conn_t *conn, int level)
{
    if (!conn || conn->n_tree < 1) return -1;
    const int32_t ntree[3] = {conn->n_tree, 1, 1};
    const double one[3] = {1.0, 1.0, 1.0};
    if (charm_forest_init_uniform(f, ntree, NULL, NULL, one, level)) return -1;
    f->conn = conn;
    return 0;
}

int charm_forest_copy(charm_forest_t *dst, const charm_forest_t *src)
{
    *dst = *src;
    dst->leaf = NULL;
    dst->cap = 0;
    if (reserve(dst, src->n > 0 ? src->n : 1)) return -1;
    memcpy(dst->leaf, src->leaf, (size_t) src->n * sizeof(charm_leaf_t));
    return 0;
}

/* ---- parallel loops over leaves ------------------------------------------ */

/* A pool of worker threads, started on the first parallel loop of the
 * process (and again in a forked child, which has none of them) and kept:
 * an adapt and a flatten run a dozen loops each, and starting threads for
 * every loop costs more than the short loops themselves. */
enum { kMaxThreads = 64 };

typedef struct {
    pthread_mutex_t mu;
    pthread_cond_t go, done;
    int nworkers;                /* threads started (chunks 1..nworkers) */
    uint64_t gen;                /* loop generation: bumped per loop */
    int pending;                 /* chunks of the current loop not finished */
    charm_forest_range_fn fn;
    void *ctx;
    int64_t n;
    int nt;                      /* chunks of the current loop */
    pid_t pid;                   /* process that started the workers */
} pool_t;

static pool_t g_pool;
/* one loop at a time uses the pool; a loop that finds it busy (a loop in
 * another thread, or one nested in a chunk) runs serially */
static pthread_mutex_t g_dispatch = PTHREAD_MUTEX_INITIALIZER;

static void *pool_worker(void *arg)
{
    const int k = (int) (intptr_t) arg;
    pool_t *p = &g_pool;
    uint64_t seen = 0;           /* workers start before the first loop */
    pthread_mutex_lock(&p->mu);
    for (;;) {
        while (p->gen == seen) pthread_cond_wait(&p->go, &p->mu);
        seen = p->gen;
        if (k < p->nt) {
            const charm_forest_range_fn fn = p->fn;
            void *ctx = p->ctx;
            const int64_t lo = p->n * k / p->nt, hi = p->n * (k + 1) / p->nt;
            pthread_mutex_unlock(&p->mu);
            fn(ctx, lo, hi);
            pthread_mutex_lock(&p->mu);
            if (--p->pending == 0) pthread_cond_signal(&p->done);
        }
    }
    return NULL;
}

/* With g_dispatch held: start the workers (one per online CPU but the
 * caller's) if this process has none. */
static void pool_start(void)
{
    pool_t *p = &g_pool;
    if (p->pid == getpid()) return;
    const long cpus = sysconf(_SC_NPROCESSORS_ONLN);
    const int want = (cpus > 1) ? (int) (cpus < kMaxThreads ? cpus : kMaxThreads) : 1;
    pthread_mutex_init(&p->mu, NULL);
    pthread_cond_init(&p->go, NULL);
    pthread_cond_init(&p->done, NULL);
    p->gen = 0;
    p->pending = 0;
    p->nworkers = 0;
    p->pid = getpid();
    pthread_attr_t at;
    pthread_attr_init(&at);
    pthread_attr_setdetachstate(&at, PTHREAD_CREATE_DETACHED);
    for (int k = 1; k < want; k++) {
        pthread_t t;
        if (pthread_create(&t, &at, pool_worker, (void *) (intptr_t) k) != 0) break;
        p->nworkers = k;
    }
    pthread_attr_destroy(&at);
}

/* Run fn(ctx, lo, hi) over [0, n) in contiguous chunks of at least
 * min_chunk iterations on up to the online CPU count of threads (the calling
 * thread takes the first chunk).  A loop with one chunk, or one that finds
 * the pool busy, runs serially on the calling thread. */
void charm_forest_parallel_for_min(int64_t n, int64_t min_chunk, charm_forest_range_fn fn, void *ctx)
{
    if (min_chunk < 1) min_chunk = 1;
    const int64_t most = n / min_chunk;   /* chunks worth a thread */
    if (most <= 1 || pthread_mutex_trylock(&g_dispatch) != 0) {
        fn(ctx, 0, n);
        return;
    }
    pool_t *p = &g_pool;
    pool_start();
    int nt = p->nworkers + 1;
    if ((int64_t) nt > most) nt = (int) most;
    if (nt <= 1) {
        pthread_mutex_unlock(&g_dispatch);
        fn(ctx, 0, n);
        return;
    }
    pthread_mutex_lock(&p->mu);
    p->fn = fn;
    p->ctx = ctx;
    p->n = n;
    p->nt = nt;
    p->pending = nt - 1;
    p->gen++;
    pthread_cond_broadcast(&p->go);
    pthread_mutex_unlock(&p->mu);
    fn(ctx, 0, n / nt);
    pthread_mutex_lock(&p->mu);
    while (p->pending > 0) pthread_cond_wait(&p->done, &p->mu);
    pthread_mutex_unlock(&p->mu);
    pthread_mutex_unlock(&g_dispatch);
}

/* Light loops: serial below 16384 iterations, chunks of 4096 or more. */
void charm_forest_parallel_for(int64_t n, charm_forest_range_fn fn, void *ctx)
{
    if (n < 16384) {
        fn(ctx, 0, n);
        return;
    }
    charm_forest_parallel_for_min(n, 4096, fn, ctx);
}

/* ---- queries ------------------------------------------------------------ */

typedef struct { const charm_forest_t *f; uint64_t *key; } keys_ctx_t;

static void keys_range(void *c, int64_t lo, int64_t hi)
{
    const keys_ctx_t *k = (const keys_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) k->key[i] = morton(k->f->leaf[i].x, k->f->leaf[i].y, k->f->leaf[i].z);
}

void charm_forest_keys(const charm_forest_t *f, uint64_t *key)
{
    keys_ctx_t c = {f, key};
    charm_forest_parallel_for(f->n, keys_range, &c);
}

int64_t charm_forest_find_k(const charm_forest_t *f, const uint64_t *keys, int32_t t, int32_t x, int32_t y,
                            int32_t z)
{
    if (x < 0 || y < 0 || z < 0 || x >= CHARM_FOREST_ROOT_LEN || y >= CHARM_FOREST_ROOT_LEN ||
        z >= CHARM_FOREST_ROOT_LEN)
        return -1;
    uint64_t key = morton(x, y, z);
    int64_t lo = 0, hi = f->n - 1, best = -1;
    while (lo <= hi) {       /* last leaf with (tree,key) <= (t,key) */
        int64_t mid = lo + (hi - lo) / 2;
        const charm_leaf_t *q = &f->leaf[mid];
        const uint64_t kq = keys ? keys[mid] : morton(q->x, q->y, q->z);
        int le = (q->tree < t) || (q->tree == t && kq <= key);
        if (le) { best = mid; lo = mid + 1; } else hi = mid - 1;
    }
    if (best < 0) return -1;
    const charm_leaf_t *q = &f->leaf[best];
    if (q->tree != t) return -1;
    int32_t len = CHARM_FOREST_QLEN(q->level);
    if (x < q->x || x >= q->x + len || y < q->y || y >= q->y + len || z < q->z || z >= q->z + len) return -1;
    return best;
}

int64_t charm_forest_find(const charm_forest_t *f, int32_t t, int32_t x, int32_t y, int32_t z)
{
    return charm_forest_find_k(f, NULL, t, x, y, z);
}

/* Map tree-local point p (possibly one root length outside along axis d) to
 * the tree that holds it.  Returns the tree id or -1 at a non-periodic
 * boundary; *wrap receives -1/+1 when a periodic wrap was taken. */
static int32_t locate_tree(const charm_forest_t *f, int32_t t, int d, int32_t p[3], int *wrap)
{
    int32_t ti[3];
    ti[0] = t % f->ntree[0];
    ti[1] = (t / f->ntree[0]) % f->ntree[1];
    ti[2] = t / (f->ntree[0] * f->ntree[1]);
    *wrap = 0;
    if (p[d] < 0) {
        p[d] += CHARM_FOREST_ROOT_LEN;
        ti[d] -= 1;
        if (ti[d] < 0) {
            if (!f->periodic[d]) return -1;
            ti[d] += f->ntree[d];
            *wrap = -1;
        }
    } else if (p[d] >= CHARM_FOREST_ROOT_LEN) {
        p[d] -= CHARM_FOREST_ROOT_LEN;
        ti[d] += 1;
        if (ti[d] >= f->ntree[d]) {
            if (!f->periodic[d]) return -1;
            ti[d] -= f->ntree[d];
            *wrap = +1;
        }
    }
    return ti[0] + f->ntree[0] * (ti[1] + f->ntree[1] * ti[2]);
}

void charm_forest_face_neighbor(const charm_forest_t *f, int64_t i, int face, charm_face_nb_t *nb)
{
    charm_forest_face_neighbor_k(f, NULL, i, face, nb);
}

/* Face neighbours across a tree face of an unstructured connectivity: the
 * exterior boxes (the same-size neighbour, or the four half-size boxes on
 * the face) are mapped into the neighbour tree and located there. */
static void face_neighbor_conn(const charm_forest_t *f, const uint64_t *keys, int64_t i, int face,
                               charm_face_nb_t *nb)
{
    const charm_leaf_t *q = &f->leaf[i];
    const int d = face / 2, up = face & 1;
    const int32_t len = CHARM_FOREST_QLEN(q->level);
    int32_t p[3] = {q->x, q->y, q->z};
    p[d] += up ? len : -len;
    nb->wrap = 0;
    nb->idx[0] = nb->idx[1] = nb->idx[2] = nb->idx[3] = -1;
    int32_t t = q->tree, r[3];
    if (p[d] >= 0 && p[d] < CHARM_FOREST_ROOT_LEN) {
        nb->nface = face ^ 1;
        r[0] = p[0]; r[1] = p[1]; r[2] = p[2];
    } else {
        const int32_t u = charm_conn_map_box(f->conn, t, face, p, len, r);
        if (u < 0) { nb->kind = CHARM_NB_BOUNDARY; nb->nface = -1; return; }
        nb->nface = f->conn->t2f[6 * (size_t) t + (size_t) face];
        t = u;
    }
    const int64_t j = charm_forest_find_k(f, keys, t, r[0], r[1], r[2]);
    const charm_leaf_t *n = &f->leaf[j];
    if (n->level == q->level) { nb->kind = CHARM_NB_SAME; nb->idx[0] = j; return; }
    if (n->level < q->level) {
        nb->kind = (n->level == q->level - 1) ? CHARM_NB_BIGGER : CHARM_NB_UNBALANCED;
        nb->idx[0] = j;
        return;
    }
    /* the four half-size boxes on our face, in our tangential order */
    const int s = (d == 0) ? 1 : 0, tt = (d == 2) ? 1 : 2;
    const int32_t h = len / 2;
    nb->kind = CHARM_NB_SMALLER;
    for (int k = 0; k < 4; k++) {
        int32_t c[3] = {p[0], p[1], p[2]}, m[3];
        if (!up) c[d] += h;
        c[s] += (k & 1) ? h : 0;
        c[tt] += (k & 2) ? h : 0;
        int32_t tk = q->tree;
        if (c[d] >= 0 && c[d] < CHARM_FOREST_ROOT_LEN) { m[0] = c[0]; m[1] = c[1]; m[2] = c[2]; }
        else tk = charm_conn_map_box(f->conn, q->tree, face, c, h, m);
        const int64_t mk = charm_forest_find_k(f, keys, tk, m[0], m[1], m[2]);
        nb->idx[k] = mk;
        if (f->leaf[mk].level != q->level + 1) nb->kind = CHARM_NB_UNBALANCED;
    }
}

void charm_forest_face_neighbor_k(const charm_forest_t *f, const uint64_t *keys, int64_t i, int face,
                                  charm_face_nb_t *nb)
{
    if (f->conn) { face_neighbor_conn(f, keys, i, face, nb); return; }
    nb->nface = face ^ 1;
    const charm_leaf_t *q = &f->leaf[i];
    int d = face / 2, up = face & 1;
    int32_t len = CHARM_FOREST_QLEN(q->level);
    int32_t p[3] = {q->x, q->y, q->z};
    p[d] += up ? len : -len;          /* lower corner of the same-size neighbour */
    int wrap;
    int32_t nt = locate_tree(f, q->tree, d, p, &wrap);
    nb->wrap = wrap;
    nb->idx[0] = nb->idx[1] = nb->idx[2] = nb->idx[3] = -1;
    if (nt < 0) { nb->kind = CHARM_NB_BOUNDARY; return; }
    int64_t j = charm_forest_find_k(f, keys, nt, p[0], p[1], p[2]);
    const charm_leaf_t *r = &f->leaf[j];
    if (r->level == q->level) { nb->kind = CHARM_NB_SAME; nb->idx[0] = j; return; }
    if (r->level < q->level) {
        nb->kind = (r->level == q->level - 1) ? CHARM_NB_BIGGER : CHARM_NB_UNBALANCED;
        nb->idx[0] = j;
        return;
    }
    /* neighbour region is subdivided: the four children adjacent to our face */
    int s = (d == 0) ? 1 : 0, tt = (d == 2) ? 1 : 2;
    int32_t h = len / 2;
    nb->kind = CHARM_NB_SMALLER;
    for (int k = 0; k < 4; k++) {
        int32_t c[3] = {p[0], p[1], p[2]};
        if (!up) c[d] += h;          /* the half of the region touching our face */
        c[s] += (k & 1) ? h : 0;
        c[tt] += (k & 2) ? h : 0;
        int64_t m = charm_forest_find_k(f, keys, nt, c[0], c[1], c[2]);
        nb->idx[k] = m;
        if (f->leaf[m].level != q->level + 1) nb->kind = CHARM_NB_UNBALANCED;
    }
}

void charm_forest_leaf_geom(const charm_forest_t *f, int64_t i, double c[3], double h[3])
{
    const charm_leaf_t *q = &f->leaf[i];
    int32_t ti[3];
    ti[0] = q->tree % f->ntree[0];
    ti[1] = (q->tree / f->ntree[0]) % f->ntree[1];
    ti[2] = q->tree / (f->ntree[0] * f->ntree[1]);
    int32_t qc[3] = {q->x, q->y, q->z};
    double inv = 1.0 / (double) CHARM_FOREST_ROOT_LEN;
    int32_t len = CHARM_FOREST_QLEN(q->level);
    for (int d = 0; d < 3; d++) {
        h[d] = f->tree_len[d] * ((double) len * inv);
        c[d] = f->origin[d] + f->tree_len[d] * ((double) ti[d] + ((double) qc[d] + 0.5 * (double) len) * inv);
    }
}

/* ---- refine / coarsen / balance ---------------------------------------- */

static void child_of(const charm_leaf_t *p, int c, charm_leaf_t *out)
{
    int32_t h = CHARM_FOREST_QLEN(p->level + 1);
    out->x = p->x + ((c & 1) ? h : 0);
    out->y = p->y + ((c & 2) ? h : 0);
    out->z = p->z + ((c & 4) ? h : 0);
    out->tree = p->tree;
    out->level = (int8_t) (p->level + 1);
}

/* refine in blocks of leaves: per block the refined count, then (after a
 * prefix sum) each block writes its leaves from its own output offset */
enum { kRefineBlk = 4096 };

typedef struct {
    const charm_forest_t *f;
    const int8_t *flag;
    int maxlevel;
    int64_t *off;        /* per block: refined leaves, then the first output index */
    charm_leaf_t *nl;
    int64_t *map;        /* old leaf -> first new index */
} refine_ctx_t;

static void refine_count_range(void *c, int64_t lo, int64_t hi)
{
    const refine_ctx_t *x = (const refine_ctx_t *) c;
    for (int64_t b = lo; b < hi; b++) {
        const int64_t i0 = b * kRefineBlk, i1 = (i0 + kRefineBlk < x->f->n) ? i0 + kRefineBlk : x->f->n;
        int64_t r = 0;
        for (int64_t i = i0; i < i1; i++) r += (x->flag[i] && x->f->leaf[i].level < x->maxlevel);
        x->off[b] = r;
    }
}

static void refine_emit_range(void *c, int64_t lo, int64_t hi)
{
    const refine_ctx_t *x = (const refine_ctx_t *) c;
    for (int64_t b = lo; b < hi; b++) {
        const int64_t i0 = b * kRefineBlk, i1 = (i0 + kRefineBlk < x->f->n) ? i0 + kRefineBlk : x->f->n;
        int64_t k = x->off[b];
        for (int64_t i = i0; i < i1; i++) {
            x->map[i] = k;
            if (x->flag[i] && x->f->leaf[i].level < x->maxlevel) {
                for (int ch = 0; ch < 8; ch++) child_of(&x->f->leaf[i], ch, &x->nl[k++]);
            } else {
                x->nl[k++] = x->f->leaf[i];
            }
        }
    }
}

int64_t charm_forest_refine_map(charm_forest_t *f, const int8_t *flag, int maxlevel,
                                charm_forest_replace_fn replace, void *user, int64_t *old_to_new)
{
    if (maxlevel < 0 || maxlevel > CHARM_FOREST_MAXLEVEL - 1) maxlevel = CHARM_FOREST_MAXLEVEL - 1;
    const int64_t nblk = (f->n + kRefineBlk - 1) / kRefineBlk;
    int64_t *off = (int64_t *) malloc(sizeof(int64_t) * (size_t) (nblk + 1));
    if (!off) return -1;
    refine_ctx_t x = {f, flag, maxlevel, off, NULL, NULL};
    charm_forest_parallel_for_min(nblk, 2, refine_count_range, &x);
    int64_t nref = 0;
    for (int64_t b = 0; b < nblk; b++) {
        const int64_t r = off[b];
        off[b] = b * kRefineBlk + 7 * nref;
        nref += r;
    }
    if (nref == 0) { free(off); return 0; }
    const int64_t nn = f->n + 7 * nref;
    charm_leaf_t *nl = (charm_leaf_t *) malloc((size_t) nn * sizeof(charm_leaf_t));
    int64_t *map = old_to_new ? old_to_new : (int64_t *) malloc((size_t) f->n * sizeof(int64_t));
    if (!nl || !map) { free(nl); if (map != old_to_new) free(map); free(off); return -1; }
    x.nl = nl;
    x.map = map;
    charm_forest_parallel_for_min(nblk, 2, refine_emit_range, &x);
    free(off);
    if (replace) {
        for (int64_t i = 0; i < f->n; i++) {
            if (flag[i] && f->leaf[i].level < maxlevel) {
                int64_t in_idx[8];
                for (int c = 0; c < 8; c++) in_idx[c] = map[i] + c;
                replace(user, f->leaf, &i, 1, nl, in_idx, 8);
            }
        }
    }
    if (map != old_to_new) free(map);
    free(f->leaf);
    f->leaf = nl;
    f->n = nn;
    f->cap = nn;
    return nref;
}

int64_t charm_forest_refine(charm_forest_t *f, const int8_t *flag, int maxlevel,
                            charm_forest_replace_fn replace, void *user)
{
    return charm_forest_refine_map(f, flag, maxlevel, replace, user, NULL);
}

static int is_family(const charm_forest_t *f, int64_t i)
{
    const charm_leaf_t *q = &f->leaf[i];
    if (q->level == 0 || i + 7 >= f->n || charm_leaf_child_id(q) != 0) return 0;
    for (int c = 1; c < 8; c++) {
        charm_leaf_t want;
        charm_leaf_t parent = *q;
        parent.level = (int8_t) (q->level - 1);
        child_of(&parent, c, &want);
        const charm_leaf_t *r = &f->leaf[i + c];
        if (r->tree != want.tree || r->level != want.level || r->x != want.x || r->y != want.y || r->z != want.z)
            return 0;
    }
    return 1;
}

int64_t charm_forest_coarsen(charm_forest_t *f, int minlevel, charm_forest_coarsen_fn pred,
                             charm_forest_replace_fn replace, void *user)
{
    if (f->n < 8) return 0;
    int8_t *merge = (int8_t *) calloc((size_t) f->n, 1);
    if (!merge) return -1;
    int64_t nm = 0;
    for (int64_t i = 0; i + 7 < f->n; i++) {
        if (!is_family(f, i)) continue;
        if (f->leaf[i].level <= minlevel) { i += 7; continue; }
        int64_t idx[8];
        for (int c = 0; c < 8; c++) idx[c] = i + c;
        if (pred && pred(user, f->leaf, idx)) { merge[i] = 1; nm++; }
        i += 7;
    }
    if (nm == 0) { free(merge); return 0; }
    int64_t nn = f->n - 7 * nm;
    charm_leaf_t *nl = (charm_leaf_t *) malloc((size_t) nn * sizeof(charm_leaf_t));
    int64_t *pidx = (int64_t *) malloc((size_t) nm * 2 * sizeof(int64_t));
    if (!nl || !pidx) { free(nl); free(pidx); free(merge); return -1; }
    int64_t k = 0, m = 0;
    for (int64_t i = 0; i < f->n;) {
        if (merge[i]) {
            charm_leaf_t p = f->leaf[i];
            p.level = (int8_t) (p.level - 1);
            int32_t len = CHARM_FOREST_QLEN(p.level);
            p.x &= ~(len - 1); p.y &= ~(len - 1); p.z &= ~(len - 1);
            pidx[2 * m] = i; pidx[2 * m + 1] = k; m++;
            nl[k++] = p;
            i += 8;
        } else {
            nl[k++] = f->leaf[i++];
        }
    }
    if (replace) {
        for (int64_t j = 0; j < nm; j++) {
            int64_t out_idx[8];
            for (int c = 0; c < 8; c++) out_idx[c] = pidx[2 * j] + c;
            replace(user, f->leaf, out_idx, 8, nl, &pidx[2 * j + 1], 1);
        }
    }
    free(pidx);
    free(merge);
    free(f->leaf);
    f->leaf = nl;
    f->n = nn;
    f->cap = nn;
    return nm;
}

typedef struct {
    charm_forest_t *f;
    int minlevel;
    charm_forest_coarsen_fn pred;
    void *user;
    int8_t *merge;       /* per old leaf: a merged family starts here */
    int64_t *off;        /* per block: merges, then the first output index */
    charm_leaf_t *nl;
    int64_t *n2o;
} coarsen_ctx_t;

static void coarsen_test_range(void *c, int64_t lo, int64_t hi)
{
    const coarsen_ctx_t *x = (const coarsen_ctx_t *) c;
    for (int64_t b = lo; b < hi; b++) {
        const int64_t i0 = b * kRefineBlk, i1 = (i0 + kRefineBlk < x->f->n) ? i0 + kRefineBlk : x->f->n;
        int64_t m = 0;
        for (int64_t i = i0; i < i1; i++) {
            /* a family starts at child id 0, so its other members never test true */
            int64_t idx[8];
            for (int ch = 0; ch < 8; ch++) idx[ch] = i + ch;
            x->merge[i] = (int8_t) (is_family(x->f, i) && x->f->leaf[i].level > x->minlevel &&
                                    x->pred(x->user, x->f->leaf, idx));
            m += x->merge[i];
        }
        x->off[b] = m;
    }
}

static void coarsen_emit_range(void *c, int64_t lo, int64_t hi)
{
    const coarsen_ctx_t *x = (const coarsen_ctx_t *) c;
    for (int64_t b = lo; b < hi; b++) {
        const int64_t i0 = b * kRefineBlk, i1 = (i0 + kRefineBlk < x->f->n) ? i0 + kRefineBlk : x->f->n;
        int64_t i = i0;
        /* skip the members of a family that starts in the block before */
        for (int64_t s = (i0 >= 7 ? i0 - 7 : 0); s < i0; s++)
            if (x->merge[s] && s + 8 > i) i = s + 8;
        int64_t k = x->off[b] + (i - i0);
        while (i < i1) {
            x->n2o[k] = i;
            if (x->merge[i]) {
                charm_leaf_t p = x->f->leaf[i];
                p.level = (int8_t) (p.level - 1);
                const int32_t len = CHARM_FOREST_QLEN(p.level);
                p.x &= ~(len - 1); p.y &= ~(len - 1); p.z &= ~(len - 1);
                x->nl[k++] = p;
                i += 8;
            } else {
                x->nl[k++] = x->f->leaf[i++];
            }
        }
    }
}

int64_t charm_forest_coarsen_map(charm_forest_t *f, int minlevel, charm_forest_coarsen_fn pred, void *user,
                                 int64_t *new_to_old)
{
    /* no predicate merges nothing, as in charm_forest_coarsen */
    if (!pred || f->n < 8) return 0;
    if (!new_to_old) return -1;
    const int64_t n = f->n, nblk = (n + kRefineBlk - 1) / kRefineBlk;
    int8_t *merge = (int8_t *) calloc((size_t) n, 1);
    int64_t *off = (int64_t *) malloc(sizeof(int64_t) * (size_t) (nblk + 1));
    if (!merge || !off) { free(merge); free(off); return -1; }
    coarsen_ctx_t x = {f, minlevel, pred, user, merge, off, NULL, new_to_old};
    charm_forest_parallel_for_min(nblk, 1, coarsen_test_range, &x);
    int64_t nm = 0;
    for (int64_t b = 0; b < nblk; b++) {
        const int64_t m = off[b];
        off[b] = b * kRefineBlk - 7 * nm;
        nm += m;
    }
    if (nm == 0) { free(merge); free(off); return 0; }
    const int64_t nn = n - 7 * nm;
    charm_leaf_t *nl = (charm_leaf_t *) malloc((size_t) nn * sizeof(charm_leaf_t));
    if (!nl) { free(merge); free(off); return -1; }
    x.nl = nl;
    charm_forest_parallel_for_min(nblk, 2, coarsen_emit_range, &x);
    new_to_old[nn] = n;
    free(merge);
    free(off);
    free(f->leaf);
    f->leaf = nl;
    f->n = nn;
    f->cap = nn;
    return nm;
}

/* A leaf must be refined when some leaf two or more levels finer touches one
 * of its faces: the same-size neighbour region is split and at least one of
 * its four children next to our face is split again. */
static int needs_split(const charm_forest_t *f, const uint64_t *keys, int64_t i)
{
    charm_face_nb_t nb;
    for (int face = 0; face < 6; face++) {
        charm_forest_face_neighbor_k(f, keys, i, face, &nb);
        if (nb.kind == CHARM_NB_UNBALANCED) {
            /* UNBALANCED is reported from both sides; only the coarse side splits */
            const charm_leaf_t *q = &f->leaf[i];
            for (int k = 0; k < 4; k++)
                if (nb.idx[k] >= 0 && f->leaf[nb.idx[k]].level > q->level + 1) return 1;
        }
    }
    return 0;
}

typedef struct { const charm_forest_t *f; const uint64_t *keys; int8_t *flag; } marks_ctx_t;

static void marks_range(void *c, int64_t lo, int64_t hi)
{
    const marks_ctx_t *m = (const marks_ctx_t *) c;
    for (int64_t i = lo; i < hi; i++) m->flag[i] = (int8_t) needs_split(m->f, m->keys, i);
}

int64_t charm_forest_balance_marks(const charm_forest_t *f, int8_t *flag)
{
    int64_t marks = 0;
    uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (f->n > 0 ? f->n : 1));
    if (keys) charm_forest_keys(f, keys);
    marks_ctx_t c = {f, keys, flag};
    charm_forest_parallel_for_min(f->n, 256, marks_range, &c);
    for (int64_t i = 0; i < f->n; i++) marks += flag[i];
    free(keys);
    return marks;
}

typedef struct {
    const charm_forest_t *f;
    const uint64_t *keys;
    const int64_t *cand;
    int8_t *flag;
} marks_at_ctx_t;

static void marks_at_range(void *c, int64_t lo, int64_t hi)
{
    const marks_at_ctx_t *m = (const marks_at_ctx_t *) c;
    for (int64_t j = lo; j < hi; j++) m->flag[m->cand[j]] = (int8_t) needs_split(m->f, m->keys, m->cand[j]);
}

int64_t charm_forest_balance_marks_at(const charm_forest_t *f, const int64_t *cand, int64_t n_cand, int8_t *flag)
{
    uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (f->n > 0 ? f->n : 1));
    if (keys) charm_forest_keys(f, keys);
    marks_at_ctx_t c = {f, keys, cand, flag};
    charm_forest_parallel_for_min(n_cand, 256, marks_at_range, &c);
    free(keys);
    int64_t marks = 0;
    for (int64_t j = 0; j < n_cand; j++) marks += flag[cand[j]];
    return marks;
}

typedef struct {
    const charm_forest_t *f;
    const uint64_t *keys;
    const int64_t *fresh;
    int32_t *nb;         /* [chunk][24] face-neighbour indices, -1 where none */
} hood_ctx_t;

static void hood_range(void *c, int64_t lo, int64_t hi)
{
    const hood_ctx_t *x = (const hood_ctx_t *) c;
    for (int64_t j = lo; j < hi; j++)
        for (int face = 0; face < 6; face++) {
            charm_face_nb_t nb;
            charm_forest_face_neighbor_k(x->f, x->keys, x->fresh[j], face, &nb);
            for (int k = 0; k < 4; k++) x->nb[24 * j + 4 * face + k] = (int32_t) nb.idx[k];
        }
}

int64_t charm_forest_fresh_neighbourhood(const charm_forest_t *f, const int64_t *fresh, int64_t n_fresh, int64_t *out)
{
    /* the face-neighbour searches run on several threads, a chunk of leaves
     * at a time, into a buffer; the marks are set on the calling thread */
    enum { kChunk = 1 << 16 };
    int8_t *mark = (int8_t *) calloc((size_t) f->n + 1, 1);
    uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (f->n > 0 ? f->n : 1));
    int32_t *nb = (int32_t *) malloc(sizeof(int32_t) * 24 * (size_t) (n_fresh < kChunk ? (n_fresh > 0 ? n_fresh : 1) : kChunk));
    if (!mark || !keys || !nb) { free(mark); free(keys); free(nb); return -1; }
    charm_forest_keys(f, keys);
    for (int64_t j0 = 0; j0 < n_fresh; j0 += kChunk) {
        const int64_t m = (n_fresh - j0 < kChunk) ? n_fresh - j0 : kChunk;
        hood_ctx_t c = {f, keys, fresh + j0, nb};
        charm_forest_parallel_for_min(m, 256, hood_range, &c);
        for (int64_t j = 0; j < m; j++) {
            mark[fresh[j0 + j]] = 1;
            for (int k = 0; k < 24; k++)
                if (nb[24 * j + k] >= 0) mark[nb[24 * j + k]] = 1;
        }
    }
    int64_t n = 0;
    for (int64_t i = 0; i < f->n; i++)
        if (mark[i]) out[n++] = i;
    free(mark);
    free(keys);
    free(nb);
    return n;
}

int64_t charm_forest_balance(charm_forest_t *f, charm_forest_replace_fn replace, void *user)
{
    int64_t total = 0;
    for (;;) {
        int8_t *flag = (int8_t *) calloc((size_t) f->n, 1);
        uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (f->n > 0 ? f->n : 1));
        if (!flag || !keys) { free(flag); free(keys); return -1; }
        charm_forest_keys(f, keys);
        marks_ctx_t c = {f, keys, flag};
        charm_forest_parallel_for_min(f->n, 256, marks_range, &c);
        int64_t marks = 0;
        for (int64_t i = 0; i < f->n; i++) marks += flag[i];
        free(keys);
        if (marks == 0) { free(flag); break; }
        int64_t r = charm_forest_refine(f, flag, -1, replace, user);
        free(flag);
        if (r < 0) return -1;
        total += r;
    }
    return total;
}

int charm_forest_is_balanced(const charm_forest_t *f)
{
    charm_face_nb_t nb;
    uint64_t *keys = (uint64_t *) malloc(sizeof(uint64_t) * (size_t) (f->n > 0 ? f->n : 1));
    if (keys) charm_forest_keys(f, keys);
    int ok = 1;
    for (int64_t i = 0; i < f->n && ok; i++)
        for (int face = 0; face < 6; face++) {
            charm_forest_face_neighbor_k(f, keys, i, face, &nb);
            if (nb.kind == CHARM_NB_UNBALANCED) { ok = 0; break; }
        }
    free(keys);
    return ok;
}

/* keep leaf_cmp referenced for debug builds that validate ordering */
int charm_forest_check_sorted(const charm_forest_t *f)
{
    for (int64_t i = 1; i < f->n; i++)
        if (leaf_cmp(&f->leaf[i - 1], &f->leaf[i]) >= 0) return 0;
    return 1;
}
