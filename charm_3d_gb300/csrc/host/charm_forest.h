/*
 * Host-side octree forest for the GPU DG solver.
 *
 * CHARM_3D keeps its mesh in p4est: a forest of octrees whose leaves are
 * Morton-ordered quadrants, refined/coarsened by callbacks and 2:1
 * face-balanced (reference: src/charm_amr.c:575-610 calls p4est_refine_ext,
 * p4est_coarsen_ext, p4est_balance_ext with CHARM_CONNECT_FACE).  p4est is not
 * part of this build, so this file provides the subset of its behaviour the
 * time step needs, on a brick of cubic trees (p8est_connectivity_new_brick
 * layout: tree id = i + ntx*(j + nty*k)):
 *
 *   - leaves sorted by (tree, Morton key of the lower corner), integer
 *     coordinates in units of 2^-CHARM_FOREST_MAXLEVEL of a tree edge, like
 *     p4est_qcoord_t (P8EST_MAXLEVEL = 19);
 *   - point location by binary search in Morton order;
 *   - face-neighbour queries across trees, with optional periodic wrap;
 *   - non-recursive refine and coarsen with replace callbacks, and a ripple
 *     2:1 face balance whose replace callback sees one level at a time;
 *   - flattening into the structure-of-arrays mesh of include/charm_gpu.h.
 *
 * Plain C99, no globals, safe to use from several handles on one thread each.
 */
#ifndef CHARM_FOREST_H
#define CHARM_FOREST_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHARM_FOREST_MAXLEVEL 19
#define CHARM_FOREST_ROOT_LEN ((int32_t) 1 << CHARM_FOREST_MAXLEVEL)
#define CHARM_FOREST_QLEN(l) ((int32_t) 1 << (CHARM_FOREST_MAXLEVEL - (l)))

typedef struct charm_leaf {
    int32_t x, y, z;     /* lower corner, tree-local integer coordinates */
    int32_t tree;        /* brick tree id */
    int8_t  level;
} charm_leaf_t;

struct charm_conn;

typedef struct charm_forest {
    int32_t ntree[3];        /* trees per axis */
    int32_t periodic[3];     /* wrap flags per axis */
    double  origin[3];       /* physical lower corner of tree (0,0,0) */
    double  tree_len[3];     /* physical edge lengths of one tree */
    int64_t n;               /* number of leaves */
    int64_t cap;
    charm_leaf_t *leaf;      /* sorted by (tree, Morton(x,y,z)) */
    /* unstructured hexahedral connectivity (charm_conn.h), or NULL for the
     * brick: with it, ntree = {n_tree, 1, 1}, no periodic wrap, and a face
     * neighbour across a tree face is found through the connectivity's
     * coordinate map (not owned by the forest) */
    const struct charm_conn *conn;
} charm_forest_t;

/* Kinds of face-neighbour relations, seen from one leaf. */
enum {
    CHARM_NB_BOUNDARY = 0,   /* domain boundary (no tree across, no wrap) */
    CHARM_NB_SAME     = 1,   /* one neighbour of the same level */
    CHARM_NB_BIGGER   = 2,   /* one neighbour one level coarser (this leaf hangs) */
    CHARM_NB_SMALLER  = 3,   /* four neighbours one level finer (mortar) */
    CHARM_NB_UNBALANCED = 4  /* neighbours two or more levels apart */
};

typedef struct charm_face_nb {
    int kind;
    int64_t idx[4];          /* neighbour leaf indices (1 or 4 used) */
    int wrap;                /* -1/0/+1: periodic wrap across the face */
    int nface;               /* the neighbours' face on this face (face ^ 1 inside a tree and in a brick) */
} charm_face_nb_t;

/* Replace callback: n_out old leaves (indices into the old array) were
 * replaced by n_in new leaves (indices into the new array).  Called after the
 * new leaf array is complete; both arrays are valid during the call. */
typedef void (*charm_forest_replace_fn)(void *user,
                                        const charm_leaf_t *old_leaves, const int64_t *out_idx, int n_out,
                                        const charm_leaf_t *new_leaves, const int64_t *in_idx, int n_in);

/* Coarsen predicate: the 8 siblings old[idx[0..7]] may be merged. */
typedef int (*charm_forest_coarsen_fn)(void *user, const charm_leaf_t *leaves, const int64_t idx[8]);

int  charm_forest_init_uniform(charm_forest_t *f, const int32_t ntree[3], const int32_t periodic[3],
                               const double origin[3], const double tree_len[3], int level);
void charm_forest_free(charm_forest_t *f);

/* Every tree of an unstructured connectivity refined uniformly to `level`;
 * the forest keeps a pointer to conn, which must outlive it. */
int  charm_forest_init_conn(charm_forest_t *f, const struct charm_conn *conn, int level);
int  charm_forest_copy(charm_forest_t *dst, const charm_forest_t *src);

/* Index of the leaf containing tree-local point (x,y,z) of tree t, or -1. */
int64_t charm_forest_find(const charm_forest_t *f, int32_t t, int32_t x, int32_t y, int32_t z);

/* Neighbour relation across face `face` (0..5, p4est numbering: -x,+x,-y,+y,-z,+z). */
void charm_forest_face_neighbor(const charm_forest_t *f, int64_t i, int face, charm_face_nb_t *nb);

/* Morton keys of the lower corners, key[i] for leaf i (n entries): with them
 * the *_k queries compare stored keys in their binary search instead of
 * recomputing one per step.  Valid until the forest changes; NULL keys make
 * the *_k queries compute them on the fly. */
void charm_forest_keys(const charm_forest_t *f, uint64_t *key);
int64_t charm_forest_find_k(const charm_forest_t *f, const uint64_t *key, int32_t t, int32_t x, int32_t y,
                            int32_t z);
void charm_forest_face_neighbor_k(const charm_forest_t *f, const uint64_t *key, int64_t i, int face,
                                  charm_face_nb_t *nb);

/* fn(ctx, lo, hi) over [0, n) split across threads (a pool of pthreads
 * started once per process, up to the online CPU count; serial below 16384
 * iterations).  fn must only write locations owned by its range.  The _min
 * form takes the smallest chunk worth a thread (small for loops whose
 * iterations search the forest). */
typedef void (*charm_forest_range_fn)(void *ctx, int64_t lo, int64_t hi);
void charm_forest_parallel_for(int64_t n, charm_forest_range_fn fn, void *ctx);
void charm_forest_parallel_for_min(int64_t n, int64_t min_chunk, charm_forest_range_fn fn, void *ctx);

/* Physical centre and edge lengths of leaf i. */
void charm_forest_leaf_geom(const charm_forest_t *f, int64_t i, double c[3], double h[3]);

/* Refine every leaf with flag[i] != 0 and level < maxlevel into its 8 children.
 * Returns the number of refined leaves, or -1 on allocation failure. */
int64_t charm_forest_refine(charm_forest_t *f, const int8_t *flag, int maxlevel,
                            charm_forest_replace_fn replace, void *user);
/* The same; when old_to_new is not NULL (room for the old leaf count) it
 * receives each old leaf's first index in the refined forest (its own, or
 * its first child's); it is left untouched when nothing is refined. */
int64_t charm_forest_refine_map(charm_forest_t *f, const int8_t *flag, int maxlevel,
                                charm_forest_replace_fn replace, void *user, int64_t *old_to_new);

/* One non-recursive pass over complete sibling families; merges those for which
 * pred() returns non-zero and whose level > minlevel.  Returns merges or -1. */
int64_t charm_forest_coarsen(charm_forest_t *f, int minlevel, charm_forest_coarsen_fn pred,
                             charm_forest_replace_fn replace, void *user);

/* The same pass with pred() called from several threads at once (it must
 * only read), no replace callback; new_to_old (required, room for the old
 * leaf count + 1) receives each new leaf's first old index, and new_to_old[new count]
 * = old count (a new leaf k is a merged family iff the difference to the
 * next entry is 8); it is left untouched when nothing is merged.  A NULL
 * pred merges nothing (returns 0); a NULL new_to_old returns -1. */
int64_t charm_forest_coarsen_map(charm_forest_t *f, int minlevel, charm_forest_coarsen_fn pred, void *user,
                                 int64_t *new_to_old);

/* 2:1 face balance by ripple refinement.  Returns leaves refined, or -1. */
int64_t charm_forest_balance(charm_forest_t *f, charm_forest_replace_fn replace, void *user);

/* One ripple pass: flag[i] = 1 for every leaf that a 2:1 face balance must
 * split now.  Returns the number of flags set. */
int64_t charm_forest_balance_marks(const charm_forest_t *f, int8_t *flag);

/* The same pass on the listed leaves only (cand, n_cand entries): flag[i]
 * is set for i in cand and left as it is elsewhere.  Returns the flags set. */
int64_t charm_forest_balance_marks_at(const charm_forest_t *f, const int64_t *cand, int64_t n_cand, int8_t *flag);

/* The leaves that a ripple pass after a refine must re-check: the new
 * leaves `fresh` and every leaf across one of their faces (a leaf that was
 * balanced before the refine can only become unbalanced next to a new
 * leaf).  Writes the sorted indices into out (room for f->n), returns the
 * count, or -1 on allocation failure. */
int64_t charm_forest_fresh_neighbourhood(const charm_forest_t *f, const int64_t *fresh, int64_t n_fresh, int64_t *out);

/* 1 if every face neighbour relation is at most one level apart. */
int charm_forest_is_balanced(const charm_forest_t *f);

/* Morton child id (0..7) of a leaf within its parent. */
int charm_leaf_child_id(const charm_leaf_t *q);

#ifdef __cplusplus
}
#endif

#endif /* CHARM_FOREST_H */
