/*
 * p4est-subset shim (test infrastructure for the oracle build only).
 *
 * CHARM_3D includes <p4est_to_p8est.h>, <p8est_bits.h>, <p8est_extended.h>
 * and <p8est_iterate.h> (reference include/charm_globals.h:8-12) and uses a
 * small part of p4est/libsc (the symbol census of its hot path).  p4est is
 * not installed here, so this header declares exactly that part, in 3D,
 * under the p4est_* names the reference uses after p4est_to_p8est.h.  The
 * implementation (p4est_shim.c) keeps one rank and runs on the host octree
 * of the GPU library (charm_forest.c).
 */
#ifndef CHARM_P4EST_SHIM_H
#define CHARM_P4EST_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <sys/types.h>

#ifdef __cplusplus
extern "C" {
#endif

#define P4_TO_P8 1
#define P4EST_DIM 3
#define P4EST_FACES 6
#define P4EST_CHILDREN 8
#define P4EST_HALF 4
#define P4EST_MAXLEVEL 19
#define P4EST_QMAXLEVEL 18
#define P4EST_ROOT_LEN ((p4est_qcoord_t) 1 << P4EST_MAXLEVEL)
#define P4EST_QUADRANT_LEN(l) ((p4est_qcoord_t) 1 << (P4EST_MAXLEVEL - (l)))

#define P4EST_ALLOC(t, n) ((t *) calloc((size_t) (n) > 0 ? (size_t) (n) : 1, sizeof(t)))
#define P4EST_ALLOC_ZERO(t, n) P4EST_ALLOC(t, n)
#define P4EST_REALLOC(p, t, n) ((t *) realloc((p), (size_t) (n) * sizeof(t)))
#define P4EST_FREE(p) free(p)
#define P4EST_ASSERT(c) ((void) 0)

typedef int32_t p4est_qcoord_t;
typedef int32_t p4est_topidx_t;
typedef int32_t p4est_locidx_t;
typedef int64_t p4est_gloidx_t;

typedef enum { P4EST_CONNECT_FACE = 31, P4EST_CONNECT_EDGE = 32, P4EST_CONNECT_CORNER = 33,
               P4EST_CONNECT_FULL = 33 } p4est_connect_type_t;

/* ---- libsc subset ---------------------------------------------------------- */
typedef int sc_MPI_Comm;
typedef int MPI_Comm;
#define sc_MPI_COMM_WORLD 0
#define sc_MPI_DOUBLE 1
#define sc_MPI_MIN 2
#define SC_CHECK_MPI(r) ((void) (r))
#define SC_MIN(a, b) ((a) < (b) ? (a) : (b))
#define SC_MAX(a, b) ((a) > (b) ? (a) : (b))
#define SC_EXTERN_C_BEGIN
#define SC_EXTERN_C_END

enum { SC_LP_DEFAULT = -1, SC_LP_ALWAYS = 0, SC_LP_TRACE, SC_LP_DEBUG, SC_LP_VERBOSE, SC_LP_INFO,
       SC_LP_STATISTICS, SC_LP_PRODUCTION, SC_LP_ESSENTIAL, SC_LP_ERROR, SC_LP_SILENT };
enum { SC_LC_GLOBAL = 1, SC_LC_NORMAL = 2 };

void sc_shim_log(int priority, const char *s);
void sc_shim_logf(int priority, const char *fmt, ...);
#define SC_GEN_LOG(package, category, priority, s) sc_shim_log((priority), (s))
#define SC_GEN_LOGF(package, category, priority, fmt, ...) sc_shim_logf((priority), (fmt), __VA_ARGS__)

double sc_MPI_Wtime(void);
int sc_MPI_Allreduce(void *send, void *recv, int count, int type, int op, sc_MPI_Comm comm);
int MPI_Finalize(void);
void sc_finalize(void);

typedef struct sc_array {
    size_t elem_size;
    size_t elem_count;
    ssize_t byte_alloc;
    char *array;
} sc_array_t;

sc_array_t *sc_array_new(size_t elem_size);
sc_array_t *sc_array_new_size(size_t elem_size, size_t elem_count);
void sc_array_destroy(sc_array_t *a);
void sc_array_init(sc_array_t *a, size_t elem_size);
void sc_array_reset(sc_array_t *a);
void sc_array_resize(sc_array_t *a, size_t new_count);
void *sc_array_push(sc_array_t *a);
static inline void *sc_array_index(sc_array_t *a, size_t i) { return a->array + a->elem_size * i; }
static inline void *sc_array_index_int(sc_array_t *a, int i) { return a->array + a->elem_size * (size_t) i; }

/* ---- forest ---------------------------------------------------------------- */
typedef struct p4est_quadrant {
    p4est_qcoord_t x, y, z;
    int8_t level, pad8;
    int16_t pad16;
    union {
        void *user_data;
        long user_long;
        int user_int;
        p4est_topidx_t which_tree;
    } p;
} p4est_quadrant_t;

typedef struct p4est_connectivity {
    p4est_topidx_t num_vertices;
    p4est_topidx_t num_trees;
    double *vertices;
    p4est_topidx_t *tree_to_vertex;
    size_t tree_attr_bytes;
    char *tree_to_attr;
    /* brick description (shim) */
    int32_t brick[3];
    int32_t periodic[3];
    double origin[3];
    double tree_len[3];
    /* unstructured hexahedral connectivity (charm_conn_t of the host
     * octree), or NULL for the brick */
    void *hexconn;
} p4est_connectivity_t;

typedef struct p4est_tree {
    sc_array_t quadrants;
    p4est_locidx_t quadrants_offset;
    int8_t maxlevel;
} p4est_tree_t;

struct charm_shim_state;

typedef struct p4est {
    sc_MPI_Comm mpicomm;
    int mpisize, mpirank;
    size_t data_size;
    void *user_pointer;
    p4est_topidx_t first_local_tree, last_local_tree;
    p4est_locidx_t local_num_quadrants;
    p4est_gloidx_t global_num_quadrants;
    sc_array_t *trees;          /* p4est_tree_t per tree; quadrants are views */
    p4est_connectivity_t *connectivity;
    struct charm_shim_state *shim;
} p4est_t;

static inline p4est_tree_t *p4est_tree_array_index(sc_array_t *array, p4est_topidx_t it)
{
    return (p4est_tree_t *) sc_array_index(array, (size_t) it);
}

typedef struct p4est_ghost {
    int mpisize;
    p4est_topidx_t num_trees;
    p4est_connect_type_t btype;
    sc_array_t ghosts;          /* p4est_quadrant_t copies */
    /* shim: source leaf and physical shift of each ghost */
    int64_t *src;
    double *shift;              /* [3 * count] */
} p4est_ghost_t;

typedef void (*p4est_init_t)(p4est_t *p4est, p4est_topidx_t which_tree, p4est_quadrant_t *quadrant);
typedef int (*p4est_refine_t)(p4est_t *p4est, p4est_topidx_t which_tree, p4est_quadrant_t *quadrant);
typedef int (*p4est_coarsen_t)(p4est_t *p4est, p4est_topidx_t which_tree, p4est_quadrant_t *quadrants[]);
typedef void (*p4est_replace_t)(p4est_t *p4est, p4est_topidx_t which_tree, int num_outgoing,
                                p4est_quadrant_t *outgoing[], int num_incoming, p4est_quadrant_t *incoming[]);
typedef int (*p4est_weight_t)(p4est_t *p4est, p4est_topidx_t which_tree, p4est_quadrant_t *quadrant);

void p4est_qcoord_to_vertex(p4est_connectivity_t *conn, p4est_topidx_t treeid, p4est_qcoord_t x,
                            p4est_qcoord_t y, p4est_qcoord_t z, double vxyz[3]);

void p4est_refine(p4est_t *p4est, int refine_recursive, p4est_refine_t refine_fn, p4est_init_t init_fn);
void p4est_refine_ext(p4est_t *p4est, int refine_recursive, int maxlevel, p4est_refine_t refine_fn,
                      p4est_init_t init_fn, p4est_replace_t replace_fn);
void p4est_coarsen(p4est_t *p4est, int coarsen_recursive, p4est_coarsen_t coarsen_fn, p4est_init_t init_fn);
void p4est_coarsen_ext(p4est_t *p4est, int coarsen_recursive, int callback_orphans, p4est_coarsen_t coarsen_fn,
                       p4est_init_t init_fn, p4est_replace_t replace_fn);
void p4est_balance(p4est_t *p4est, p4est_connect_type_t btype, p4est_init_t init_fn);
void p4est_balance_ext(p4est_t *p4est, p4est_connect_type_t btype, p4est_init_t init_fn, p4est_replace_t replace_fn);
p4est_gloidx_t p4est_partition(p4est_t *p4est, int allow_for_coarsening, p4est_weight_t weight_fn);

p4est_ghost_t *p4est_ghost_new(p4est_t *p4est, p4est_connect_type_t btype);
void p4est_ghost_destroy(p4est_ghost_t *ghost);
void p4est_ghost_exchange_data(p4est_t *p4est, p4est_ghost_t *ghost, void *ghost_data);

#ifdef __cplusplus
}
#endif

#include "p8est_iterate.h"

#endif /* CHARM_P4EST_SHIM_H */
