/* p4est_iterate subset for the oracle build (see p4est_to_p8est.h). */
#ifndef CHARM_P8EST_ITERATE_SHIM_H
#define CHARM_P8EST_ITERATE_SHIM_H
#include "p4est_to_p8est.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct p4est_iter_volume_info {
    p4est_t *p4est;
    p4est_ghost_t *ghost_layer;
    p4est_quadrant_t *quad;
    p4est_locidx_t quadid;
    p4est_topidx_t treeid;
} p4est_iter_volume_info_t;

typedef struct p4est_iter_face_side {
    p4est_topidx_t treeid;
    int8_t face;
    int8_t is_hanging;
    union {
        struct {
            int8_t is_ghost;
            p4est_quadrant_t *quad;
            p4est_locidx_t quadid;
        } full;
        struct {
            int8_t is_ghost[4];
            p4est_quadrant_t *quad[4];
            p4est_locidx_t quadid[4];
        } hanging;
    } is;
} p4est_iter_face_side_t;

typedef struct p4est_iter_face_info {
    p4est_t *p4est;
    p4est_ghost_t *ghost_layer;
    int8_t orientation;
    int8_t tree_boundary;
    sc_array_t sides;
} p4est_iter_face_info_t;

typedef void (*p4est_iter_volume_t)(p4est_iter_volume_info_t *info, void *user_data);
typedef void (*p4est_iter_face_t)(p4est_iter_face_info_t *info, void *user_data);

static inline p4est_iter_face_side_t *p4est_iter_fside_array_index_int(sc_array_t *array, int it)
{
    return (p4est_iter_face_side_t *) sc_array_index_int(array, it);
}

void p4est_iterate(p4est_t *p4est, p4est_ghost_t *ghost_layer, void *user_data, p4est_iter_volume_t iter_volume,
                   p4est_iter_face_t iter_face, void *iter_edge, void *iter_corner);
#define p8est_iterate p4est_iterate

#ifdef __cplusplus
}
#endif
#endif
