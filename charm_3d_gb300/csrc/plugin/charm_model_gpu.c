/*
 * GPU model plugin for CHARM_3D: a drop-in timestep_single_fn / get_dt_fn.
 *
 * Compiled inside the reference's tree (it includes the reference's own
 * charm_globals.h and p4est), it replaces the pair that the model's init
 * registers, charm_model_ns_init (reference
 * src/models/ns/charm_model_ns_init.cpp:79-88) or charm_model_euler_init
 * (src/models/euler/charm_model_euler_init.cpp:18), and steps the model
 * it replaced (SSP-RK3 or forward Euler):
 *
 *     charm_model_gpu_init(ctx, CHARM_GPU_PREC_FP64, 0);
 *
 * after charm_init_context_yaml() has filled ctx from task.yaml.  The time
 * loop (charm_timesteps, src/charm_timesteps.c:23-51) is unchanged.
 *
 * Per step the plugin keeps the reference's prologue of
 * charm_model_ns_timestep_single (src/models/ns/charm_model.c:197-242):
 * every REFINE_PERIOD steps it brings the state back to the quadrants and
 * runs the reference's own charm_adapt on the CPU (p4est refine/coarsen/
 * balance with its L2 projection), then re-flattens the forest; every
 * FILE_OUTPUT_STEP steps it brings the state back for charm_write_solution.
 * Otherwise the conserved state stays in HBM and the whole SSP-RK3 step
 * (residual, update, limiter, combinations) runs in libcharm_gpu.so.
 *
 * Flattening walks the forest with p4est_iterate, so the face list is the
 * one the reference's own face callbacks see.  Single MPI rank: ghost
 * quadrants are rejected.  Geometry: a forest of axis-aligned boxes (bricks
 * of cube trees) goes to the box kernels; any other forest (the
 * tree-per-hexahedron connectivity of a gmsh mesh, trees in any
 * orientation) goes to the general-hexahedron kernels with every leaf's
 * corners from p4est_qcoord_to_vertex and p4est's own face sides.
 */
#include "charm_globals.h"
#include "charm_amr.h"
#include "charm_eos.h"
#include "charm_fluxes.h"
#include "charm_limiter.h"
#include "charm_models.h"
#include "charm_gpu.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    charm_gpu_handle_t h;
    int precision;
    int model;             /* CHARM_GPU_MODEL_* of the pair the plugin replaced */
    int device;
    int mesh_valid;        /* forest unchanged since the last upload */
    int device_newer;      /* HBM holds a newer state than the quadrants */
    int status;            /* last non-zero status */
    /* flattened arrays (owned) */
    int64_t n_elem, n_face, n_bface, cap_face, cap_bface;
    double *center;
    int8_t *level;
    int32_t *face_elem0, *face_elem1, *face_all;
    uint8_t *face_info;
    int32_t *bface_elem;
    int8_t *bface_face, *bface_bnd;
    double tree_len[3];
    double *state;         /* [V][B][E] staging buffer */
    /* general hexahedra: set when a leaf is not an axis-aligned box of the
     * common tree scale or a face joins other than opposite box faces */
    int hex;
    double *vertex;        /* [8][3][E] leaf corners */
    int32_t *hface_elem0, *hface_elem1, *hface_all;
    uint8_t *hface_info;
    int8_t *hface_face0, *hface_face1, *hface_face_all;
    int64_t n_hface, cap_hface;
} charm_gpu_plugin_t;

static charm_gpu_plugin_t g_gpu;

int charm_model_gpu_status(void) { return g_gpu.status; }

static void plugin_error(int rc, const char *where)
{
    g_gpu.status = rc;
    CHARM_GLOBAL_LERRORF("GPU plugin: %s failed: %d (%s)\n", where, rc, charm_gpu_last_error());
}

/* ---- flattening ------------------------------------------------------------- */

typedef struct {
    p4est_t *p4est;
    int err;
} flat_ctx_t;

static int64_t local_index(p4est_t *p4est, p4est_topidx_t treeid, p4est_locidx_t quadid)
{
    p4est_tree_t *tree = p4est_tree_array_index(p4est->trees, treeid);
    return (int64_t) tree->quadrants_offset + quadid;
}

static void flat_volume(p4est_iter_volume_info_t *info, void *user)
{
    flat_ctx_t *fc = (flat_ctx_t *) user;
    charm_data_t *d = charm_get_quad_data(info->quad);
    int64_t i = local_index(info->p4est, info->treeid, info->quadid);
    const int64_t E = g_gpu.n_elem;
    int k;
    if (i < 0 || i >= E) { fc->err = 1; return; }
    for (k = 0; k < 3; k++) g_gpu.center[k * E + i] = d->par.g.c[k];
    g_gpu.level[i] = info->quad->level;
    /* the leaf's corners, as charm_quad_get_vertices computes them
     * (src/charm_geom.c:12-31) */
    p4est_qcoord_t l = P4EST_QUADRANT_LEN(info->quad->level);
    double v[8][3];
    for (k = 0; k < 8; k++) {
        p4est_qcoord_to_vertex(info->p4est->connectivity, info->treeid, info->quad->x + ((k & 1) ? l : 0),
                               info->quad->y + ((k & 2) ? l : 0), info->quad->z + ((k & 4) ? l : 0), v[k]);
        for (int dd = 0; dd < 3; dd++) g_gpu.vertex[(int64_t) (3 * k + dd) * E + i] = v[k][dd];
    }
    /* a box: every corner at the lower or upper end of each axis as its
     * corner bits say, edges of the common tree scale */
    if (i == 0)
        for (k = 0; k < 3; k++) g_gpu.tree_len[k] = ldexp(d->par.g.dh[k], info->quad->level);
    for (int dd = 0; dd < 3; dd++) {
        const double lo = v[0][dd], hi = v[7][dd];
        if (fabs(ldexp(hi - lo, info->quad->level) - g_gpu.tree_len[dd]) > 1e-12 * g_gpu.tree_len[dd]) g_gpu.hex = 1;
        for (k = 0; k < 8; k++)
            if (v[k][dd] != (((k >> dd) & 1) ? hi : lo)) g_gpu.hex = 1;
    }
}

static void push_face(int64_t a, int64_t b, unsigned info)
{
    if (g_gpu.n_face == g_gpu.cap_face) {
        g_gpu.cap_face = g_gpu.cap_face ? 2 * g_gpu.cap_face : 1024;
        g_gpu.face_elem0 = (int32_t *) realloc(g_gpu.face_elem0, sizeof(int32_t) * (size_t) g_gpu.cap_face);
        g_gpu.face_elem1 = (int32_t *) realloc(g_gpu.face_elem1, sizeof(int32_t) * (size_t) g_gpu.cap_face);
        g_gpu.face_info = (uint8_t *) realloc(g_gpu.face_info, (size_t) g_gpu.cap_face);
    }
    g_gpu.face_elem0[g_gpu.n_face] = (int32_t) a;
    g_gpu.face_elem1[g_gpu.n_face] = (int32_t) b;
    g_gpu.face_info[g_gpu.n_face] = (uint8_t) info;
    g_gpu.n_face++;
}

/* a record of the general-hexahedron form: p4est's side order, both faces */
static void push_hface(int64_t a, int64_t b, unsigned info, int fa, int fb)
{
    if (g_gpu.n_hface == g_gpu.cap_hface) {
        g_gpu.cap_hface = g_gpu.cap_hface ? 2 * g_gpu.cap_hface : 1024;
        g_gpu.hface_elem0 = (int32_t *) realloc(g_gpu.hface_elem0, sizeof(int32_t) * (size_t) g_gpu.cap_hface);
        g_gpu.hface_elem1 = (int32_t *) realloc(g_gpu.hface_elem1, sizeof(int32_t) * (size_t) g_gpu.cap_hface);
        g_gpu.hface_info = (uint8_t *) realloc(g_gpu.hface_info, (size_t) g_gpu.cap_hface);
        g_gpu.hface_face0 = (int8_t *) realloc(g_gpu.hface_face0, (size_t) g_gpu.cap_hface);
        g_gpu.hface_face1 = (int8_t *) realloc(g_gpu.hface_face1, (size_t) g_gpu.cap_hface);
    }
    g_gpu.hface_elem0[g_gpu.n_hface] = (int32_t) a;
    g_gpu.hface_elem1[g_gpu.n_hface] = (int32_t) b;
    g_gpu.hface_info[g_gpu.n_hface] = (uint8_t) info;
    g_gpu.hface_face0[g_gpu.n_hface] = (int8_t) fa;
    g_gpu.hface_face1[g_gpu.n_hface] = (int8_t) fb;
    g_gpu.n_hface++;
}

static void push_bface(int64_t e, int face, int bnd)
{
    if (g_gpu.n_bface == g_gpu.cap_bface) {
        g_gpu.cap_bface = g_gpu.cap_bface ? 2 * g_gpu.cap_bface : 1024;
        g_gpu.bface_elem = (int32_t *) realloc(g_gpu.bface_elem, sizeof(int32_t) * (size_t) g_gpu.cap_bface);
        g_gpu.bface_face = (int8_t *) realloc(g_gpu.bface_face, (size_t) g_gpu.cap_bface);
        g_gpu.bface_bnd = (int8_t *) realloc(g_gpu.bface_bnd, (size_t) g_gpu.cap_bface);
    }
    g_gpu.bface_elem[g_gpu.n_bface] = (int32_t) e;
    g_gpu.bface_face[g_gpu.n_bface] = (int8_t) face;
    g_gpu.bface_bnd[g_gpu.n_bface] = (int8_t) bnd;
    g_gpu.n_bface++;
}

/* Boundary id of tree face `face`: the index of attr->bnd[face] in ctx->bnd. */
static int bnd_index(p4est_t *p4est, p4est_topidx_t treeid, int face)
{
    charm_ctx_t *ctx = charm_get_ctx(p4est);
    charm_tree_attr_t *attr = charm_get_tree_attr(p4est, treeid);
    if (!attr->bnd[face]) return -1;
    return (int) (((char *) attr->bnd[face] - ctx->bnd->array) / (ptrdiff_t) ctx->bnd->elem_size);
}

static void flat_face(p4est_iter_face_info_t *info, void *user)
{
    flat_ctx_t *fc = (flat_ctx_t *) user;
    sc_array_t *sides = &info->sides;
    p4est_iter_face_side_t *s0 = p4est_iter_fside_array_index_int(sides, 0);
    if (sides->elem_count == 1) {
        int b = bnd_index(info->p4est, s0->treeid, s0->face);
        if (s0->is.full.is_ghost || b < 0) { fc->err = 2; return; }
        push_bface(local_index(info->p4est, s0->treeid, s0->is.full.quadid), s0->face, b);
        return;
    }
    p4est_iter_face_side_t *s1 = p4est_iter_fside_array_index_int(sides, 1);
    /* the general-hexahedron records keep p4est's side order (side 0 gives
     * the normal, as in the reference's face callbacks) */
    if (s0->is_hanging || s1->is_hanging) {
        const int h0 = s0->is_hanging;
        p4est_iter_face_side_t *hs = h0 ? s0 : s1, *fs = h0 ? s1 : s0;
        if (fs->is.full.is_ghost) { fc->err = 3; return; }
        const int64_t big = local_index(info->p4est, fs->treeid, fs->is.full.quadid);
        for (int k = 0; k < 4; k++) {
            if (hs->is.hanging.is_ghost[k]) { fc->err = 3; return; }
            const int64_t sm = local_index(info->p4est, hs->treeid, hs->is.hanging.quadid[k]);
            const unsigned bits = (unsigned) (s0->face / 2) | ((h0 ? 1u : 2u) << 2) | ((unsigned) k << 4);
            if (h0) push_hface(sm, big, bits, s0->face, s1->face);
            else push_hface(big, sm, bits, s0->face, s1->face);
        }
    } else {
        if (s0->is.full.is_ghost || s1->is.full.is_ghost) { fc->err = 3; return; }
        push_hface(local_index(info->p4est, s0->treeid, s0->is.full.quadid),
                   local_index(info->p4est, s1->treeid, s1->is.full.quadid), (unsigned) (s0->face / 2), s0->face,
                   s1->face);
    }
    /* a box forest joins a leaf's face 2 dir + 1 to the other's face 2 dir */
    if ((s0->face ^ 1) != s1->face) g_gpu.hex = 1;
    /* order the sides so that side 0 is the leaf whose face 2*dir+1 is on the face */
    if (!(s0->face & 1)) {
        p4est_iter_face_side_t *t = s0;
        s0 = s1;
        s1 = t;
    }
    const int d = s0->face / 2;
    if (!s0->is_hanging && !s1->is_hanging) {
        if (s0->is.full.is_ghost || s1->is.full.is_ghost) { fc->err = 3; return; }
        int64_t a = local_index(info->p4est, s0->treeid, s0->is.full.quadid);
        int64_t b = local_index(info->p4est, s1->treeid, s1->is.full.quadid);
        /* periodic wrap: the two centres are further apart than one leaf */
        double dc = g_gpu.center[d * g_gpu.n_elem + b] - g_gpu.center[d * g_gpu.n_elem + a];
        unsigned wrap = (dc < 0.0) ? 0x40u : 0u;
        push_face(a, b, (unsigned) d | wrap);
        return;
    }
    /* hanging face: one record per small leaf, in the hanging side's order */
    const int small_is_0 = s0->is_hanging;
    p4est_iter_face_side_t *hs = small_is_0 ? s0 : s1, *fs = small_is_0 ? s1 : s0;
    if (fs->is.full.is_ghost) { fc->err = 3; return; }
    int64_t big = local_index(info->p4est, fs->treeid, fs->is.full.quadid);
    for (int k = 0; k < 4; k++) {
        if (hs->is.hanging.is_ghost[k]) { fc->err = 3; return; }
        int64_t sm = local_index(info->p4est, hs->treeid, hs->is.hanging.quadid[k]);
        double dc = g_gpu.center[d * g_gpu.n_elem + (small_is_0 ? big : sm)] -
                    g_gpu.center[d * g_gpu.n_elem + (small_is_0 ? sm : big)];
        unsigned wrap = (dc < 0.0) ? 0x40u : 0u;
        unsigned info_bits = (unsigned) d | ((small_is_0 ? 1u : 2u) << 2) | ((unsigned) k << 4) | wrap;
        if (small_is_0) push_face(sm, big, info_bits);
        else push_face(big, sm, info_bits);
    }
}

/* Flatten the local forest into a charm_gpu_mesh_t whose arrays live in the
 * plugin until the next call.  Returns a CHARM_GPU_* status. */
int charm_model_gpu_flatten(p4est_t *p4est, charm_gpu_mesh_t *mesh)
{
    flat_ctx_t fc = {p4est, 0};
    g_gpu.n_elem = p4est->local_num_quadrants;
    g_gpu.n_face = g_gpu.n_bface = g_gpu.n_hface = 0;
    g_gpu.hex = 0;
    g_gpu.center = (double *) realloc(g_gpu.center, sizeof(double) * 3 * (size_t) g_gpu.n_elem);
    g_gpu.level = (int8_t *) realloc(g_gpu.level, (size_t) g_gpu.n_elem);
    g_gpu.vertex = (double *) realloc(g_gpu.vertex, sizeof(double) * 24 * (size_t) g_gpu.n_elem);
    if (!g_gpu.center || !g_gpu.level || !g_gpu.vertex) return CHARM_GPU_ENOMEM;
    p4est_iterate(p4est, NULL, &fc, flat_volume, NULL, NULL, NULL);
    if (fc.err) return CHARM_GPU_EINVAL;
    p4est_iterate(p4est, NULL, &fc, NULL, flat_face, NULL, NULL);
    if (fc.err) return fc.err == 3 ? CHARM_GPU_ENOTSUP : CHARM_GPU_EINVAL;
    /* mortar sub-faces of one big face stay consecutive, as the ABI requires */
    g_gpu.face_all = (int32_t *) realloc(g_gpu.face_all, sizeof(int32_t) * 2 * (size_t) (g_gpu.n_face + 1));
    memcpy(g_gpu.face_all, g_gpu.face_elem0, sizeof(int32_t) * (size_t) g_gpu.n_face);
    memcpy(g_gpu.face_all + g_gpu.n_face, g_gpu.face_elem1, sizeof(int32_t) * (size_t) g_gpu.n_face);
    mesh->n_elem = g_gpu.n_elem;
    mesh->center = g_gpu.center;
    mesh->level = g_gpu.level;
    for (int k = 0; k < 3; k++) mesh->tree_len[k] = g_gpu.tree_len[k];
    mesh->n_face = g_gpu.n_face;
    mesh->face_elem = g_gpu.face_all;
    mesh->face_info = g_gpu.face_info;
    mesh->n_bface = g_gpu.n_bface;
    mesh->bface_elem = g_gpu.bface_elem;
    mesh->bface_face = g_gpu.bface_face;
    mesh->bface_bnd = g_gpu.bface_bnd;
    /* the general-hexahedron form of the same faces */
    const int64_t nh = g_gpu.n_hface;
    g_gpu.hface_all = (int32_t *) realloc(g_gpu.hface_all, sizeof(int32_t) * 2 * (size_t) (nh + 1));
    g_gpu.hface_face_all = (int8_t *) realloc(g_gpu.hface_face_all, 2 * (size_t) (nh + 1));
    if (!g_gpu.hface_all || !g_gpu.hface_face_all) return CHARM_GPU_ENOMEM;
    if (nh) {
        memcpy(g_gpu.hface_all, g_gpu.hface_elem0, sizeof(int32_t) * (size_t) nh);
        memcpy(g_gpu.hface_all + nh, g_gpu.hface_elem1, sizeof(int32_t) * (size_t) nh);
        memcpy(g_gpu.hface_face_all, g_gpu.hface_face0, (size_t) nh);
        memcpy(g_gpu.hface_face_all + nh, g_gpu.hface_face1, (size_t) nh);
    }
    return CHARM_GPU_OK;
}

/* After charm_model_gpu_flatten: 1 when the forest needs the
 * general-hexahedron kernels, and then that form of the mesh (the face
 * records in p4est's side order with both sides' faces, and the corners). */
int charm_model_gpu_flatten_hex(charm_gpu_mesh_t *mesh, charm_gpu_hex_t *hex)
{
    mesh->n_face = g_gpu.n_hface;
    mesh->face_elem = g_gpu.hface_all;
    mesh->face_info = g_gpu.hface_info;
    hex->vertex = g_gpu.vertex;
    hex->face_face = g_gpu.hface_face_all;
    return g_gpu.hex;
}

/* ---- configuration from the reference context ------------------------------- */

void charm_model_gpu_timestep_single(p4est_t *p4est, charm_real_t *dt, p4est_ghost_t **_ghost,
                                     charm_data_t **_ghost_data);

/* The model of a context, told apart as the reference does, by the step its
 * model init registered: charm_model_euler_init's forward-Euler step
 * (src/models/euler/charm_model_euler_init.cpp:18) or the NS model's
 * SSP-RK3 step; once the plugin pair is registered, the model it replaced. */
static int model_of(const charm_ctx_t *ctx)
{
    if (ctx->timestep_single_fn == charm_model_euler_timestep_single) return CHARM_GPU_MODEL_EULER;
    if (ctx->timestep_single_fn == charm_model_gpu_timestep_single) return g_gpu.model;
    return CHARM_GPU_MODEL_NS;
}

int charm_model_gpu_config(charm_ctx_t *ctx, int precision, charm_gpu_config_t *cfg)
{
    size_t i;
    int k;
    memset(cfg, 0, sizeof(*cfg));
    cfg->model = model_of(ctx);
    if (ctx->flux_fn == charm_calc_flux_lf) cfg->flux = CHARM_GPU_FLUX_LF;
    else if (ctx->flux_fn == charm_calc_flux_hllc) cfg->flux = CHARM_GPU_FLUX_HLLC;
    else if (ctx->flux_fn == charm_calc_flux_cd) cfg->flux = CHARM_GPU_FLUX_CD;
    else if (ctx->flux_fn == charm_calc_flux_godunov) cfg->flux = CHARM_GPU_FLUX_GODUNOV;
    else return CHARM_GPU_ENOTSUP;
    if (ctx->lim_fn == NULL) cfg->limiter = CHARM_GPU_LIM_NONE;
    else if (ctx->lim_fn == charm_limiter_bj) cfg->limiter = CHARM_GPU_LIM_BJ;
    else return CHARM_GPU_ENOTSUP;
    if (ctx->mat->elem_count < 1) return CHARM_GPU_EINVAL;
    charm_mat_t *mat = (charm_mat_t *) sc_array_index(ctx->mat, 0);
    if (mat->eos_fn == charm_mat_eos_ideal) cfg->eos = CHARM_GPU_EOS_IDEAL;
    else if (mat->eos_fn == charm_mat_eos_mix) cfg->eos = CHARM_GPU_EOS_MIX;
    else return CHARM_GPU_ENOTSUP;
    cfg->precision = precision;
    cfg->dt_mode = CHARM_GPU_DT_TAU;
    if (ctx->comp->elem_count > CHARM_GPU_MAX_COMP || ctx->bnd->elem_count > CHARM_GPU_MAX_BND) return CHARM_GPU_ENOTSUP;
    cfg->n_comp = (int) ctx->comp->elem_count;
    for (i = 0; i < ctx->comp->elem_count; i++) {
        charm_comp_t *c = (charm_comp_t *) sc_array_index(ctx->comp, i);
        charm_gpu_comp_t *g = &cfg->comp[i];
        g->m = c->m; g->ml0 = c->ml0; g->kp0 = c->kp0; g->t0 = c->t0; g->ts = c->ts;
        g->sig = c->sig; g->ek = c->ek; g->h0 = c->h0;
        g->cp_type = c->cp_type == COMP_CP_POLYNOM ? CHARM_GPU_CP_POLYNOM : CHARM_GPU_CP_CONST;
        g->kp_type = c->kp_type == COMP_KP_SATHERLAND ? CHARM_GPU_LAW_SUTHERLAND : CHARM_GPU_LAW_CONST;
        g->ml_type = c->ml_type == COMP_ML_SATHERLAND ? CHARM_GPU_LAW_SUTHERLAND : CHARM_GPU_LAW_CONST;
        if (c->cp->elem_count > CHARM_GPU_MAX_CP) return CHARM_GPU_ENOTSUP;
        g->n_cp = (int) c->cp->elem_count;
        for (k = 0; k < g->n_cp; k++) g->cp[k] = *(charm_real_t *) sc_array_index(c->cp, (size_t) k);
    }
    cfg->n_bnd = (int) ctx->bnd->elem_count;
    for (i = 0; i < ctx->bnd->elem_count; i++) {
        charm_bnd_t *b = (charm_bnd_t *) sc_array_index(ctx->bnd, i);
        cfg->bnd[i].type = (int) b->type;
        int np = b->type == BOUND_INLET ? 5 : b->type == BOUND_WALL_NO_SLIP ? 1 :
                 b->type == BOUND_MASS_FLOW ? 7 + cfg->n_comp : 0;
        for (k = 0; k < np; k++) cfg->bnd[i].params[k] = b->params[k];
    }
    if (ctx->reg && ctx->reg->elem_count) {
        charm_reg_t *r = (charm_reg_t *) sc_array_index(ctx->reg, 0);
        for (k = 0; k < 3; k++) cfg->grav[k] = r->grav[k];
    }
    cfg->tau = ctx->dt;
    cfg->cfl = ctx->CFL;
    if (cfg->model == CHARM_GPU_MODEL_NS) {   /* ctx->model is a union: the ns member only for NS */
        cfg->t_ref = ctx->model.ns.t_ref;
        cfg->use_visc = ctx->model.ns.use_visc;
        cfg->use_diff = ctx->model.ns.use_diff;
    }
    cfg->p_order = CHARM_BASE_FN_COUNT == 10 ? 2 : 1;   /* include/charm_def.h:177 */
    cfg->n_react = 0;
    if (ctx->reactions) {   /* charm_reaction_t list of src/models/ns/charm_model_ns_init.cpp:58-77 */
        if ((int) ctx->reactions->elem_count > CHARM_GPU_MAX_REACT) return CHARM_GPU_ENOTSUP;
        cfg->n_react = (int) ctx->reactions->elem_count;
        for (i = 0; i < cfg->n_react; i++) {
            charm_reaction_t *r = (charm_reaction_t *) sc_array_index(ctx->reactions, i);
            for (k = 0; k < 3; k++) { cfg->react[i].left[k] = r->left_comps[k]; cfg->react[i].right[k] = r->right_comps[k]; }
            cfg->react[i].a = r->a;
            cfg->react[i].e = r->e;
            cfg->react[i].n = r->n;
        }
    }
    return CHARM_GPU_OK;
}

/* ---- state transfer ----------------------------------------------------------- */

typedef struct {
    int dir;   /* 0: quadrants -> staging, 1: staging -> quadrants */
    int nc;
    int64_t E;
} xfer_ctx_t;

static void xfer_volume(p4est_iter_volume_info_t *info, void *user)
{
    xfer_ctx_t *x = (xfer_ctx_t *) user;
    charm_data_t *d = charm_get_quad_data(info->quad);
    int64_t i = local_index(info->p4est, info->treeid, info->quadid);
    const int B = CHARM_BASE_FN_COUNT;
    double *u = g_gpu.state;
    for (int k = 0; k < B; k++) {
        double *dst[4] = {&d->par.c.ru[k], &d->par.c.rv[k], &d->par.c.rw[k], &d->par.c.re[k]};
        for (int v = 0; v < 4; v++) {
            if (x->dir == 0) u[(v * B + k) * x->E + i] = *dst[v];
            else *dst[v] = u[(v * B + k) * x->E + i];
        }
        for (int j = 0; j < x->nc; j++) {
            if (x->dir == 0) u[((4 + j) * B + k) * x->E + i] = d->par.c.rc[j][k];
            else d->par.c.rc[j][k] = u[((4 + j) * B + k) * x->E + i];
        }
    }
}

static int transfer(p4est_t *p4est, int to_quadrants)
{
    xfer_ctx_t x = {to_quadrants, (int) charm_get_comp_count(p4est), p4est->local_num_quadrants};
    size_t n = (size_t) (4 + x.nc) * CHARM_BASE_FN_COUNT * (size_t) x.E;
    g_gpu.state = (double *) realloc(g_gpu.state, sizeof(double) * n);
    if (!g_gpu.state) return CHARM_GPU_ENOMEM;
    if (to_quadrants) {
        int rc = charm_gpu_get_state(g_gpu.h, g_gpu.state, 0);
        if (rc) return rc;
        p4est_iterate(p4est, NULL, &x, xfer_volume, NULL, NULL, NULL);
        return CHARM_GPU_OK;
    }
    p4est_iterate(p4est, NULL, &x, xfer_volume, NULL, NULL, NULL);
    return charm_gpu_set_state(g_gpu.h, g_gpu.state, 0);
}

/* Bring the newest state back into the quadrants' user data (before output,
 * adapt, or at the end of the run). */
int charm_model_gpu_download(p4est_t *p4est)
{
    if (!g_gpu.h || !g_gpu.device_newer) return CHARM_GPU_OK;
    int rc = transfer(p4est, 1);
    if (!rc) g_gpu.device_newer = 0;
    return rc;
}

static int upload_all(p4est_t *p4est)
{
    charm_gpu_mesh_t mesh;
    charm_gpu_hex_t hex;
    int rc = charm_model_gpu_flatten(p4est, &mesh);
    if (rc) return rc;
    if (charm_model_gpu_flatten_hex(&mesh, &hex)) rc = charm_gpu_upload_mesh_hex(g_gpu.h, &mesh, &hex);
    else rc = charm_gpu_upload_mesh(g_gpu.h, &mesh);
    if (rc) return rc;
    if ((rc = transfer(p4est, 0))) return rc;
    g_gpu.mesh_valid = 1;
    return CHARM_GPU_OK;
}

/* ---- the plugin pair ------------------------------------------------------------- */

charm_real_t charm_model_gpu_get_dt(p4est_t *p4est)
{
    /* the reference's get_dt returns the fixed TAU (src/models/ns/charm_model.c:49) */
    return charm_get_ctx(p4est)->dt;
}

void charm_model_gpu_timestep_single(p4est_t *p4est, charm_real_t *dt, p4est_ghost_t **_ghost,
                                     charm_data_t **_ghost_data)
{
    charm_ctx_t *ctx = charm_get_ctx(p4est);
    int rc;
    if (!g_gpu.h) {
        charm_gpu_config_t cfg;
        if ((rc = charm_model_gpu_config(ctx, g_gpu.precision, &cfg))) { plugin_error(rc, "config"); return; }
        if ((rc = charm_gpu_create(&g_gpu.h, &cfg, g_gpu.device))) { plugin_error(rc, "create"); return; }
        g_gpu.mesh_valid = 0;
    }
    if (ctx->refine_period) {
        if (!(ctx->timestep % ctx->refine_period)) {
            if (ctx->timestep) {
                if ((rc = charm_model_gpu_download(p4est))) { plugin_error(rc, "download"); return; }
                charm_adapt(p4est, *_ghost, *_ghost_data);
                if (*_ghost) {
                    p4est_ghost_destroy(*_ghost);
                    CHARM_FREE(*_ghost_data);
                    *_ghost = NULL;
                    *_ghost_data = NULL;
                }
                g_gpu.mesh_valid = 0;
            }
            *dt = ctx->get_dt_fn(p4est);
        }
    } else {
        *dt = ctx->get_dt_fn(p4est);
    }
    if (!(ctx->timestep % ctx->write_period)) {
        if ((rc = charm_model_gpu_download(p4est))) { plugin_error(rc, "download"); return; }
        charm_write_solution(p4est);
    }
    if (!g_gpu.mesh_valid) {
        if ((rc = upload_all(p4est))) { plugin_error(rc, "upload"); return; }
    }
    if ((rc = charm_gpu_step(g_gpu.h, *dt, NULL))) { plugin_error(rc, "step"); return; }
    g_gpu.device_newer = 1;
}

/* The handle and every flattened array, released (the state on the device
 * is not brought back). */
static void release_all(void)
{
    if (g_gpu.h) charm_gpu_destroy(g_gpu.h);
    free(g_gpu.center); free(g_gpu.level); free(g_gpu.face_elem0); free(g_gpu.face_elem1); free(g_gpu.face_all);
    free(g_gpu.face_info); free(g_gpu.bface_elem); free(g_gpu.bface_face); free(g_gpu.bface_bnd); free(g_gpu.state);
    free(g_gpu.vertex); free(g_gpu.hface_elem0); free(g_gpu.hface_elem1); free(g_gpu.hface_all); free(g_gpu.hface_info);
    free(g_gpu.hface_face0); free(g_gpu.hface_face1); free(g_gpu.hface_face_all);
    memset(&g_gpu, 0, sizeof(g_gpu));
}

/* Register the plugin pair in place of the model's (call after
 * charm_init_context_yaml).  precision: CHARM_GPU_PREC_FP64 or _MIXED.  A
 * second call releases what the first one's run held. */
void charm_model_gpu_init(charm_ctx_t *ctx, int precision, int device)
{
    const int model = model_of(ctx);
    release_all();
    g_gpu.model = model;
    g_gpu.precision = precision;
    g_gpu.device = device;
    ctx->timestep_single_fn = charm_model_gpu_timestep_single;
    ctx->get_dt_fn = charm_model_gpu_get_dt;
}

/* Download the final state and release the GPU handle. */
void charm_model_gpu_finalize(p4est_t *p4est)
{
    if (g_gpu.h) charm_model_gpu_download(p4est);
    release_all();
}
