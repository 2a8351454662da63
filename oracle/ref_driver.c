/*
 * Driver for the reference build of the oracle (test infrastructure).
 *
 * Links CHARM_3D's own sources, compiled unmodified, against the p4est
 * shim, and exposes a small C API for the tests: build a case (the context
 * charm_init_context_yaml would build, reference src/charm_init_yaml.cpp:333-413),
 * inject a state, run time steps through ctx->timestep_single_fn exactly as
 * charm_timesteps does (src/charm_timesteps.c:23-51), and read back states,
 * residuals, geometry, the face list and the adapted forest.
 *
 * One case at a time (global state), single thread.
 */
#include "charm_globals.h"
#include "charm_base_func.h"
#include "charm_bnd_cond.h"
#include "charm_eos.h"
#include "charm_fluxes.h"
#include "charm_limiter.h"
#include "charm_models.h"
#include "charm_amr.h"

#include "charm_gpu.h"

/* shim extras (p4est_shim.c) */
p4est_connectivity_t *charm_shim_conn_hex(int32_t n_vert, const double *vert, int32_t n_tree, const int32_t *t2v,
                                          size_t attr_bytes);
p4est_connectivity_t *charm_shim_conn_brick(int nx, int ny, int nz, const int periodic[3], const double origin[3],
                                            const double tree_len[3], size_t attr_bytes);
void charm_shim_conn_destroy(p4est_connectivity_t *c);
p4est_t *p4est_new_ext(int mpicomm, p4est_connectivity_t *conn, p4est_locidx_t min_quadrants, int min_level,
                       int fill_uniform, size_t data_size, p4est_init_t init_fn, void *user_pointer);
void p4est_destroy(p4est_t *p);
int64_t charm_shim_count(p4est_t *p);
p4est_quadrant_t *charm_shim_quad(p4est_t *p, int64_t i);
int32_t charm_shim_tree(p4est_t *p, int64_t i);
extern void (*charm_shim_ghost_shift)(void *data, const double shift[3]);

/* reference functions without a header declaration */
void charm_model_ns_timestep_conv(p4est_t *p4est, p4est_ghost_t *ghost, charm_data_t *ghost_data);

/* The reference's output module is not part of the path: its two entry
 * points become no-ops here (src/charm_output.c:56-132). */
void charm_write_solution(p4est_t *p4est) { (void) p4est; }
void charm_log_statistics(p4est_t *p4est, int timestep, charm_real_t time, charm_real_t dt, charm_real_t calc_time)
{
    (void) p4est; (void) timestep; (void) time; (void) dt; (void) calc_time;
}

static charm_ctx_t g_ctx;
static p4est_connectivity_t *g_conn = NULL;
static p4est_t *g_p4est = NULL;
static p4est_ghost_t *g_ghost = NULL;
static charm_data_t *g_ghost_data = NULL;
static int g_step = 0;
static double g_dt = 0.0;

static void ghost_shift(void *data, const double s[3])
{
    charm_data_t *d = (charm_data_t *) data;
    int i, j, k;
    for (k = 0; k < 3; k++) d->par.g.c[k] += s[k];
    for (i = 0; i < CHARM_FACES; i++) {
        for (k = 0; k < 3; k++) d->par.g.fc[i][k] += s[k];
        for (j = 0; j < CHARM_FACE_GP_COUNT; j++)
            for (k = 0; k < 3; k++) d->par.g.face_gp[i][j][k] += s[k];
    }
    for (j = 0; j < CHARM_QUAD_GP_COUNT; j++)
        for (k = 0; k < 3; k++) d->par.g.quad_gp[j][k] += s[k];
}

static void free_ghost(void)
{
    if (g_ghost) p4est_ghost_destroy(g_ghost);
    free(g_ghost_data);
    g_ghost = NULL;
    g_ghost_data = NULL;
}

static void free_case(void)
{
    size_t i;
    free_ghost();
    if (g_p4est) p4est_destroy(g_p4est);
    g_p4est = NULL;
    if (g_conn) charm_shim_conn_destroy(g_conn);
    g_conn = NULL;
    if (g_ctx.comp) {
        for (i = 0; i < g_ctx.comp->elem_count; i++) sc_array_destroy(((charm_comp_t *) sc_array_index(g_ctx.comp, i))->cp);
        sc_array_destroy(g_ctx.comp);
    }
    if (g_ctx.bnd) {
        for (i = 0; i < g_ctx.bnd->elem_count; i++) free(((charm_bnd_t *) sc_array_index(g_ctx.bnd, i))->params);
        sc_array_destroy(g_ctx.bnd);
    }
    if (g_ctx.mat) sc_array_destroy(g_ctx.mat);
    if (g_ctx.reg) sc_array_destroy(g_ctx.reg);
    if (g_ctx.reactions) sc_array_destroy(g_ctx.reactions);
    free(g_ctx.msh);
    memset(&g_ctx, 0, sizeof(g_ctx));
}

void ref_free(void) { free_case(); }

/* Region used by charm_init_initial_condition for the first fill; the tests
 * overwrite the state with ref_set_state. */
typedef struct ref_region {
    double v[3], t, p;
    double c[CHARM_GPU_MAX_COMP];
} ref_region_t;

/* The context charm_init_context_yaml builds from a case (everything but the
 * mesh). */
static int build_ctx(const charm_gpu_config_t *cfg, const ref_region_t *region, double max_err, int min_level,
                     int max_level, int refine_period)
{
    int i, k;
    free_case();
    charm_ctx_t *ctx = &g_ctx;
    memset(ctx, 0, sizeof(*ctx));
    if (cfg->n_comp < 1 || cfg->n_comp > CHARM_GPU_MAX_COMP) return 1;

    /* components (src/charm_init_yaml.cpp:98-165) */
    ctx->comp = sc_array_new(sizeof(charm_comp_t));
    for (i = 0; i < cfg->n_comp; i++) {
        charm_comp_t *c = (charm_comp_t *) sc_array_push(ctx->comp);
        memset(c, 0, sizeof(*c));
        snprintf(c->name, sizeof(c->name), "C%d", i);
        c->id = i;
        c->m = cfg->comp[i].m;
        c->ml0 = cfg->comp[i].ml0;
        c->kp0 = cfg->comp[i].kp0;
        c->t0 = cfg->comp[i].t0;
        c->ts = cfg->comp[i].ts;
        c->sig = cfg->comp[i].sig;
        c->ek = cfg->comp[i].ek;
        c->h0 = cfg->comp[i].h0;
        c->cp_type = cfg->comp[i].cp_type == CHARM_GPU_CP_POLYNOM ? COMP_CP_POLYNOM : COMP_CP_CONST;
        c->kp_type = cfg->comp[i].kp_type == CHARM_GPU_LAW_SUTHERLAND ? COMP_KP_SATHERLAND : COMP_KP_CONST;
        c->ml_type = cfg->comp[i].ml_type == CHARM_GPU_LAW_SUTHERLAND ? COMP_ML_SATHERLAND : COMP_ML_CONST;
        c->cp = sc_array_new(sizeof(charm_real_t));
        for (k = 0; k < cfg->comp[i].n_cp; k++) *(charm_real_t *) sc_array_push(c->cp) = cfg->comp[i].cp[k];
    }
    /* boundaries (:21-95) */
    ctx->bnd = sc_array_new(sizeof(charm_bnd_t));
    for (i = 0; i < cfg->n_bnd; i++) {
        charm_bnd_t *b = (charm_bnd_t *) sc_array_push(ctx->bnd);
        memset(b, 0, sizeof(*b));
        snprintf(b->name, sizeof(b->name), "B%d", i);
        b->type = (charm_bnd_types_t) cfg->bnd[i].type;
        b->params = (charm_real_t *) calloc(7 + CHARM_GPU_MAX_COMP, sizeof(charm_real_t));
        for (k = 0; k < 7 + CHARM_GPU_MAX_COMP; k++) b->params[k] = cfg->bnd[i].params[k];
        switch (b->type) {
        case BOUND_INLET: b->bnd_fn = charm_bnd_cond_fn_inlet; break;
        case BOUND_OUTLET: b->bnd_fn = charm_bnd_cond_fn_outlet; break;
        case BOUND_WALL_SLIP: b->bnd_fn = charm_bnd_cond_fn_wall_slip; break;
        case BOUND_WALL_NO_SLIP: b->bnd_fn = charm_bnd_cond_fn_wall_no_slip; break;
        case BOUND_MASS_FLOW: b->bnd_fn = charm_bnd_cond_fn_mass_flow; break;
        default: return 2;
        }
    }
    /* material (:168-201) */
    ctx->mat = sc_array_new(sizeof(charm_mat_t));
    {
        charm_mat_t *m = (charm_mat_t *) sc_array_push(ctx->mat);
        memset(m, 0, sizeof(*m));
        m->id = 0;
        snprintf(m->name, sizeof(m->name), "MAT");
        m->eos_fn = cfg->eos == CHARM_GPU_EOS_MIX ? charm_mat_eos_mix : charm_mat_eos_ideal;
    }
    /* region (:203-260) */
    ctx->reg = sc_array_new(sizeof(charm_reg_t));
    {
        charm_reg_t *r = (charm_reg_t *) sc_array_push(ctx->reg);
        memset(r, 0, sizeof(*r));
        r->id = 0;
        r->mat_id = 0;
        for (k = 0; k < 3; k++) { r->v[k] = region->v[k]; r->grav[k] = cfg->grav[k]; }
        r->t = region->t;
        r->p = region->p;
        for (k = 0; k < cfg->n_comp; k++) r->c[k] = region->c[k];
    }
    ctx->msh = (charm_mesh_info_t *) calloc(1, sizeof(charm_mesh_info_t));
    ctx->reactions = NULL;
    if (cfg->n_react > 0) {   /* src/models/ns/charm_model_ns_init.cpp:15-77 */
        ctx->reactions = sc_array_new(sizeof(charm_reaction_t));
        for (i = 0; i < cfg->n_react; i++) {
            charm_reaction_t *r = (charm_reaction_t *) sc_array_push(ctx->reactions);
            for (k = 0; k < 3; k++) { r->left_comps[k] = cfg->react[i].left[k]; r->right_comps[k] = cfg->react[i].right[k]; }
            r->a = cfg->react[i].a;
            r->e = cfg->react[i].e;
            r->n = cfg->react[i].n;
        }
    }
    /* control (:352-413) */
    switch (cfg->flux) {
    case CHARM_GPU_FLUX_LF: ctx->flux_fn = charm_calc_flux_lf; break;
    case CHARM_GPU_FLUX_GODUNOV: ctx->flux_fn = charm_calc_flux_godunov; break;
    case CHARM_GPU_FLUX_HLLC: ctx->flux_fn = charm_calc_flux_hllc; break;
    default: ctx->flux_fn = charm_calc_flux_cd; break;
    }
    ctx->lim_fn = cfg->limiter == CHARM_GPU_LIM_BJ ? charm_limiter_bj : NULL;
    ctx->max_err = max_err;
    ctx->refine_period = refine_period;
    ctx->repartition_period = 0;
    ctx->min_level = min_level;
    ctx->max_level = max_level;
    ctx->write_period = 1 << 30;
    ctx->log_period = 1 << 30;
    ctx->dt = cfg->tau;
    ctx->CFL = cfg->cfl;
    ctx->time = 1.0e300;
    ctx->model.ns.use_visc = cfg->use_visc;
    ctx->model.ns.use_diff = cfg->use_diff;
    ctx->model.ns.t_ref = cfg->t_ref;
    if (cfg->model == CHARM_GPU_MODEL_EULER) {
        ctx->get_dt_fn = charm_model_euler_get_dt;
        ctx->timestep_single_fn = charm_model_euler_timestep_single;
    } else {
        ctx->get_dt_fn = charm_model_ns_get_dt;
        ctx->timestep_single_fn = charm_model_ns_timestep_single;
    }
    ctx->timestep = 0;
    return 0;
}

int ref_setup(const charm_gpu_config_t *cfg, const int32_t brick[3], const int32_t periodic[3],
              const double origin[3], const double tree_len[3], int level, const int8_t bnd_of_side[6],
              const ref_region_t *region, double max_err, int min_level, int max_level, int refine_period)
{
    int i, k;
    int rc = build_ctx(cfg, region, max_err, min_level, max_level, refine_period);
    if (rc) return rc;
    charm_ctx_t *ctx = &g_ctx;
    /* mesh: brick of trees with boundary attributes on the domain sides */
    g_conn = charm_shim_conn_brick(brick[0], brick[1], brick[2], (const int *) periodic, origin, tree_len,
                                   sizeof(charm_tree_attr_t));
    for (k = 0; k < brick[2]; k++)
        for (int j = 0; j < brick[1]; j++)
            for (i = 0; i < brick[0]; i++) {
                int t = i + brick[0] * (j + brick[1] * k);
                charm_tree_attr_t *a = (charm_tree_attr_t *) &g_conn->tree_to_attr[sizeof(charm_tree_attr_t) * t];
                int idx[3] = {i, j, k};
                for (int f = 0; f < 6; f++) {
                    int d = f / 2, up = f & 1;
                    int edge = up ? (idx[d] == brick[d] - 1) : (idx[d] == 0);
                    a->bnd[f] = (edge && !periodic[d]) ? (charm_bnd_t *) sc_array_index(ctx->bnd, bnd_of_side[f]) : NULL;
                }
                a->reg = (charm_reg_t *) sc_array_index(ctx->reg, 0);
            }
    charm_shim_ghost_shift = ghost_shift;
    g_p4est = p4est_new_ext(0, g_conn, 0, level, 1, sizeof(charm_data_t), charm_init_initial_condition, ctx);
    charm_set_p4est(g_p4est);
    g_step = 0;
    g_dt = 0.0;
    return 0;
}

/* The case on an unstructured hexahedral mesh (the connectivity that
 * charm_conn_reader_msh builds, src/charm_connectivity.c:315-519): n_tree
 * hexahedra with corner vertices in p4est order, tree_bnd [6 n_tree] the
 * boundary of every tree face without a neighbour (-1 elsewhere). */
int ref_setup_hex(const charm_gpu_config_t *cfg, int32_t n_vert, const double *vert, int32_t n_tree,
                  const int32_t *t2v, const int8_t *tree_bnd, int level, const ref_region_t *region, double max_err,
                  int min_level, int max_level, int refine_period)
{
    int rc = build_ctx(cfg, region, max_err, min_level, max_level, refine_period);
    if (rc) return rc;
    charm_ctx_t *ctx = &g_ctx;
    g_conn = charm_shim_conn_hex(n_vert, vert, n_tree, t2v, sizeof(charm_tree_attr_t));
    if (!g_conn) return 3;
    for (int t = 0; t < n_tree; t++) {
        charm_tree_attr_t *a = (charm_tree_attr_t *) &g_conn->tree_to_attr[sizeof(charm_tree_attr_t) * t];
        for (int f = 0; f < 6; f++) {
            const int b = tree_bnd[6 * t + f];
            a->bnd[f] = (b >= 0) ? (charm_bnd_t *) sc_array_index(ctx->bnd, (size_t) b) : NULL;
        }
        a->reg = (charm_reg_t *) sc_array_index(ctx->reg, 0);
    }
    charm_shim_ghost_shift = ghost_shift;
    g_p4est = p4est_new_ext(0, g_conn, 0, level, 1, sizeof(charm_data_t), charm_init_initial_condition, ctx);
    charm_set_p4est(g_p4est);
    g_step = 0;
    g_dt = 0.0;
    return 0;
}

int64_t ref_count(void) { return g_p4est ? charm_shim_count(g_p4est) : -1; }

static int n_comp(void) { return (int) g_ctx.comp->elem_count; }

int ref_set_state(const double *u)
{
    int64_t E = charm_shim_count(g_p4est), i;
    int nc = n_comp(), k, j;
    const int B = CHARM_BASE_FN_COUNT;
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        memset(&d->par.c, 0, sizeof(d->par.c));
        /* model fields start at zero, as after the initial fill: with fewer
         * than 2 species the diffusion coefficients are never written
         * (src/models/ns/charm_model_ns_diff.c:74-76), and leaves made by
         * refinement would otherwise keep whatever their memory held */
        memset(&d->par.model.ns, 0, sizeof(d->par.model.ns));
        for (k = 0; k < B; k++) {
            d->par.c.ru[k] = u[(0 * B + k) * E + i];
            d->par.c.rv[k] = u[(1 * B + k) * E + i];
            d->par.c.rw[k] = u[(2 * B + k) * E + i];
            d->par.c.re[k] = u[(3 * B + k) * E + i];
            for (j = 0; j < nc; j++) d->par.c.rc[j][k] = u[((4 + j) * B + k) * E + i];
        }
    }
    free_ghost();
    return 0;
}

int ref_get_state(double *u)
{
    int64_t E = charm_shim_count(g_p4est), i;
    int nc = n_comp(), k, j;
    const int B = CHARM_BASE_FN_COUNT;
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        for (k = 0; k < B; k++) {
            u[(0 * B + k) * E + i] = d->par.c.ru[k];
            u[(1 * B + k) * E + i] = d->par.c.rv[k];
            u[(2 * B + k) * E + i] = d->par.c.rw[k];
            u[(3 * B + k) * E + i] = d->par.c.re[k];
            for (j = 0; j < nc; j++) u[((4 + j) * B + k) * E + i] = d->par.c.rc[j][k];
        }
    }
    return 0;
}

/* The cell-centre fields the reference's output writes per cell
 * (charm_interpolate_cell_solution, src/charm_output.c:10-52): the same two
 * calls, charm_get_fields at the centre and charm_param_cons_to_prim, for
 * every leaf; out[f * E + e] for R, P, E, E_TOT, U, V, W, T, then C_i. */
int ref_cell_fields(double *out)
{
    int64_t E = charm_shim_count(g_p4est), i;
    int nc = n_comp(), j;
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        charm_cons_t cons;
        charm_prim_t prim;
        charm_get_fields(d, d->par.g.c, &cons);
        charm_param_cons_to_prim(g_p4est, &prim, &cons);
        const double f[8] = {prim.r, prim.p, prim.e, prim.e_tot, prim.u, prim.v, prim.w, prim.t};
        for (j = 0; j < 8; j++) out[j * E + i] = f[j];
        for (j = 0; j < nc; j++) out[(8 + j) * E + i] = prim.c[j];
    }
    return 0;
}

static void ensure_ghost(void)
{
    if (!g_ghost) {
        g_ghost = p4est_ghost_new(g_p4est, CHARM_CONNECT_FULL);
        g_ghost_data = CHARM_ALLOC(charm_data_t, g_ghost->ghosts.elem_count);
    }
    p4est_ghost_exchange_data(g_p4est, g_ghost, g_ghost_data);
}

/* nsteps of the time loop of charm_timesteps (src/charm_timesteps.c:32-47). */
int ref_run(int nsteps, double *dt_out)
{
    int s;
    ensure_ghost();
    g_dt = g_ctx.get_dt_fn(g_p4est);
    for (s = 0; s < nsteps; s++) {
        g_ctx.timestep = g_step;
        g_ctx.timestep_single_fn(g_p4est, &g_dt, &g_ghost, &g_ghost_data);
        g_ctx.t += g_dt;
        g_step++;
    }
    if (dt_out) *dt_out = g_dt;
    return 0;
}

/* Residual int_* of the current state (zero + volume/face integrals,
 * src/models/ns/charm_model.c:248-252). */
void charm_model_ns_timestep_diff(p4est_t *p4est, p4est_ghost_t *ghost, charm_data_t *ghost_data);

int ref_residual(double *res)
{
    int64_t E = charm_shim_count(g_p4est), i;
    int nc = n_comp(), k, j;
    const int B = CHARM_BASE_FN_COUNT;
    ensure_ghost();
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        memset(d->int_ru, 0, sizeof(d->int_ru));
        memset(d->int_rv, 0, sizeof(d->int_rv));
        memset(d->int_rw, 0, sizeof(d->int_rw));
        memset(d->int_re, 0, sizeof(d->int_re));
        memset(d->int_rc, 0, sizeof(d->int_rc));
        d->par.model.ns.chem_rhs = 0.;
    }
    p4est_ghost_exchange_data(g_p4est, g_ghost, g_ghost_data);
    /* the order of charm_model_ns_timestep_single's stage (src/models/ns/charm_model.c:248-251) */
    charm_model_ns_timestep_diff(g_p4est, g_ghost, g_ghost_data);
    charm_model_ns_timestep_conv(g_p4est, g_ghost, g_ghost_data);
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        for (k = 0; k < B; k++) {
            res[(0 * B + k) * E + i] = d->int_ru[k];
            res[(1 * B + k) * E + i] = d->int_rv[k];
            res[(2 * B + k) * E + i] = d->int_rw[k];
            res[(3 * B + k) * E + i] = d->int_re[k];
            for (j = 0; j < nc; j++) res[((4 + j) * B + k) * E + i] = d->int_rc[j][k];
        }
    }
    return 0;
}

/* One limiter pass (src/limiters/charm_limiter.c:9-15). */
int ref_limit(void)
{
    ensure_ghost();
    charm_limiter(g_p4est, g_ghost, g_ghost_data);
    return 0;
}

/* Geometry per element: c[3] dh[3] volume a_inv[16] area[6] -> 29 doubles. */
int ref_geometry(double *out)
{
    int64_t E = charm_shim_count(g_p4est), i;
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        double *o = out + 29 * i;
        int k, j;
        for (k = 0; k < 3; k++) { o[k] = d->par.g.c[k]; o[3 + k] = d->par.g.dh[k]; }
        o[6] = d->par.g.volume;
        for (k = 0; k < 4; k++)
            for (j = 0; j < 4; j++) o[7 + 4 * k + j] = d->par.g.a_inv[k][j];
        for (k = 0; k < 6; k++) o[23 + k] = d->par.g.area[k];
    }
    return 0;
}

/* Face list as the reference's face callbacks see it: per face
 * (nsides, side0 face, side0 hanging, 4 ids, side1 face, side1 hanging, 4 ids)
 * = 13 int64; ghost quadrants appear as -1 - (source leaf index). */
typedef struct { int64_t *buf; int64_t n, cap; } face_acc_t;

static int64_t quad_index(p4est_quadrant_t *q, int is_ghost)
{
    if (is_ghost) {
        /* ghosts are copies; identify by coordinates among the leaves */
        int64_t E = charm_shim_count(g_p4est), i;
        for (i = 0; i < E; i++) {
            p4est_quadrant_t *r = charm_shim_quad(g_p4est, i);
            if (r->x == q->x && r->y == q->y && r->z == q->z && r->level == q->level) {
                /* tree must match too: ghosts keep their tree coordinates */
                return -1 - i;
            }
        }
        return -1000000000;
    }
    return (int64_t) (q - charm_shim_quad(g_p4est, 0));
}

static void face_rec_fn(p4est_iter_face_info_t *info, void *user)
{
    face_acc_t *acc = (face_acc_t *) user;
    if (acc->n + 13 > acc->cap) {
        acc->cap = acc->cap ? 2 * acc->cap : 1024;
        acc->buf = (int64_t *) realloc(acc->buf, sizeof(int64_t) * (size_t) acc->cap);
    }
    int64_t *r = acc->buf + acc->n;
    int ns = (int) info->sides.elem_count, s, k;
    for (k = 0; k < 13; k++) r[k] = -2;
    r[0] = ns;
    for (s = 0; s < ns; s++) {
        p4est_iter_face_side_t *sd = p4est_iter_fside_array_index_int(&info->sides, s);
        r[1 + 6 * s] = sd->face;
        r[2 + 6 * s] = sd->is_hanging;
        if (sd->is_hanging)
            for (k = 0; k < 4; k++) r[3 + 6 * s + k] = quad_index(sd->is.hanging.quad[k], sd->is.hanging.is_ghost[k]);
        else
            r[3 + 6 * s] = quad_index(sd->is.full.quad, sd->is.full.is_ghost);
    }
    acc->n += 13;
}

static face_acc_t g_faces;

int64_t ref_faces_count(void)
{
    free(g_faces.buf);
    memset(&g_faces, 0, sizeof(g_faces));
    ensure_ghost();
    p4est_iterate(g_p4est, g_ghost, &g_faces, NULL, face_rec_fn, NULL, NULL);
    return g_faces.n / 13;
}

int ref_faces_copy(int64_t *out)
{
    memcpy(out, g_faces.buf, sizeof(int64_t) * (size_t) g_faces.n);
    return 0;
}

/* Leaves of the current forest: x y z tree level per leaf. */
int ref_leaves(int32_t *out)
{
    int64_t E = charm_shim_count(g_p4est), i;
    for (i = 0; i < E; i++) {
        p4est_quadrant_t *q = charm_shim_quad(g_p4est, i);
        out[5 * i + 0] = q->x; out[5 * i + 1] = q->y; out[5 * i + 2] = q->z;
        out[5 * i + 3] = charm_shim_tree(g_p4est, i);
        out[5 * i + 4] = q->level;
    }
    return 0;
}

/* One adapt of the reference (src/charm_amr.c:575-610), then a fresh ghost
 * layer as the models do after adapting. */
int64_t ref_adapt(void)
{
    ensure_ghost();
    charm_adapt(g_p4est, g_ghost, g_ghost_data);
    free_ghost();
    return charm_shim_count(g_p4est);
}

/* Density-gradient estimate grad_u[3] left by the last adapt's indicator pass
 * for leaves that survived it unchanged (NaN for new leaves). */
int ref_grad(double *out)
{
    int64_t E = charm_shim_count(g_p4est), i;
    for (i = 0; i < E; i++) {
        charm_data_t *d = (charm_data_t *) charm_shim_quad(g_p4est, i)->p.user_data;
        out[3 * i + 0] = d->par.a.grad_u[0];
        out[3 * i + 1] = d->par.a.grad_u[1];
        out[3 * i + 2] = d->par.a.grad_u[2];
    }
    return 0;
}

/* Direct calls into the reference's flux functions for point tests:
 * prim = 2 x (r u v w p) for a single-species ideal gas of the current case. */
/* The reference's exact Riemann solver rim_orig (src/charm_fluxes.c:8-180)
 * on n inputs (rL pL uL vL wL rR pR uR vR wR gam each) -> (r e p u v w). */
int ref_rim(int64_t n, const double *in, double *out)
{
    int64_t i;
    for (i = 0; i < n; i++) {
        const double *a = in + 11 * i;
        double *o = out + 6 * i;
        rim_orig(&o[0], &o[1], &o[2], &o[3], &o[4], &o[5], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9],
                 a[10]);
    }
    return 0;
}

int ref_point_flux(const double *prim2, const double n[3], double *q)
{
    charm_prim_t pr[2];
    int s, i;
    int nc = n_comp();
    memset(pr, 0, sizeof(pr));
    for (s = 0; s < 2; s++) {
        charm_cons_t c;
        charm_prim_t p;
        memset(&c, 0, sizeof(c));
        memset(&p, 0, sizeof(p));
        p.mat_id = 0;
        p.r = prim2[5 * s + 0];
        p.u = prim2[5 * s + 1];
        p.v = prim2[5 * s + 2];
        p.w = prim2[5 * s + 3];
        p.p = prim2[5 * s + 4];
        for (i = 0; i < nc; i++) p.c[i] = (i == 0) ? 1.0 : 0.0;
        /* e from (r,p) with the case's EOS: flag 1 */
        charm_mat_t *m = charm_mat_find_by_id(&g_ctx, 0);
        m->eos_fn(g_p4est, &p, 1);
        p.e_tot = p.e + 0.5 * (p.u * p.u + p.v * p.v + p.w * p.w);
        /* round-trip through conserved variables as the path does */
        charm_param_prim_to_cons(g_p4est, &c, &p);
        c.mat_id = 0;
        charm_param_cons_to_prim(g_p4est, &pr[s], &c);
    }
    double nn[3] = {n[0], n[1], n[2]};
    g_ctx.flux_fn(g_p4est, pr, &q[0], &q[1], &q[2], &q[3], &q[4], nn);
    return 0;
}

int ref_step_count(void) { return g_step; }

/* Refine the leaves with flags[i] > 0 (one level, not above maxlevel) and
 * 2:1-balance, initialising new leaves with the reference's own
 * charm_init_initial_condition (geometry + region state).  Used to build
 * meshes with hanging faces for the tests. */
static const int8_t *g_refine_flags = NULL;

static int refine_by_flag(p4est_t *p, p4est_topidx_t t, p4est_quadrant_t *q)
{
    (void) t;
    return g_refine_flags[q - charm_shim_quad(p, 0)] > 0;
}

int64_t ref_refine_flags(const int8_t *flags, int maxlevel)
{
    g_refine_flags = flags;
    p4est_refine_ext(g_p4est, 0, maxlevel, refine_by_flag, charm_init_initial_condition, NULL);
    p4est_balance_ext(g_p4est, P4EST_CONNECT_FACE, charm_init_initial_condition, NULL);
    g_refine_flags = NULL;
    free_ghost();
    return charm_shim_count(g_p4est);
}

p4est_t *ref_driver_p4est(void) { return g_p4est; }
