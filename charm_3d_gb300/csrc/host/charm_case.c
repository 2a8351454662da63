/*
 * charm_case.c - CHARM_3D's case file (task.yaml) into the solver's
 * configuration: the part of charm_init_context_yaml (reference
 * src/charm_init_yaml.cpp:333-428) and of the model initialisers
 * (src/models/ns/charm_model_ns_init.cpp:14-89,
 * src/models/euler/charm_model_euler_init.cpp:14-18) that the time step
 * reads, with the same keys, the same names for the plugin choices and the
 * same checks.  Errors return CHARM_GPU_EINVAL (or ENOTSUP for a choice the
 * GPU path does not build) with the message in charm_gpu_last_error(); the
 * reference prints and exits instead.
 */
#include "charm_gpu.h"
#include "charm_yaml.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void charm_internal_set_error(const char *msg);

static int case_fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    charm_internal_set_error(buf);
    return code;
}

/* version a.b.c >= the reader's 0.1.1 (YAML_VERSION, reference
 * include/charm_version.h:9; check as _charm_init_yaml_check_version) */
static int version_ok(const char *v)
{
    int a[3], n = 0;
    const char *s = v;
    while (n < 3) {
        char *end = NULL;
        long x = strtol(s, &end, 10);
        if (end == s) return 0;
        a[n++] = (int) x;
        if (*end == '.') s = end + 1;
        else { s = end; break; }
    }
    if (n != 3 || *s) return 0;
    const int c[3] = {0, 1, 1};
    for (int i = 0; i < 3; i++) {
        if (a[i] > c[i]) return 1;
        if (a[i] < c[i]) return 0;
    }
    return 1;
}

#define REQ_D(node, key, dst)                                                                              \
    do {                                                                                                   \
        if (charm_yaml_double(charm_yaml_get((node), (key)), &(dst)))                                     \
            return case_fail(CHARM_GPU_EINVAL, "task.yaml: '%s' missing or not a number (%s)", (key), where); \
    } while (0)
#define REQ_I(node, key, dst)                                                                              \
    do {                                                                                                   \
        if (charm_yaml_int(charm_yaml_get((node), (key)), &(dst)))                                        \
            return case_fail(CHARM_GPU_EINVAL, "task.yaml: '%s' missing or not an integer (%s)", (key), where); \
    } while (0)
#define REQ_S(node, key, dst)                                                                              \
    do {                                                                                                   \
        (dst) = charm_yaml_str(charm_yaml_get((node), (key)));                                             \
        if (!(dst) || !(dst)[0])                                                                           \
            return case_fail(CHARM_GPU_EINVAL, "task.yaml: '%s' missing (%s)", (key), where);              \
    } while (0)

static void copy_name(char *dst, size_t cap, const char *src)
{
    snprintf(dst, cap, "%s", src ? src : "");
}

/* x, y, z of a {x: .., y: .., z: ..} map */
static int vec3(const charm_ynode_t *n, double v[3], const char *key, const char *where)
{
    const char *axes[3] = {"x", "y", "z"};
    if (!n || n->type != CHARM_Y_MAP) return case_fail(CHARM_GPU_EINVAL, "task.yaml: '%s' must be {x, y, z} (%s)", key, where);
    for (int d = 0; d < 3; d++)
        if (charm_yaml_double(charm_yaml_get(n, axes[d]), &v[d]))
            return case_fail(CHARM_GPU_EINVAL, "task.yaml: '%s.%s' missing (%s)", key, axes[d], where);
    return CHARM_GPU_OK;
}

/* components (_charm_init_fetch_comp, src/charm_init_yaml.cpp:101-159) */
static int read_comps(const charm_ynode_t *list, charm_case_t *cs)
{
    const char *where = "components";
    if (!list || list->type != CHARM_Y_SEQ || list->n < 1)
        return case_fail(CHARM_GPU_EINVAL, "task.yaml: 'components' must be a non-empty list");
    if (list->n > CHARM_GPU_MAX_COMP)
        return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: %d components, at most %d", list->n, CHARM_GPU_MAX_COMP);
    cs->cfg.n_comp = list->n;
    for (int i = 0; i < list->n; i++) {
        const charm_ynode_t *c = list->items[i];
        charm_gpu_comp_t *k = &cs->cfg.comp[i];
        const char *s;
        REQ_I(c, "id", cs->comp_id[i]);
        REQ_S(c, "name", s);
        copy_name(cs->comp_name[i], sizeof(cs->comp_name[i]), s);
        REQ_S(c, "cp_type", s);
        if (!strcmp(s, "CONST")) k->cp_type = CHARM_GPU_CP_CONST;
        else if (!strcmp(s, "POLYNOM")) k->cp_type = CHARM_GPU_CP_POLYNOM;
        else return case_fail(CHARM_GPU_EINVAL, "Unknown Cp type '%s'. Use: CONST, POLYNOM.", s);
        REQ_S(c, "kp_type", s);
        if (!strcmp(s, "CONST")) k->kp_type = CHARM_GPU_LAW_CONST;
        else if (!strcmp(s, "SATHERLAND")) k->kp_type = CHARM_GPU_LAW_SUTHERLAND;
        else return case_fail(CHARM_GPU_EINVAL, "Unknown KP type '%s'. Use: CONST, SATHERLAND.", s);
        REQ_S(c, "ml_type", s);
        if (!strcmp(s, "CONST")) k->ml_type = CHARM_GPU_LAW_CONST;
        else if (!strcmp(s, "SATHERLAND")) k->ml_type = CHARM_GPU_LAW_SUTHERLAND;
        else return case_fail(CHARM_GPU_EINVAL, "Unknown ML type '%s'. Use: CONST, SATHERLAND.", s);
        REQ_D(c, "M", k->m);
        REQ_D(c, "ML0", k->ml0);
        REQ_D(c, "KP0", k->kp0);
        REQ_D(c, "T0", k->t0);
        REQ_D(c, "TS", k->ts);
        REQ_D(c, "Sig", k->sig);
        REQ_D(c, "ek", k->ek);
        REQ_D(c, "h0", k->h0);
        const charm_ynode_t *cp = charm_yaml_get(c, "Cp");
        if (!cp || cp->type != CHARM_Y_SEQ || cp->n < 1)
            return case_fail(CHARM_GPU_EINVAL, "task.yaml: component '%s': 'Cp' must be a non-empty list", cs->comp_name[i]);
        if (cp->n > CHARM_GPU_MAX_CP)
            return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: component '%s': more than %d Cp coefficients",
                             cs->comp_name[i], CHARM_GPU_MAX_CP);
        k->n_cp = cp->n;
        for (int j = 0; j < cp->n; j++)
            if (charm_yaml_double(cp->items[j], &k->cp[j]))
                return case_fail(CHARM_GPU_EINVAL, "task.yaml: component '%s': Cp[%d] is not a number", cs->comp_name[i], j);
    }
    return CHARM_GPU_OK;
}

/* boundaries (_charm_init_fetch_bnd, src/charm_init_yaml.cpp:22-99); the
 * type names of charm_bnd_type_by_name (src/charm_globals.c:14-20) */
static int read_bnds(const charm_ynode_t *list, charm_case_t *cs)
{
    static const char *types[] = {"BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_NO_SLIP",
                                  "BOUND_MASS_FLOW"};
    const char *where = "boundaries";
    if (!list || list->type != CHARM_Y_SEQ) return case_fail(CHARM_GPU_EINVAL, "task.yaml: 'boundaries' must be a list");
    if (list->n > CHARM_GPU_MAX_BND)
        return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: %d boundaries, at most %d", list->n, CHARM_GPU_MAX_BND);
    cs->cfg.n_bnd = list->n;
    for (int b = 0; b < list->n; b++) {
        const charm_ynode_t *n = list->items[b];
        charm_gpu_bnd_t *bd = &cs->cfg.bnd[b];
        const char *s;
        REQ_S(n, "name", s);
        copy_name(cs->bnd_name[b], sizeof(cs->bnd_name[b]), s);
        REQ_S(n, "type", s);
        bd->type = -1;
        for (int t = 0; t < 5; t++)
            if (!strcmp(s, types[t])) bd->type = t;
        if (bd->type < 0) return case_fail(CHARM_GPU_EINVAL, "task.yaml: unknown boundary type '%s' of '%s'", s, cs->bnd_name[b]);
        const charm_ynode_t *par = charm_yaml_get(n, "parameters");
        where = cs->bnd_name[b];
        switch (bd->type) {
        case CHARM_GPU_BND_INLET: {
            double v[3];
            int rc = vec3(charm_yaml_get(par, "V"), v, "V", where);
            if (rc) return rc;
            bd->params[0] = v[0]; bd->params[1] = v[1]; bd->params[2] = v[2];
            REQ_D(par, "T", bd->params[3]);
            REQ_D(par, "P", bd->params[4]);
            break;
        }
        case CHARM_GPU_BND_WALL_NO_SLIP:
            REQ_D(par, "T", bd->params[0]);
            break;
        case CHARM_GPU_BND_MASS_FLOW: {
            REQ_D(par, "M", bd->params[0]);
            REQ_D(par, "P", bd->params[1]);
            REQ_D(par, "T", bd->params[2]);
            REQ_D(par, "CosX", bd->params[3]);
            REQ_D(par, "CosY", bd->params[4]);
            REQ_D(par, "CosZ", bd->params[5]);
            bd->params[6] = bd->params[1];   /* the stored static pressure starts at P */
            const charm_ynode_t *cc = charm_yaml_get(par, "components");
            const int nc = (cc && cc->type == CHARM_Y_SEQ) ? cc->n : 0;
            if (nc > cs->cfg.n_comp)
                return case_fail(CHARM_GPU_EINVAL, "BOUND_MASS_FLOW: Too many components specified. Must be %d", cs->cfg.n_comp);
            if (nc < cs->cfg.n_comp)
                return case_fail(CHARM_GPU_EINVAL, "BOUND_MASS_FLOW: Too few components specified. Must be %d", cs->cfg.n_comp);
            for (int i = 0; i < nc; i++)
                if (charm_yaml_double(cc->items[i], &bd->params[7 + i]))
                    return case_fail(CHARM_GPU_EINVAL, "BOUND_MASS_FLOW: component %d is not a number (%s)", i, where);
            break;
        }
        default:   /* outlet, slip wall: no parameters */
            break;
        }
        where = "boundaries";
    }
    return CHARM_GPU_OK;
}

/* materials: the EOS of material 0 (_charm_init_fetch_mat, :179-203) */
static int read_mats(const charm_ynode_t *list, charm_case_t *cs)
{
    const char *where = "materials";
    if (!list || list->type != CHARM_Y_SEQ || list->n < 1)
        return case_fail(CHARM_GPU_EINVAL, "task.yaml: 'materials' must be a non-empty list");
    for (int i = 0; i < list->n; i++) {
        const char *s;
        int id;
        REQ_I(list->items[i], "id", id);
        REQ_S(list->items[i], "name", s);
        REQ_S(list->items[i], "eof_type", s);
        int eos;
        if (!strcmp(s, "IDEAL")) eos = CHARM_GPU_EOS_IDEAL;
        else if (!strcmp(s, "MIX")) eos = CHARM_GPU_EOS_MIX;
        else if (!strcmp(s, "TABLE")) return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: the TABLE EOS is not built on the GPU");
        else return case_fail(CHARM_GPU_EINVAL, "task.yaml: unknown EOS type '%s'. Use: IDEAL, MIX.", s);
        if (i == 0) cs->cfg.eos = eos;
        else if (eos != cs->cfg.eos)
            return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: materials with different EOS (one material on the GPU)");
    }
    return CHARM_GPU_OK;
}

/* regions (_charm_init_fetch_reg, :214-263) */
static int read_regs(const charm_ynode_t *list, charm_case_t *cs)
{
    const char *where = "regions";
    if (!list || list->type != CHARM_Y_SEQ || list->n < 1)
        return case_fail(CHARM_GPU_EINVAL, "task.yaml: 'regions' must be a non-empty list");
    if (list->n > CHARM_CASE_MAX_REG) return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: more than %d regions", CHARM_CASE_MAX_REG);
    cs->n_reg = list->n;
    for (int r = 0; r < list->n; r++) {
        const charm_ynode_t *n = list->items[r];
        charm_case_region_t *rg = &cs->reg[r];
        const char *s;
        REQ_I(n, "id", rg->id);
        REQ_S(n, "name", s);
        copy_name(rg->name, sizeof(rg->name), s);
        REQ_I(n, "material_id", rg->material_id);
        const charm_ynode_t *par = charm_yaml_get(n, "parameters");
        where = rg->name;
        int rc = vec3(charm_yaml_get(par, "V"), rg->v, "V", where);
        if (rc) return rc;
        REQ_D(par, "T", rg->t);
        REQ_D(par, "P", rg->p);
        if ((rc = vec3(charm_yaml_get(par, "G"), rg->grav, "G", where))) return rc;
        const charm_ynode_t *cc = charm_yaml_get(n, "components");
        if (cc && cc->type != CHARM_Y_SEQ) return case_fail(CHARM_GPU_EINVAL, "task.yaml: region '%s': 'components' must be a list", rg->name);
        double sum = 0.0;
        for (int i = 0; cc && i < cc->n; i++) {
            int id;
            double c;
            REQ_I(cc->items[i], "id", id);
            REQ_D(cc->items[i], "concentration", c);
            int idx = -1;
            for (int k = 0; k < cs->cfg.n_comp; k++)
                if (cs->comp_id[k] == id) idx = k;
            if (idx < 0) return case_fail(CHARM_GPU_EINVAL, "Unknown component id %d for region '%s' in file 'task.yaml'", id, rg->name);
            rg->c[idx] = c;
        }
        for (int k = 0; k < cs->cfg.n_comp; k++) sum += rg->c[k];
        /* the reference's test (src/charm_init_yaml.cpp:249) */
        if (fabs(sum) - 1.0 > 1.e-12)
            return case_fail(CHARM_GPU_EINVAL, "Sum of concentrations for region '%s' is not equal to 1 in file 'task.yaml'", rg->name);
        where = "regions";
    }
    /* the GPU path takes one gravity vector for the mesh (charm_gpu_config_t.grav) */
    for (int r = 1; r < cs->n_reg; r++)
        for (int d = 0; d < 3; d++)
            if (cs->reg[r].grav[d] != cs->reg[0].grav[d])
                return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: regions with different gravity (one vector on the GPU)");
    for (int d = 0; d < 3; d++) cs->cfg.grav[d] = cs->reg[0].grav[d];
    return CHARM_GPU_OK;
}

/* reactions of the NS model (_charm_model_ns_chem_init_fetch_reaction, charm_model_ns_init.cpp:14-57) */
static int read_reactions(const charm_ynode_t *list, charm_case_t *cs)
{
    const char *where = "reactions";
    if (!list) return CHARM_GPU_OK;
    if (list->type != CHARM_Y_SEQ) return case_fail(CHARM_GPU_EINVAL, "task.yaml: 'reactions' must be a list");
    if (list->n > CHARM_GPU_MAX_REACT) return case_fail(CHARM_GPU_ENOTSUP, "task.yaml: more than %d reactions", CHARM_GPU_MAX_REACT);
    cs->cfg.n_react = list->n;
    for (int r = 0; r < list->n; r++) {
        const charm_ynode_t *n = list->items[r];
        charm_gpu_reaction_t *re = &cs->cfg.react[r];
        REQ_D(n, "a", re->a);
        REQ_D(n, "e", re->e);
        REQ_D(n, "n", re->n);
        const char *side[2] = {"left", "right"};
        for (int s = 0; s < 2; s++) {
            int32_t *dst = s ? re->right : re->left;
            for (int k = 0; k < 3; k++) dst[k] = -1;
            const charm_ynode_t *l = charm_yaml_get(n, side[s]);
            if (l && l->type != CHARM_Y_SEQ) return case_fail(CHARM_GPU_EINVAL, "task.yaml: reaction %d: '%s' must be a list", r, side[s]);
            for (int k = 0; l && k < l->n; k++) {
                int comp;
                if (k >= 3) return case_fail(CHARM_GPU_EINVAL, "More than 3 components in reaction!");
                if (charm_yaml_int(l->items[k], &comp))
                    return case_fail(CHARM_GPU_EINVAL, "task.yaml: reaction %d: component index is not an integer", r);
                if (!(-1 <= comp && comp < cs->cfg.n_comp))
                    return case_fail(CHARM_GPU_EINVAL, "Wrong component number in reaction: %d, but total components count: %d",
                                     comp, cs->cfg.n_comp);
                dst[k] = comp;
            }
        }
    }
    return CHARM_GPU_OK;
}

static int read_case(const charm_ynode_t *root, charm_case_t *cs)
{
    const char *where = "top level", *s;
    memset(cs, 0, sizeof(*cs));
    cs->cfg.p_order = 1;
    cs->cfg.precision = CHARM_GPU_PREC_FP64;
    cs->cfg.dt_mode = CHARM_GPU_DT_TAU;   /* the reference's get_dt returns TAU */
    if (!root || root->type != CHARM_Y_MAP) return case_fail(CHARM_GPU_EINVAL, "task.yaml: the document must be a mapping");
    REQ_S(root, "method", s);
    if (strcmp(s, "CHARM_3D")) return case_fail(CHARM_GPU_EINVAL, "Method name must be 'CHARM_3D'");
    REQ_S(root, "version", s);
    if (!version_ok(s)) return case_fail(CHARM_GPU_EINVAL, "Wrong YAML version. Must be 0.1.1 or higher.");

    const charm_ynode_t *control = charm_yaml_get(root, "control");
    where = "control";
    if (!control || control->type != CHARM_Y_MAP) return case_fail(CHARM_GPU_EINVAL, "task.yaml: 'control' missing");
    REQ_S(control, "FLUX_TYPE", s);
    if (!strcmp(s, "LF")) cs->cfg.flux = CHARM_GPU_FLUX_LF;
    else if (!strcmp(s, "GODUNOV")) cs->cfg.flux = CHARM_GPU_FLUX_GODUNOV;
    else if (!strcmp(s, "HLLC")) cs->cfg.flux = CHARM_GPU_FLUX_HLLC;
    else if (!strcmp(s, "CD")) cs->cfg.flux = CHARM_GPU_FLUX_CD;
    else return case_fail(CHARM_GPU_EINVAL, "Unknown flux type '%s'. Use: LF, GODUNOV, HLLC, CD.", s);
    REQ_S(control, "LIMITER", s);
    if (!strcmp(s, "NONE")) cs->cfg.limiter = CHARM_GPU_LIM_NONE;
    else if (!strcmp(s, "BJ")) cs->cfg.limiter = CHARM_GPU_LIM_BJ;
    else return case_fail(CHARM_GPU_EINVAL, "Unknown limiter type '%s'. Use: NONE, BJ.", s);
    REQ_D(control, "MAX_ERROR", cs->max_error);
    REQ_I(control, "REFINE_PERIOD", cs->refine_period);
    REQ_I(control, "REPARTITION_PERIOD", cs->repartition_period);
    REQ_I(control, "MIN_LEVEL", cs->min_level);
    REQ_I(control, "MAX_LEVEL", cs->max_level);
    REQ_I(control, "FILE_OUTPUT_STEP", cs->file_output_step);
    REQ_I(control, "LOG_OUTPUT_STEP", cs->log_output_step);
    REQ_D(control, "TAU", cs->cfg.tau);
    REQ_D(control, "CFL", cs->cfg.cfl);
    REQ_D(control, "TMAX", cs->tmax);

    int rc;
    if ((rc = read_comps(charm_yaml_get(root, "components"), cs))) return rc;
    if ((rc = read_bnds(charm_yaml_get(root, "boundaries"), cs))) return rc;
    if ((rc = read_mats(charm_yaml_get(root, "materials"), cs))) return rc;
    if ((rc = read_regs(charm_yaml_get(root, "regions"), cs))) return rc;
    const charm_ynode_t *mesh = charm_yaml_get(root, "mesh");
    where = "mesh";
    REQ_S(mesh, "files_type", s);
    copy_name(cs->mesh_type, sizeof(cs->mesh_type), s);
    REQ_S(mesh, "name", s);
    copy_name(cs->mesh_name, sizeof(cs->mesh_name), s);

    const charm_ynode_t *model = charm_yaml_get(control, "MODEL");
    where = "control.MODEL";
    REQ_S(model, "name", s);
    if (!strcmp(s, "EULER")) {
        cs->cfg.model = CHARM_GPU_MODEL_EULER;   /* charm_model_euler_init reads nothing else */
    } else if (!strcmp(s, "NS")) {
        cs->cfg.model = CHARM_GPU_MODEL_NS;
        REQ_I(model, "use_visc", cs->cfg.use_visc);
        REQ_I(model, "use_diffusion", cs->cfg.use_diff);
        REQ_D(model, "t_ref", cs->cfg.t_ref);
        if ((rc = read_reactions(charm_yaml_get(root, "reactions"), cs))) return rc;
    } else {
        return case_fail(CHARM_GPU_EINVAL, "Unknown model type '%s'. Use: EULER, NS.", s);
    }
    return CHARM_GPU_OK;
}

int charm_case_parse_yaml(const char *text, charm_case_t *out)
{
    char err[256];
    if (!text || !out) return case_fail(CHARM_GPU_EINVAL, "null argument");
    charm_ynode_t *root = charm_yaml_parse(text, err, sizeof(err));
    if (!root) return case_fail(CHARM_GPU_EINVAL, "task.yaml: %s", err[0] ? err : "out of memory");
    const int rc = read_case(root, out);
    charm_yaml_free(root);
    return rc;
}

int charm_case_read_yaml(const char *path, charm_case_t *out)
{
    char err[512];
    if (!path || !out) return case_fail(CHARM_GPU_EINVAL, "null argument");
    charm_ynode_t *root = charm_yaml_load(path, err, sizeof(err));
    if (!root) return case_fail(CHARM_GPU_EINVAL, "%s: %s", path, err[0] ? err : "out of memory");
    const int rc = read_case(root, out);
    charm_yaml_free(root);
    return rc;
}
