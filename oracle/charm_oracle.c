/*
 * CPU restatement of CHARM_3D's explicit DG time step (test infrastructure).
 *
 * ORACLE ONLY.  Used by the tests, by __graft_entry__.smoke() as the checker
 * and by bench.py's CPU-baseline leg; never part of the GPU product path.
 *
 * It runs on the same flattened mesh the GPU library consumes
 * (charm_gpu_mesh_t, include/charm_gpu.h) and restates the reference's
 * arithmetic in plain C99, FP64, following each reference function in order:
 * per-element geometry and mass matrix (src/charm_geom.c), basis functions
 * (src/charm_base_func.c), cons<->prim and EOS (src/charm_globals.c:183-223,
 * src/charm_eos.c), fluxes (src/charm_fluxes.c), boundary conditions
 * (src/charm_bnd_cond.c), volume and surface integrals
 * (src/models/ns/charm_model_ns_conv.c), update and SSP-RK3
 * (src/models/ns/charm_model.c) and the Barth-Jespersen limiter
 * (src/limiters/charm_limiter_bj.c).  Unlike the GPU kernels it evaluates
 * the basis from coordinates, builds and inverts each mass matrix, and
 * takes cell means by quadrature, as the reference does.
 *
 * Pinned against the reference's own code (oracle/_ref, built by
 * oracle/build_ref.py) and against the committed fixtures in tests/golden/.
 *
 * Compile with -ffp-contract=off so that x86 and Arm give the same bits.
 */
#include "charm_gpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* basis size and quadrature sizes of the oracle instance `o` in scope:
 * p1 (4 functions) with the reference's rules (8 Gauss points per cell, 6
 * triangle points per face), or p2 (10 functions, the reference's
 * charm_base_func with CHARM_BASE_FN_COUNT = 10) with 27-point and 9-point
 * tensor Gauss rules (the reference's 8/6 rules under-integrate p2) */
#define NBMAX 10
#define NQMAX 27
#define NFQMAX 9
#define NB (o->nb)
#define NQ (o->nq)
#define NFQ (o->nfq)
#define MAXV (4 + CHARM_GPU_MAX_COMP)

static const double gR = 8.31446261815324;   /* src/charm_eos.c:8 */
static const double EPS = 1.e-12;            /* include/charm_def.h:158 */

typedef struct {
    double r, u, v, w, e, e_tot, p, t, cz, gam, cp, cv, m;
    double c[CHARM_GPU_MAX_COMP];
} prim_t;

typedef struct {
    double c[3], dh[3], vol;
    double qgp[NQMAX][3], qgj[NQMAX];
    double a_inv[NBMAX][NBMAX];
    double v[8][3];                 /* corners of a general hexahedron (p4est order) */
} elem_geom_t;

typedef struct oracle {
    charm_gpu_config_t cfg;
    int nb, nq, nfq;                /* basis functions, cell and face quadrature points */
    int64_t E, F, Fb;
    int V;
    elem_geom_t *g;
    int hex;                        /* general hexahedra: geometry from the corners */
    int8_t *face_face;              /* [2][F] face numbers of both sides (hex) */
    int32_t *face_elem;
    uint8_t *face_info;
    int32_t *bface_elem;
    int8_t *bface_face, *bface_bnd;
    double *u, *u_old, *res;        /* [V][B][E] */
    double *lim_nb;                 /* [E][6][V] limiter neighbour values */
    double *vis;                    /* [E][9][NB] tau xx yy zz xy xz yz, q x y z (after A^-1) */
    double *dif;                    /* [E][n_comp] species diffusion coefficients */
    double *chem_rhs;               /* [E] chemical heat release of the stage */
} oracle_t;

/* ---- component laws and EOS --------------------------------------------- */

static double comp_cp(const charm_gpu_comp_t *c, double t)
{   /* charm_comp_calc_cp, src/charm_globals.c:603-625 (ml_type guards the polynomial) */
    if (c->cp_type == CHARM_GPU_CP_CONST) return c->cp[0];
    if (c->ml_type == CHARM_GPU_CP_POLYNOM) {
        double res = 0., tt = 1.;
        for (int i = 0; i < c->n_cp; i++) { res += tt * c->cp[i]; tt *= t; }
        return res;
    }
    return c->cp[0];
}

static double comp_cp_dt(const charm_gpu_comp_t *c, double t)
{   /* :628-648 */
    double res = 0., tt = 1.;
    for (int i = 1; i < c->n_cp; i++) { res += tt * c->cp[i] * i; tt *= t; }
    return res;
}

static void calc_t(const oracle_t *o, prim_t *p)
{   /* _calc_t, src/charm_eos.c:12-54 */
    double m_ = 0.0, tt = 1.0;
    for (int i = 0; i < o->cfg.n_comp; i++) m_ += p->c[i] / o->cfg.comp[i].m;
    double rm = gR * m_;
    for (int j = 0; j < 100; j++) {
        double cp = 0.0, cp_dt = 0.0;
        for (int i = 0; i < o->cfg.n_comp; i++) {
            cp += p->c[i] * comp_cp(&o->cfg.comp[i], tt);
            cp_dt += p->c[i] * comp_cp_dt(&o->cfg.comp[i], tt);
        }
        double ft = (cp - rm) * tt - p->e;
        double ft_dt = (cp - rm) + cp_dt * tt;
        double tt1 = tt - ft / ft_dt;
        if (pow(tt1 - tt, 2) < EPS) { tt = tt1; break; }
        tt = tt1;
    }
    p->t = tt;
}

static void eos_switch(prim_t *p, int flag)
{   /* _charm_mat_eos_switch, src/charm_eos.c:57-96 */
    switch (flag) {
    case 0:
        if (p->r < EPS) p->r = EPS;
        p->p = p->r * p->e * (p->gam - 1);
        p->cz = sqrt(p->gam * p->p / p->r);
        break;
    case 1:
        if (p->r < EPS) p->r = EPS;
        if (p->p < EPS) p->p = EPS;
        p->e = p->p / (p->r * (p->gam - 1));
        p->t = p->e / p->cv;
        break;
    case 2:
        if (p->p < EPS) p->p = EPS;
        p->r = p->p * p->m / (p->t * gR);
        p->cz = sqrt(p->gam * p->p / p->r);
        break;
    case 3:
        if (p->p < EPS) p->p = EPS;
        p->r = p->p * p->m / (p->t * gR);
        p->cz = sqrt(p->gam * p->p / p->r);
        p->e = p->p / (p->r * (p->gam - 1));
        break;
    case 4:
        if (p->r < EPS) p->r = EPS;
        p->p = p->r * p->e * (p->gam - 1);
        p->cz = sqrt(p->gam * p->p / p->r);
        p->t = p->e / p->cv;
        break;
    }
}

static void eos(const oracle_t *o, prim_t *p, int flag)
{   /* charm_mat_eos_ideal / charm_mat_eos_mix, src/charm_eos.c:98-148 */
    const charm_gpu_comp_t *c0 = &o->cfg.comp[0];
    if (c0->cp_type == CHARM_GPU_CP_POLYNOM && (flag == 1 || flag == 4)) calc_t(o, p);
    double t = p->t;
    if (o->cfg.eos == CHARM_GPU_EOS_IDEAL) {
        p->cp = comp_cp(c0, t);
        p->m = c0->m;
    } else {
        double M_ = 0.;
        p->cp = 0.;
        for (int i = 0; i < o->cfg.n_comp; i++) {
            M_ += p->c[i] / o->cfg.comp[i].m;
            p->cp += p->c[i] * comp_cp(&o->cfg.comp[i], t);
        }
        p->m = 1. / M_;
    }
    p->cv = p->cp - gR / p->m;
    p->gam = p->cp / p->cv;
    eos_switch(p, flag);
}

static void cons_to_prim(const oracle_t *o, const double *U, prim_t *p)
{   /* charm_param_cons_to_prim, src/charm_globals.c:183-208 */
    int nc = o->cfg.n_comp;
    p->r = 0.;
    for (int i = 0; i < nc; i++) p->r += U[4 + i];
    p->u = U[0] / p->r;
    p->v = U[1] / p->r;
    p->w = U[2] / p->r;
    p->e_tot = U[3] / p->r;
    p->e = p->e_tot - 0.5 * (p->u * p->u + p->v * p->v + p->w * p->w);
    for (int i = 0; i < nc; i++) {
        p->c[i] = U[4 + i] / p->r;
        if (p->c[i] < 0.) p->c[i] = 0.;
        if (p->c[i] > 1.) p->c[i] = 1.;
    }
    p->t = 0.;
    eos(o, p, 4);
}

static void prim_to_cons(const oracle_t *o, const prim_t *p, double *U)
{   /* charm_param_prim_to_cons, :211-223 */
    U[0] = p->r * p->u;
    U[1] = p->r * p->v;
    U[2] = p->r * p->w;
    U[3] = p->r * (p->e + 0.5 * (p->u * p->u + p->v * p->v + p->w * p->w));
    for (int i = 0; i < o->cfg.n_comp; i++) U[4 + i] = p->r * p->c[i];
}

/* ---- boundary conditions (src/charm_bnd_cond.c:21-146) -------------------- */

static void bnd_cond(const oracle_t *o, int bid, const prim_t *in, prim_t *out, const double n[3])
{
    const charm_gpu_bnd_t *b = &o->cfg.bnd[bid];
    *out = *in;
    switch (b->type) {
    case CHARM_GPU_BND_INLET:
        out->u = b->params[0]; out->v = b->params[1]; out->w = b->params[2];
        out->t = b->params[3]; out->p = b->params[4];
        break;
    case CHARM_GPU_BND_WALL_SLIP: {
        double v[3] = {in->u, in->v, in->w};
        double svn = v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
        double vv[3] = {n[0] * svn, n[1] * svn, n[2] * svn};
        for (int i = 0; i < 3; i++) { v[i] -= vv[i]; v[i] -= vv[i]; }
        out->u = v[0]; out->v = v[1]; out->w = v[2];
        break;
    }
    case CHARM_GPU_BND_WALL_NO_SLIP: {
        double v[3] = {in->u, in->v, in->w};
        double svn = v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
        double vv[3] = {n[0] * svn, n[1] * svn, n[2] * svn};
        for (int i = 0; i < 3; i++) v[i] -= vv[i];
        out->u = v[0]; out->v = v[1]; out->w = v[2];
        out->t = b->params[0];
        break;
    }
    case CHARM_GPU_BND_MASS_FLOW: {
        const double *par = b->params;
        double flow_dir = n[0] * par[3] + n[1] * par[4] + n[2] * par[5];
        if (flow_dir > 0.) {
            double vel = out->u * n[0] + out->v * n[1] + out->w * n[2];
            if (vel < out->cz) out->p = par[6];   /* stored pressure, not written back */
        } else {
            for (int i = 0; i < o->cfg.n_comp; i++) out->c[i] = par[7 + i];
            eos(o, out, 0);
            double v2 = out->u * out->u + out->v * out->v + out->w * out->w;
            if (v2 > out->cz * out->cz) out->p = par[1];
            double k = pow(par[0] * (out->cp - out->cv) / (out->p * flow_dir), 2.) / (2. * out->cp);
            out->t = (-1 + sqrt(1.0 + 4.0 * k * par[2])) / (2. * k);
            double vel = fabs(par[0] / (out->r * flow_dir));
            out->u = par[3] * vel; out->v = par[4] * vel; out->w = par[5] * vel;
        }
        break;
    }
    default:
        break;   /* outlet */
    }
    eos(o, out, 3);
    out->e_tot = out->e + 0.5 * (out->u * out->u + out->v * out->v + out->w * out->w);
}

/* ---- fluxes (src/charm_fluxes.c) ------------------------------------------- */

static void flux_lf(const oracle_t *o, const prim_t pr[2], const double n[3], double *q)
{   /* :255-315 */
    int fc = 4 + o->cfg.n_comp;
    double ff[MAXV][2], uu[MAXV][2], vn[2];
    for (int i = 0; i < 2; i++) {
        vn[i] = pr[i].u * n[0] + pr[i].v * n[1] + pr[i].w * n[2];
        uu[0][i] = pr[i].r * pr[i].u;
        uu[1][i] = pr[i].r * pr[i].v;
        uu[2][i] = pr[i].r * pr[i].w;
        uu[3][i] = pr[i].r * pr[i].e_tot;
        ff[0][i] = pr[i].r * vn[i] * pr[i].u + pr[i].p * n[0];
        ff[1][i] = pr[i].r * vn[i] * pr[i].v + pr[i].p * n[1];
        ff[2][i] = pr[i].r * vn[i] * pr[i].w + pr[i].p * n[2];
        ff[3][i] = (pr[i].r * pr[i].e_tot + pr[i].p) * vn[i];
        for (int j = 4; j < fc; j++) {
            uu[j][i] = pr[i].r * pr[i].c[j - 4];
            ff[j][i] = pr[i].r * vn[i] * pr[i].c[j - 4];
        }
    }
    double a0 = fabs(vn[0]) + pr[0].cz, a1 = fabs(vn[1]) + pr[1].cz;
    double alpha = a0 > a1 ? a0 : a1;
    for (int i = 0; i < fc; i++) q[i] = 0.5 * (ff[i][1] + ff[i][0] - alpha * (uu[i][1] - uu[i][0]));
}

static void flux_cd(const oracle_t *o, const prim_t pr[2], const double n[3], double *q)
{   /* :513-559 */
    int fc = 4 + o->cfg.n_comp;
    double ff[MAXV][2], vn[2];
    for (int i = 0; i < 2; i++) {
        vn[i] = pr[i].u * n[0] + pr[i].v * n[1] + pr[i].w * n[2];
        ff[0][i] = pr[i].r * vn[i] * pr[i].u + pr[i].p * n[0];
        ff[1][i] = pr[i].r * vn[i] * pr[i].v + pr[i].p * n[1];
        ff[2][i] = pr[i].r * vn[i] * pr[i].w + pr[i].p * n[2];
        ff[3][i] = (pr[i].r * pr[i].e_tot + pr[i].p) * vn[i];
        for (int j = 4; j < fc; j++) ff[j][i] = pr[i].r * pr[i].c[j - 4] * vn[i];
    }
    for (int i = 0; i < fc; i++) q[i] = 0.5 * (ff[i][1] + ff[i][0]);
}

static void normal_frame(const double n[3], double nt[3][3])
{   /* :458-488 */
    nt[0][0] = n[0]; nt[0][1] = n[1]; nt[0][2] = n[2];
    double ri = sqrt(n[0] * n[0] + n[1] * n[1]);
    if (ri > EPS) {
        nt[1][0] = -n[1] / ri; nt[1][1] = n[0] / ri; nt[1][2] = 0.;
    } else {
        ri = sqrt(n[1] * n[1] + n[2] * n[2]);
        if (ri > EPS) {
            nt[1][0] = 0.; nt[1][1] = -n[2] / ri; nt[1][2] = n[1] / ri;
        } else {
            ri = sqrt(n[0] * n[0] + n[2] * n[2]);
            nt[1][0] = -n[2] / ri; nt[1][1] = 0.; nt[1][2] = n[0] / ri;
        }
    }
    nt[2][0] = nt[0][1] * nt[1][2] - nt[0][2] * nt[1][1];
    nt[2][1] = -nt[0][0] * nt[1][2] + nt[0][2] * nt[1][0];
    nt[2][2] = nt[0][0] * nt[1][1] - nt[0][1] * nt[1][0];
}

#define F_HLLC_U(UK, FK, SK, SS, PK, RK, VK) (((SS) * ((SK) * (UK) - (FK)) + (SK) * ((PK) + (RK) * ((SK) - (VK)) * ((SS) - (VK)))) / ((SK) - (SS)))
#define F_HLLC_V(UK, FK, SK, SS, PK, RK, VK) (((SS) * ((SK) * (UK) - (FK))) / ((SK) - (SS)))
#define F_HLLC_E(UK, FK, SK, SS, PK, RK, VK) (((SS) * ((SK) * (UK) - (FK)) + (SK) * ((PK) + (RK) * ((SK) - (VK)) * ((SS) - (VK))) * (SS)) / ((SK) - (SS)))

static void hllc_x(const oracle_t *o, const prim_t pr[2], double *qu, double *qv, double *qw, double *qe, double *qc)
{   /* _charm_calc_flux_hllc_x_1, :324-437 */
    int nc = o->cfg.n_comp;
    double p_pvrs = 0.5 * (pr[0].p + pr[1].p) - 0.5 * (pr[1].u - pr[0].u) * 0.25 * (pr[0].r + pr[1].r) * (pr[0].cz + pr[1].cz);
    double p_star = (p_pvrs > 0.) ? p_pvrs : 0.;
    double ql = (p_star <= pr[0].p) ? 1 : sqrt(1. + (pr[0].gam + 1.) * (p_star / pr[0].p - 1.) / (2. * pr[0].gam));
    double qr = (p_star <= pr[1].p) ? 1 : sqrt(1. + (pr[1].gam + 1.) * (p_star / pr[1].p - 1.) / (2. * pr[1].gam));
    double sl = pr[0].u - pr[0].cz * ql, sr = pr[1].u + pr[1].cz * qr;
    if (sl > sr) { double t = sl; sl = sr; sr = t; }
    double s_star = pr[1].p - pr[0].p;
    s_star += pr[0].r * pr[0].u * (sl - pr[0].u);
    s_star -= pr[1].r * pr[1].u * (sr - pr[1].u);
    s_star /= (pr[0].r * (sl - pr[0].u) - pr[1].r * (sr - pr[1].u));
    if (s_star < sl) s_star = sl;
    if (s_star > sr) s_star = sr;
    if (sl >= 0.) {
        *qu = pr[0].r * pr[0].u * pr[0].u + pr[0].p;
        *qv = pr[0].r * pr[0].v * pr[0].u;
        *qw = pr[0].r * pr[0].w * pr[0].u;
        *qe = (pr[0].r * pr[0].e_tot + pr[0].p) * pr[0].u;
        for (int i = 0; i < nc; i++) qc[i] = pr[0].r * pr[0].u * pr[0].c[i];
    } else if (sr <= 0.) {
        *qu = pr[1].r * pr[1].u * pr[1].u + pr[1].p;
        *qv = pr[1].r * pr[1].v * pr[1].u;
        *qw = pr[1].r * pr[1].w * pr[1].u;
        *qe = (pr[1].r * pr[1].e_tot + pr[1].p) * pr[1].u;
        for (int i = 0; i < nc; i++) qc[i] = pr[1].r * pr[1].u * pr[1].c[i];
    } else {
        int k = (s_star >= 0) ? 0 : 1;
        double sk = k ? sr : sl;
        const prim_t *p = &pr[k];
        *qu = F_HLLC_U(p->r * p->u, p->r * p->u * p->u + p->p, sk, s_star, p->p, p->r, p->u);
        *qv = F_HLLC_V(p->r * p->v, p->r * p->u * p->v, sk, s_star, p->p, p->r, p->u);
        *qw = F_HLLC_V(p->r * p->w, p->r * p->u * p->w, sk, s_star, p->p, p->r, p->u);
        *qe = F_HLLC_E(p->r * p->e_tot, (p->r * p->e_tot + p->p) * p->u, sk, s_star, p->p, p->r, p->u);
        for (int i = 0; i < nc; i++) qc[i] = F_HLLC_V(p->r * p->c[i], p->r * p->c[i] * p->u, sk, s_star, p->p, p->r, p->u);
    }
}

static void flux_hllc(const oracle_t *o, const prim_t pr[2], const double n[3], double *q)
{   /* charm_calc_flux_hllc, :439-510 */
    double nt[3][3];
    normal_frame(n, nt);
    prim_t pp[2];
    for (int i = 0; i < 2; i++) {
        double vv[3] = {pr[i].u, pr[i].v, pr[i].w};
        pp[i] = pr[i];
        pp[i].u = vv[0] * nt[0][0] + vv[1] * nt[0][1] + vv[2] * nt[0][2];
        pp[i].v = vv[0] * nt[1][0] + vv[1] * nt[1][1] + vv[2] * nt[1][2];
        pp[i].w = vv[0] * nt[2][0] + vv[1] * nt[2][1] + vv[2] * nt[2][2];
    }
    double fu, fv, fw;
    hllc_x(o, pp, &fu, &fv, &fw, &q[3], &q[4]);
    q[0] = fu * nt[0][0] + fv * nt[1][0] + fw * nt[2][0];
    q[1] = fu * nt[0][1] + fv * nt[1][1] + fw * nt[2][1];
    q[2] = fu * nt[0][2] + fv * nt[1][2] + fw * nt[2][2];
}

/* rim_orig, :8-180 */
static void rim_orig(double *RI, double *EI, double *PI, double *UI, double *VI, double *WI, double RB, double PB,
                     double UB, double VB, double WB, double RE, double PE, double UE, double VE, double WE, double gam)
{
    double AGAM = (gam - 1.0), DGAM = (2.0 / AGAM), EGAM = (AGAM / (gam + 1.0));
    double GGAM = (sqrt(gam * AGAM)), HGAM = (AGAM / 2.0), FGAM = (3.0 * gam - 1.0), OGAM = (AGAM / (2.0 * gam));
    double QGAM = (gam + 1.0), PGAM = (QGAM / (2.0 * gam)), RGAM = (4.0 * gam), SGAM = (gam * AGAM), TGAM = (QGAM / 2.0);
    (void) EGAM;
    double RF = 0, RS = 0, EF = 0, ES = 0, SBL, SFL, SSL, SEL, D, FS1, F1, ZNB, PKB, ZFB, PKE, ZNE, F2, FS2, ZFE, DP,
           UBD, RUBD, UF = 0, UED, RUED, US = 0, PPE, PPB, P;
    double eps = 1.e-5;
    double CB = sqrt(gam * PB / RB), CE = sqrt(gam * PE / RE);
    double EB = CB * CB / SGAM, EE = CE * CE / SGAM;
    double RCB = RB * CB, RCE = RE * CE, DU = UB - UE;
    if (DU < -2.0 * (CB + CE) / AGAM) {
        RF = RS = EF = ES = 0.0;
        SBL = UB - CB; SFL = UB + 2.0 * CB / AGAM; SSL = UE - 2.0 * CE / AGAM; SEL = UE + CE;
    } else {
        P = (PB * RCE + PE * RCB + DU * RCB * RCE) / (RCB + RCE);
        int step = 0;
        do {
            if (P < eps) P = eps;
            PPB = P / PB;
            if (PB <= P) {
                PKB = PGAM * PPB + OGAM; ZNB = RCB * sqrt(PKB);
                F1 = (P - PB) / ZNB; FS1 = (QGAM * PPB + FGAM) / (RGAM * ZNB * PKB);
            } else {
                ZFB = CB * exp(log(PPB) * OGAM); F1 = DGAM * (ZFB - CB); FS1 = ZFB / (gam * P);
            }
            PPE = P / PE;
            if (PE <= P) {
                PKE = PGAM * PPE + OGAM; ZNE = RCE * sqrt(PKE);
                F2 = (P - PE) / ZNE; FS2 = (QGAM * PPE + FGAM) / (RGAM * ZNE * PKE);
            } else {
                ZFE = CE * exp(log(PPE) * OGAM); F2 = DGAM * (ZFE - CE); FS2 = ZFE / (gam * P);
            }
            DP = (DU - F1 - F2) / (FS1 + FS2);
            P = P + DP;
        } while ((fabs(DU - F1 - F2) > eps) && (++step < 5000));
        PPB = P / PB; PPE = P / PE;
        ZFB = CB * exp(log(PPB) * OGAM); ZFE = CE * exp(log(PPE) * OGAM);
        if (PB <= P) {
            D = UB - sqrt((TGAM * P + HGAM * PB) / RB);
            UBD = UB - D; RUBD = RB * UBD;
            RF = RUBD * RUBD / (PB - P + RUBD * UBD);
            UF = D + RUBD / RF; EF = P / (AGAM * RF); SBL = D; SFL = D;
        } else {
            EF = ZFB * ZFB / SGAM; UF = UB + DGAM * (CB - ZFB); RF = P / (AGAM * EF);
            SBL = UB - CB; SFL = UF - ZFB;
        }
        if (PE <= P) {
            D = UE + sqrt((TGAM * P + HGAM * PE) / RE);
            UED = UE - D; RUED = RE * UED;
            RS = RUED * RUED / (PE - P + RUED * UED);
            US = D + RUED / RS; ES = P / (AGAM * RS); SEL = D; SSL = D;
        } else {
            ES = ZFE * ZFE / SGAM; US = UE - DGAM * (CE - ZFE); RS = P / (AGAM * ES);
            SSL = US + ZFE; SEL = UE + CE;
        }
    }
    if (SEL <= 0.0) { *RI = RE; *EI = EE; *UI = UE; *VI = VE; *WI = WE; *PI = AGAM * (*EI) * (*RI); return; }
    if (SBL >= 0.0) { *RI = RB; *EI = EB; *UI = UB; *VI = VB; *WI = WB; *PI = AGAM * (*EI) * (*RI); return; }
    if ((SSL >= 0.0) && (SFL <= 0.0)) {
        if (US >= 0.0) { *RI = RF; *EI = EF; *UI = UF; *VI = VB; *WI = WB; }
        else { *RI = RS; *EI = ES; *UI = US; *VI = VE; *WI = WE; }
        *PI = AGAM * (*EI) * (*RI);
        return;
    }
    if (SFL > 0.0) {
        *UI = (UB + DGAM * GGAM * sqrt(EB)) / (1 + DGAM); *VI = VB; *WI = WB;
        *EI = ((*UI) * (*UI)) / SGAM; *RI = RB * exp(log((*EI) / EB) * (1 / AGAM));
    } else {
        *UI = (UE - DGAM * GGAM * sqrt(EE)) / (1 + DGAM); *VI = VE; *WI = WE;
        *EI = ((*UI) * (*UI)) / SGAM; *RI = RE * exp(log((*EI) / EE) * (1 / AGAM));
    }
    *PI = AGAM * (*EI) * (*RI);
}

static void flux_godunov(const oracle_t *o, const prim_t pr[2], const double n[3], double *q)
{   /* the commented-out body of charm_calc_flux_godunov (:182-253), completed:
       species upwinded by the interface mass flux, gamma of side 0 */
    double nt[3][3], vn[2][3], ri, ei, pi, uu[3], uv[3];
    normal_frame(n, nt);
    for (int i = 0; i < 2; i++) {
        double vv[3] = {pr[i].u, pr[i].v, pr[i].w};
        for (int j = 0; j < 3; j++) vn[i][j] = vv[0] * nt[j][0] + vv[1] * nt[j][1] + vv[2] * nt[j][2];
    }
    rim_orig(&ri, &ei, &pi, &uu[0], &uu[1], &uu[2], pr[0].r, pr[0].p, vn[0][0], vn[0][1], vn[0][2], pr[1].r, pr[1].p,
             vn[1][0], vn[1][1], vn[1][2], pr[0].gam);
    for (int i = 0; i < 3; i++) {
        uv[i] = 0.;
        for (int j = 0; j < 3; j++) uv[i] += nt[j][i] * uu[j];
    }
    double qr = ri * uu[0];
    q[0] = qr * uv[0] + pi * n[0];
    q[1] = qr * uv[1] + pi * n[1];
    q[2] = qr * uv[2] + pi * n[2];
    q[3] = (ri * (ei + 0.5 * (uv[0] * uv[0] + uv[1] * uv[1] + uv[2] * uv[2])) + pi) * uu[0];
    for (int i = 0; i < o->cfg.n_comp; i++) q[4 + i] = qr * ((qr >= 0.) ? pr[0].c[i] : pr[1].c[i]);
}

static void num_flux(const oracle_t *o, const prim_t pr[2], const double n[3], double *q)
{
    switch (o->cfg.flux) {
    case CHARM_GPU_FLUX_LF: flux_lf(o, pr, n, q); break;
    case CHARM_GPU_FLUX_HLLC: flux_hllc(o, pr, n, q); break;
    case CHARM_GPU_FLUX_CD: flux_cd(o, pr, n, q); break;
    default: flux_godunov(o, pr, n, q); break;
    }
}

/* ---- geometry (src/charm_geom.c) ------------------------------------------ */

static double base_func(const double *x, int k, const double c[3], const double dh[3])
{   /* charm_base_func, src/charm_base_func.c:8-35 (p1: k < 4; p2: k < 10) */
    switch (k) {
    case 0: return 1.;
    case 1: return (x[0] - c[0]) / dh[0];
    case 2: return (x[1] - c[1]) / dh[1];
    case 3: return (x[2] - c[2]) / dh[2];
    case 4: return (x[0] - c[0]) * (x[0] - c[0]) / (dh[0] * dh[0]);
    case 5: return (x[1] - c[1]) * (x[1] - c[1]) / (dh[1] * dh[1]);
    case 6: return (x[2] - c[2]) * (x[2] - c[2]) / (dh[2] * dh[2]);
    case 7: return (x[0] - c[0]) * (x[1] - c[1]) / (dh[0] * dh[1]);
    case 8: return (x[0] - c[0]) * (x[2] - c[2]) / (dh[0] * dh[2]);
    case 9: return (x[1] - c[1]) * (x[2] - c[2]) / (dh[1] * dh[2]);
    default: return 0.;
    }
}

static double base_func_grad(const double *x, int k, const double c[3], const double dh[3], int dir)
{   /* charm_base_func_dx/dy/dz, :38-125 */
    if (k == 0) return 0.;
    if (k <= 3) return (k == dir + 1) ? 1. / dh[dir] : 0.;
    if (k <= 6) return (k == dir + 4) ? 2. * (x[dir] - c[dir]) / (dh[dir] * dh[dir]) : 0.;
    {   /* 7: xy, 8: xz, 9: yz */
        const int p0 = (k == 9) ? 1 : 0, p1 = (k == 7) ? 1 : 2;
        if (dir == p0) return (x[p1] - c[p1]) / (dh[p0] * dh[p1]);
        if (dir == p1) return (x[p0] - c[p0]) / (dh[p0] * dh[p1]);
        return 0.;
    }
}

static void matr_inv(int n, double a_src[NBMAX][NBMAX], double am[NBMAX][NBMAX])
{   /* Gauss-Jordan with partial pivoting, src/charm_globals.c:285-394 */
    double a[NBMAX][NBMAX];
    int mask[NBMAX], i, j, ni, nj;
    memcpy(a, a_src, sizeof(a));
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++) am[i][j] = (i == j) ? 1.0 : 0.0;
    for (i = 0; i < n; i++) mask[i] = i;
    for (i = 0; i < n; i++) {
        int maxind = i;
        double fmaxval = fabs(a[i][i]);
        for (ni = i + 1; ni < n; ni++)
            if (fabs(fmaxval) <= fabs(a[ni][i])) { fmaxval = fabs(a[ni][i]); maxind = ni; }
        if (i != maxind) {
            for (nj = 0; nj < n; nj++) {
                double t = a[i][nj]; a[i][nj] = a[maxind][nj]; a[maxind][nj] = t;
                t = am[i][nj]; am[i][nj] = am[maxind][nj]; am[maxind][nj] = t;
            }
            int ti = mask[i]; mask[i] = mask[maxind]; mask[maxind] = ti;
        }
        double aii = a[i][i];
        for (j = 0; j < n; j++) { a[i][j] /= aii; am[i][j] /= aii; }
        for (ni = 0; ni < n; ni++) {
            if (ni == i) continue;
            double fc = a[ni][i];
            for (nj = 0; nj < n; nj++) { a[ni][nj] -= fc * a[i][nj]; am[ni][nj] -= fc * am[i][nj]; }
        }
    }
}

/* 3-point Gauss-Legendre on [-1/2, 1/2] and its weights (sum 1), for the p2 rules */
static const double GL3X[3] = {-0.38729833462074168852, 0.0, 0.38729833462074168852};   /* sqrt(3/5)/2 */
static const double GL3W[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};

static void trilinear(const double v[8][3], const double ref[3], double x[3])
{   /* point of the trilinear map, src/charm_geom.c:47-66 */
    double wx[2] = {1. - ref[0], 1. + ref[0]}, wy[2] = {1. - ref[1], 1. + ref[1]}, wz[2] = {1. - ref[2], 1. + ref[2]};
    int vi = 0;
    x[0] = x[1] = x[2] = 0.;
    for (int iz = 0; iz < 2; iz++)
        for (int iy = 0; iy < 2; iy++) {
            double yf = wz[iz] * wy[iy];
            for (int ix = 0; ix < 2; ix++) {
                double xf = yf * wx[ix] / 8.;
                for (int k = 0; k < 3; k++) x[k] += xf * v[vi][k];
                vi++;
            }
        }
}

static void elem_vertices(const elem_geom_t *g, double v[8][3])
{   /* box vertices, x fastest (charm_quad_get_vertices, src/charm_geom.c:12-31) */
    for (int i = 0; i < 8; i++) {
        v[i][0] = g->c[0] + ((i & 1) ? 0.5 : -0.5) * g->dh[0];
        v[i][1] = g->c[1] + ((i & 2) ? 0.5 : -0.5) * g->dh[1];
        v[i][2] = g->c[2] + ((i & 4) ? 0.5 : -0.5) * g->dh[2];
    }
}

static void elem_geom(const oracle_t *o, elem_geom_t *g, const double c[3], const double h[3])
{   /* charm_geom_quad_calc for a box (src/charm_geom.c:496-530) */
    double v[8][3];
    const double s3 = 1. / sqrt(3.);
    for (int k = 0; k < 3; k++) { g->c[k] = c[k]; g->dh[k] = h[k]; }
    elem_vertices(g, v);
    g->vol = 0.;
    if (o->nb == 4) {
        for (int i = 0; i < NQ; i++) {
            double ref[3] = {(i & 1) ? s3 : -s3, (i & 2) ? s3 : -s3, (i & 4) ? s3 : -s3};
            trilinear(v, ref, g->qgp[i]);
            g->qgj[i] = (h[0] * 0.5) * (h[1] * 0.5) * (h[2] * 0.5);   /* det J of a box */
            g->vol += g->qgj[i];
        }
    } else {   /* 3 x 3 x 3 Gauss, x fastest */
        for (int i = 0; i < NQ; i++) {
            const int ix = i % 3, iy = (i / 3) % 3, iz = i / 9;
            g->qgp[i][0] = c[0] + GL3X[ix] * h[0];
            g->qgp[i][1] = c[1] + GL3X[iy] * h[1];
            g->qgp[i][2] = c[2] + GL3X[iz] * h[2];
            g->qgj[i] = h[0] * h[1] * h[2] * GL3W[ix] * GL3W[iy] * GL3W[iz];
            g->vol += g->qgj[i];
        }
    }
    double a[NBMAX][NBMAX];
    for (int i = 0; i < NB; i++)
        for (int j = 0; j < NB; j++) {
            a[i][j] = 0.;
            for (int q = 0; q < NQ; q++)
                a[i][j] += g->qgj[q] * base_func(g->qgp[q], i, g->c, g->dh) * base_func(g->qgp[q], j, g->c, g->dh);
        }
    matr_inv(NB, a, g->a_inv);
}

/* Face quadrature points of face f of a box (_charm_face_calc_gp_by_tri,
 * src/charm_geom.c:443-494) and the per-point weight gw*gj. */
static void face_points(const oracle_t *o, const elem_geom_t *g, int f, double gp[NFQMAX][3], double gwj[NFQMAX])
{
    if (o->nb != 4) {   /* p2: 3 x 3 Gauss on the face, lower tangential axis fastest */
        const int d = f / 2, sa = (d == 0) ? 1 : 0, ta = (d == 2) ? 1 : 2;
        const double area = g->dh[sa] * g->dh[ta];
        for (int i = 0; i < 9; i++) {
            const int is = i % 3, it = i / 3;
            gp[i][d] = g->c[d] + ((f & 1) ? 0.5 : -0.5) * g->dh[d];
            gp[i][sa] = g->c[sa] + GL3X[is] * g->dh[sa];
            gp[i][ta] = g->c[ta] + GL3X[it] * g->dh[ta];
            gwj[i] = area * GL3W[is] * GL3W[it];
        }
        return;
    }
    static const int ftv[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
    double v8[8][3], v[4][3];
    if (o->hex) memcpy(v8, g->v, sizeof(v8));
    else elem_vertices(g, v8);
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 3; k++) v[i][k] = v8[ftv[f][i]][k];
    const double a = 2.0 / 3.0, b = 1.0 / 6.0;
    for (int i = 0; i < 2; i++) {
        double pt[3][3];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) pt[j][k] = v[i + j][k];
        double a1 = pt[0][0] - pt[2][0], a2 = pt[1][0] - pt[2][0], a3 = pt[2][0];
        double b1 = pt[0][1] - pt[2][1], b2 = pt[1][1] - pt[2][1], b3 = pt[2][1];
        double c1 = pt[0][2] - pt[2][2], c2 = pt[1][2] - pt[2][2], c3 = pt[2][2];
        double E_ = a1 * a1 + b1 * b1 + c1 * c1, F_ = a2 * a2 + b2 * b2 + c2 * c2, G_ = a1 * a2 + b1 * b2 + c1 * c2;
        double gj = sqrt(E_ * F_ - G_ * G_);
        gp[3 * i + 0][0] = a * a1 + b * a2 + a3; gp[3 * i + 0][1] = a * b1 + b * b2 + b3; gp[3 * i + 0][2] = a * c1 + b * c2 + c3;
        gp[3 * i + 1][0] = b * a1 + a * a2 + a3; gp[3 * i + 1][1] = b * b1 + a * b2 + b3; gp[3 * i + 1][2] = b * c1 + a * c2 + c3;
        gp[3 * i + 2][0] = b * a1 + b * a2 + a3; gp[3 * i + 2][1] = b * b1 + b * b2 + b3; gp[3 * i + 2][2] = b * c1 + b * c2 + c3;
        for (int j = 0; j < 3; j++) gwj[3 * i + j] = gj * (1. / 6.);
    }
}

/* Face normal of face f made to point out of the element (src/charm_geom.c:181-211
 * and the flip of src/models/euler/charm_model.c:332-344). */
static void outward_normal(int f, double n[3])
{
    n[0] = n[1] = n[2] = 0.;
    n[f / 2] = (f & 1) ? 1. : -1.;
}

/* The same on a general hexahedron: the normal of the plane through the
 * face's first three corners (_charm_face_calc_normal, src/charm_geom.c:
 * 181-211), turned to point from the cell centre to the face centre as the
 * face callbacks turn it (src/models/ns/charm_model_ns_conv.c:226-241). */
static void hex_normal(const elem_geom_t *g, int f, double n[3])
{
    static const int ftv[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
    double a[3], b[3], l[3];
    for (int k = 0; k < 3; k++) {
        a[k] = g->v[ftv[f][1]][k] - g->v[ftv[f][0]][k];
        b[k] = g->v[ftv[f][2]][k] - g->v[ftv[f][0]][k];
        l[k] = (g->v[ftv[f][0]][k] + g->v[ftv[f][1]][k] + g->v[ftv[f][2]][k] + g->v[ftv[f][3]][k]) / 4. - g->c[k];
    }
    n[0] = a[1] * b[2] - a[2] * b[1];
    n[1] = a[2] * b[0] - a[0] * b[2];
    n[2] = a[0] * b[1] - a[1] * b[0];
    const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; k++) n[k] /= nl;
    if (n[0] * l[0] + n[1] * l[1] + n[2] * l[2] < 0)
        for (int k = 0; k < 3; k++) n[k] *= -1.0;
}

static void elem_normal(const oracle_t *o, int64_t e, int f, double n[3])
{
    if (o->hex) hex_normal(&o->g[e], f, n);
    else outward_normal(f, n);
}

/* Geometry of a general hexahedron from its corners (charm_geom_quad_calc,
 * src/charm_geom.c:496-530): the 8 Gauss points of the trilinear map with
 * the determinants of its Jacobian (_charm_quad_calc_gp_at_point, :40-128),
 * dh = the corners' bounding box (:157-169), the centre, the volume and the
 * inverted mass matrix.  Returns -1 for a non-positive determinant. */
static int hex_elem_geom(const oracle_t *o, elem_geom_t *g, const double v[8][3])
{
    const double s3 = 1. / sqrt(3.);
    memcpy(g->v, v, sizeof(g->v));
    const double r0[3] = {0., 0., 0.};
    trilinear(v, r0, g->c);
    for (int k = 0; k < 3; k++) {
        double lo = v[0][k], hi = v[0][k];
        for (int i = 1; i < 8; i++) {
            if (lo > v[i][k]) lo = v[i][k];
            if (hi < v[i][k]) hi = v[i][k];
        }
        g->dh[k] = hi - lo;
    }
    g->vol = 0.;
    for (int q = 0; q < 8; q++) {
        const double ref[3] = {(q & 1) ? s3 : -s3, (q & 2) ? s3 : -s3, (q & 4) ? s3 : -s3};
        trilinear(v, ref, g->qgp[q]);
        /* Jacobian: d/dksi, d/deta, d/dmu of the trilinear map */
        double jac[3][3] = {{0.}};
        for (int dir = 0; dir < 3; dir++) {
            int vi = 0;
            for (int iz = 0; iz < 2; iz++)
                for (int iy = 0; iy < 2; iy++)
                    for (int ix = 0; ix < 2; ix++) {
                        const int idx[3] = {ix, iy, iz};
                        double f = 1. / 8.;
                        for (int a = 0; a < 3; a++)
                            f *= (a == dir) ? (idx[a] ? 1. : -1.) : (idx[a] ? 1. + ref[a] : 1. - ref[a]);
                        for (int k = 0; k < 3; k++) jac[k][dir] += f * v[vi][k];
                        vi++;
                    }
        }
        const double det = jac[0][0] * (jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1]) -
                           jac[0][1] * (jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0]) +
                           jac[0][2] * (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]);
        if (!(det > 0.)) return -1;
        g->qgj[q] = det;   /* gw = 1 */
        g->vol += det;
    }
    double a[NBMAX][NBMAX];
    for (int i = 0; i < NB; i++)
        for (int j = 0; j < NB; j++) {
            a[i][j] = 0.;
            for (int q = 0; q < NQ; q++)
                a[i][j] += g->qgj[q] * base_func(g->qgp[q], i, g->c, g->dh) * base_func(g->qgp[q], j, g->c, g->dh);
        }
    matr_inv(NB, a, g->a_inv);
    return 0;
}

/* ---- state helpers ---------------------------------------------------------- */

static void get_fields(const oracle_t *o, const double *u, int64_t e, const double c[3], const double dh[3],
                       const double *x, double *U)
{   /* charm_get_fields, src/charm_base_func.c:198-211 */
    for (int v = 0; v < o->V; v++) {
        double r = 0.;
        for (int k = 0; k < NB; k++) r += u[(v * NB + k) * o->E + e] * base_func(x, k, c, dh);
        U[v] = r;
    }
}

static void get_fields_avg(const oracle_t *o, const double *u, int64_t e, double *U)
{   /* charm_get_fields_avg, :214-240 */
    const elem_geom_t *g = &o->g[e];
    for (int v = 0; v < o->V; v++) U[v] = 0.;
    for (int q = 0; q < NQ; q++) {
        double Uq[MAXV];
        double gjw = g->qgj[q] / g->vol;
        get_fields(o, u, e, g->c, g->dh, g->qgp[q], Uq);
        for (int v = 0; v < o->V; v++) U[v] += Uq[v] * gjw;
    }
}

/* centre of the side-1 element as seen from side 0 (periodic wraps put the
 * neighbour one period away; use the adjacent image) */
static void side1_center(const oracle_t *o, int64_t f, double c1[3])
{
    const int32_t e0 = o->face_elem[f], e1 = o->face_elem[o->F + f];
    const int d = o->face_info[f] & 3;
    memcpy(c1, o->g[e1].c, sizeof(double) * 3);
    if (o->face_info[f] & 0x40) c1[d] = o->g[e0].c[d] + 0.5 * (o->g[e0].dh[d] + o->g[e1].dh[d]);
}

static void diffusion(oracle_t *o, const double *u);
static void visc_grad(oracle_t *o, const double *u);
static void visc_integrals(oracle_t *o, const double *u, double *res);

/* ---- residual (src/models/ns/charm_model_ns_conv.c) ------------------------ */

static void residual(oracle_t *o, const double *u, double *res)
{
    const int64_t E = o->E;
    const int V = o->V;
    memset(res, 0, sizeof(double) * (size_t) V * NB * (size_t) E);
    if (o->cfg.use_visc && o->cfg.model == CHARM_GPU_MODEL_NS) {   /* charm_model_ns_timestep_diff */
        diffusion(o, u);
        visc_grad(o, u);
        visc_integrals(o, u, res);
    }
    /* volume integrals (:23-89) */
    for (int64_t e = 0; e < E; e++) {
        const elem_geom_t *g = &o->g[e];
        for (int q = 0; q < NQ; q++) {
            const double *x = g->qgp[q];
            double U[MAXV];
            prim_t p;
            get_fields(o, u, e, g->c, g->dh, x, U);
            cons_to_prim(o, U, &p);
            double F[3][MAXV];
            F[0][0] = U[0] * p.u + p.p; F[0][1] = U[0] * p.v; F[0][2] = U[0] * p.w; F[0][3] = U[0] * p.e_tot + p.p * p.u;
            F[1][0] = U[1] * p.u; F[1][1] = U[1] * p.v + p.p; F[1][2] = U[1] * p.w; F[1][3] = U[1] * p.e_tot + p.p * p.v;
            F[2][0] = U[2] * p.u; F[2][1] = U[2] * p.v; F[2][2] = U[2] * p.w + p.p; F[2][3] = U[2] * p.e_tot + p.p * p.w;
            for (int i = 0; i < o->cfg.n_comp; i++) {
                F[0][4 + i] = U[0] * p.c[i]; F[1][4 + i] = U[1] * p.c[i]; F[2][4 + i] = U[2] * p.c[i];
            }
            const double gjw = g->qgj[q];
            for (int k = 0; k < NB; k++) {
                double px = base_func_grad(x, k, g->c, g->dh, 0) * gjw, py = base_func_grad(x, k, g->c, g->dh, 1) * gjw,
                       pz = base_func_grad(x, k, g->c, g->dh, 2) * gjw, phi = base_func(x, k, g->c, g->dh) * gjw;
                for (int v = 0; v < V; v++) {
                    double gr = (v < 3) ? p.r * o->cfg.grav[v] * phi : 0.;
                    res[(v * NB + k) * E + e] -= (F[0][v] * px + F[1][v] * py + F[2][v] * pz) + gr;
                }
            }
        }
    }
    /* interior faces, conforming and hanging (:174-331) */
    for (int64_t f = 0; f < o->F; f++) {
        const int32_t e[2] = {o->face_elem[f], o->face_elem[o->F + f]};
        const int d = o->face_info[f] & 3, kind = (o->face_info[f] >> 2) & 3;
        double c1[3];
        if (o->hex) memcpy(c1, o->g[e[1]].c, sizeof(c1));
        else side1_center(o, f, c1);
        const double *cs[2] = {o->g[e[0]].c, c1};
        /* points on side 0's face (conforming / side 0 small) or side 1's face */
        const int hs = (kind == 2) ? 1 : 0;
        elem_geom_t pg = o->g[e[hs]];
        memcpy(pg.c, cs[hs], sizeof(double) * 3);
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        if (o->hex) {   /* the side's own face numbers; n from side 0's face */
            face_points(o, &pg, o->face_face[hs ? o->F + f : f], gp, gwj);
            hex_normal(&o->g[e[0]], o->face_face[f], n);
        } else {
            face_points(o, &pg, hs ? 2 * d : 2 * d + 1, gp, gwj);
            outward_normal(2 * d + 1, n);
        }
        for (int q = 0; q < NFQ; q++) {
            prim_t pr[2];
            for (int s = 0; s < 2; s++) {
                double U[MAXV];
                get_fields(o, u, e[s], cs[s], o->g[e[s]].dh, gp[q], U);
                cons_to_prim(o, U, &pr[s]);
            }
            double qf[MAXV];
            num_flux(o, pr, n, qf);
            for (int s = 0; s < 2; s++)
                for (int k = 0; k < NB; k++) {
                    double bfv = (s ? -1. : 1.) * base_func(gp[q], k, cs[s], o->g[e[s]].dh) * gwj[q];
                    for (int v = 0; v < V; v++) res[(v * NB + k) * E + e[s]] += qf[v] * bfv;
                }
        }
    }
    /* boundary faces (:96-171) */
    for (int64_t j = 0; j < o->Fb; j++) {
        const int32_t e = o->bface_elem[j];
        const int f = o->bface_face[j], bid = o->bface_bnd[j];
        const elem_geom_t *g = &o->g[e];
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        face_points(o, g, f, gp, gwj);
        elem_normal(o, e, f, n);
        for (int q = 0; q < NFQ; q++) {
            double U[MAXV];
            prim_t pr[2];
            get_fields(o, u, e, g->c, g->dh, gp[q], U);
            cons_to_prim(o, U, &pr[0]);
            bnd_cond(o, bid, &pr[0], &pr[1], n);
            double qf[MAXV];
            num_flux(o, pr, n, qf);
            for (int k = 0; k < NB; k++) {
                double bfv = base_func(gp[q], k, g->c, g->dh) * gwj[q];
                for (int v = 0; v < V; v++) res[(v * NB + k) * E + e] += qf[v] * bfv;
            }
        }
    }
}

/* ---- viscous terms (src/models/ns/charm_model_ns_diff*.c) ------------------ */

static double comp_ml(const charm_gpu_comp_t *c, double t)
{   /* charm_comp_calc_ml, src/charm_globals.c:651-662 */
    if (c->ml_type == CHARM_GPU_LAW_SUTHERLAND) return c->ml0 * sqrt(pow(t / c->t0, 3)) * (c->t0 + c->ts) / (t + c->ts);
    return c->ml0;
}

static double comp_kp(const charm_gpu_comp_t *c, double t)
{   /* charm_comp_calc_kp, :665-676 */
    if (c->kp_type == CHARM_GPU_LAW_SUTHERLAND) return c->kp0 * sqrt(pow(t / c->t0, 3)) * (c->t0 + c->ts) / (t + c->ts);
    return c->kp0;
}

static double comp_h(const oracle_t *o, const charm_gpu_comp_t *c, double t)
{   /* charm_comp_calc_enthalpy, :679-694: h0 + integral of the cp polynomial from t_ref */
    double h = c->h0;
    for (int i = 0; i < c->n_cp; i++) {
        double t2 = pow(t, i + 1) / (i + 1), t1 = pow(o->cfg.t_ref, i + 1) / (i + 1);
        h += c->cp[i] * (t2 - t1);
    }
    return h;
}

static double visc_mu(const oracle_t *o, const prim_t *p)
{   /* charm_get_visc_mu, src/charm_globals.c:515-538 (molar-fraction weighted) */
    double s = 0., mu = 0.;
    for (int i = 0; i < o->cfg.n_comp; i++) {
        double cm = p->c[i] / o->cfg.comp[i].m;
        s += cm;
        mu += cm * comp_ml(&o->cfg.comp[i], p->t);
    }
    return mu / s;
}

static double heat_k(const oracle_t *o, const prim_t *p)
{   /* charm_get_heat_k, :541-558 */
    double kt = 0.;
    for (int i = 0; i < o->cfg.n_comp; i++) kt += p->c[i] * comp_kp(&o->cfg.comp[i], p->t);
    return kt;
}

static void prim_at(const oracle_t *o, const double *u, int64_t e, const double c[3], const double *x, prim_t *p)
{
    double U[MAXV];
    get_fields(o, u, e, c, o->g[e].dh, x, U);
    cons_to_prim(o, U, p);
}

/* tau (6) and q (3) of element e at x from the lifted coefficients
 * (charm_get_visc_tau / charm_get_heat_q, src/charm_base_func.c:343-373) */
static void vis_at(const oracle_t *o, int64_t e, const double c[3], const double *x, double t[9])
{
    for (int f = 0; f < 9; f++) {
        t[f] = 0.;
        for (int k = 0; k < NB; k++) t[f] += o->vis[(e * 9 + f) * NB + k] * base_func(x, k, c, o->g[e].dh);
    }
}

static void diffusion(oracle_t *o, const double *u)
{   /* _charm_model_ns_timestep_diffusion_quad_iter_fn, src/models/ns/charm_model_ns_diff.c:18-71 */
    const int nc = o->cfg.n_comp;
    if (nc < 2) return;
    for (int64_t e = 0; e < o->E; e++) {
        prim_t p;
        double x[CHARM_GPU_MAX_COMP], s = 0.;
        prim_at(o, u, e, o->g[e].c, o->g[e].c, &p);
        double pabs = p.p / 101325.0;
        for (int i = 0; i < nc; i++) o->dif[e * nc + i] = 0.;
        if (!o->cfg.use_diff) continue;
        for (int i = 0; i < nc; i++) { x[i] = p.c[i] / o->cfg.comp[i].m; s += x[i]; }
        for (int i = 0; i < nc; i++) x[i] /= s;
        for (int i = 0; i < nc; i++) {
            if (fabs(p.c[i] - 1.) <= EPS) { o->dif[e * nc + i] = 0.; continue; }
            const charm_gpu_comp_t *ci = &o->cfg.comp[i];
            double s_xd = 0.;
            for (int j = 0; j < nc; j++) {
                const charm_gpu_comp_t *cj = &o->cfg.comp[j];
                double td = p.t / sqrt(ci->ek * cj->ek);
                double wd = 1.06036 / pow(td, 0.1561) + 0.1930 / exp(0.47635 * td) + 1.03587 / exp(1.52996 * td) +
                            1.76474 / exp(3.89411 * td);
                double dij = (2.628e-7) * sqrt(0.5 * (1.0 / (1000.0 * ci->m) + 1.0 / (1000.0 * cj->m))) *
                             sqrt(p.t * p.t * p.t) / (pabs * pow((0.5 * (ci->sig + cj->sig)), 2.0) * wd);
                s_xd += i == j ? 0. : x[j] / dij;
            }
            o->dif[e * nc + i] = (1. - x[i]) / s_xd;
        }
    }
}

/* one face point of the lifting: the central values -> q[9] (tau xx yy zz xy
 * xz yz, heat x y z) as in src/models/ns/charm_model_ns_diff_grad.c:150-176, 266-305 */
static void grad_face_q(const oracle_t *o, double mu, double kt, double fr, double ft, double fu, double fv,
                        double fw, const double *fc, const double *dm, const double n[3], double q[9])
{
    const double lambda = 0.;   /* charm_get_visc_lambda, src/charm_globals.c:509-512 */
    const double lp = (lambda + 4. * mu / 3.), lm = (lambda - 2. * mu / 3.);
    q[0] = lp * fu * n[0] + lm * fv * n[1] + lm * fw * n[2];
    q[1] = lm * fu * n[0] + lp * fv * n[1] + lm * fw * n[2];
    q[2] = lm * fu * n[0] + lm * fv * n[1] + lp * fw * n[2];
    q[3] = mu * (fu * n[1] + fv * n[0]);
    q[4] = mu * (fw * n[0] + fu * n[2]);
    q[5] = mu * (fw * n[1] + fv * n[2]);
    q[6] = kt * ft * n[0];
    q[7] = kt * ft * n[1];
    q[8] = kt * ft * n[2];
    for (int i = 0; i < o->cfg.n_comp; i++) {
        double h = comp_h(o, &o->cfg.comp[i], ft);
        q[6] += h * fr * dm[i] * fc[i] * n[0];
        q[7] += h * fr * dm[i] * fc[i] * n[1];
        q[8] += h * fr * dm[i] * fc[i] * n[2];
    }
}

static void grad_add(oracle_t *o, double *acc, int64_t e, const double q[9], double bfv, int k)
{
    for (int f = 0; f < 6; f++) acc[(e * 9 + f) * NB + k] += q[f] * bfv;
    for (int f = 6; f < 9; f++) acc[(e * 9 + f) * NB + k] -= q[f] * bfv;
}

/* charm_model_ns_timestep_diff_grad (src/models/ns/charm_model_ns_diff_grad.c) */
static void visc_grad(oracle_t *o, const double *u)
{
    const int64_t E = o->E;
    const int nc = o->cfg.n_comp;
    double *acc = (double *) calloc((size_t) E * 9 * NB, sizeof(double));
    /* volume (:21-77) */
    for (int64_t e = 0; e < E; e++) {
        const elem_geom_t *g = &o->g[e];
        for (int q = 0; q < NQ; q++) {
            const double *x = g->qgp[q];
            prim_t p;
            prim_at(o, u, e, g->c, x, &p);
            const double kt = heat_k(o, &p), lambda = 0., mu = visc_mu(o, &p);
            const double lp = (lambda + 4. * mu / 3.), lm = (lambda - 2. * mu / 3.);
            for (int k = 0; k < NB; k++) {
                const double px = base_func_grad(x, k, g->c, g->dh, 0) * g->qgj[q],
                             py = base_func_grad(x, k, g->c, g->dh, 1) * g->qgj[q],
                             pz = base_func_grad(x, k, g->c, g->dh, 2) * g->qgj[q];
                double *a = &acc[e * 9 * NB];
                a[0 * NB + k] -= (lp * p.u * px + lm * p.v * py + lm * p.w * pz);
                a[1 * NB + k] -= (lm * p.u * px + lp * p.v * py + lm * p.w * pz);
                a[2 * NB + k] -= (lm * p.u * px + lm * p.v * py + lp * p.w * pz);
                a[3 * NB + k] -= mu * (p.u * py + p.v * px);
                a[4 * NB + k] -= mu * (p.w * px + p.u * pz);
                a[5 * NB + k] -= mu * (p.w * py + p.v * pz);
                double tqx = kt * p.t * px, tqy = kt * p.t * py, tqz = kt * p.t * pz;
                for (int i = 0; i < nc; i++) {
                    double h = comp_h(o, &o->cfg.comp[i], p.t);
                    tqx += h * p.r * o->dif[e * nc + i] * p.c[i] * px;
                    tqy += h * p.r * o->dif[e * nc + i] * p.c[i] * py;
                    tqz += h * p.r * o->dif[e * nc + i] * p.c[i] * pz;
                }
                a[6 * NB + k] += tqx;
                a[7 * NB + k] += tqy;
                a[8 * NB + k] += tqz;
            }
        }
    }
    /* interior faces, conforming and hanging (:194-450) */
    for (int64_t f = 0; f < o->F; f++) {
        const int32_t e[2] = {o->face_elem[f], o->face_elem[o->F + f]};
        const int d = o->face_info[f] & 3, kind = (o->face_info[f] >> 2) & 3;
        double c1[3];
        side1_center(o, f, c1);
        const double *cs[2] = {o->g[e[0]].c, c1};
        const int hs = (kind == 2) ? 1 : 0;
        elem_geom_t pg = o->g[e[hs]];
        memcpy(pg.c, cs[hs], sizeof(double) * 3);
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        face_points(o, &pg, hs ? 2 * d : 2 * d + 1, gp, gwj);
        outward_normal(2 * d + 1, n);
        for (int q = 0; q < NFQ; q++) {
            prim_t pr[2];
            double mu[2], kt = 0.;
            for (int s = 0; s < 2; s++) {
                prim_at(o, u, e[s], cs[s], gp[q], &pr[s]);
                mu[s] = visc_mu(o, &pr[s]);
                kt += heat_k(o, &pr[s]);
            }
            const double fmu = 0.5 * (mu[0] + mu[1]);
            kt *= 0.5;
            double fc[CHARM_GPU_MAX_COMP], dm[CHARM_GPU_MAX_COMP];
            for (int i = 0; i < nc; i++) {
                fc[i] = (pr[0].c[i] + pr[1].c[i]) * 0.5;
                dm[i] = (o->dif[e[0] * nc + i] + o->dif[e[1] * nc + i]) * 0.5;
            }
            double qq[9];
            grad_face_q(o, fmu, kt, (pr[0].r + pr[1].r) * 0.5, (pr[0].t + pr[1].t) * 0.5, (pr[0].u + pr[1].u) * 0.5,
                        (pr[0].v + pr[1].v) * 0.5, (pr[0].w + pr[1].w) * 0.5, fc, dm, n, qq);
            for (int k = 0; k < NB; k++)
                for (int s = 0; s < 2; s++) {
                    double bfv = (s ? -1. : 1.) * base_func(gp[q], k, cs[s], o->g[e[s]].dh) * gwj[q];
                    grad_add(o, acc, e[s], qq, bfv, k);
                }
        }
    }
    /* boundary faces (:83-180) */
    for (int64_t j = 0; j < o->Fb; j++) {
        const int32_t e = o->bface_elem[j];
        const int f = o->bface_face[j], bid = o->bface_bnd[j];
        const elem_geom_t *g = &o->g[e];
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        face_points(o, g, f, gp, gwj);
        outward_normal(f, n);
        const int noslip = o->cfg.bnd[bid].type == CHARM_GPU_BND_WALL_NO_SLIP;
        for (int q = 0; q < NFQ; q++) {
            prim_t pr[2];
            prim_at(o, u, e, g->c, gp[q], &pr[0]);
            const double mu = visc_mu(o, &pr[0]), kt = heat_k(o, &pr[0]);
            bnd_cond(o, bid, &pr[0], &pr[1], n);
            double fu, fv, fw, ft;
            if (noslip) { fu = fv = fw = 0.; ft = o->cfg.bnd[bid].params[0]; }
            else {
                fu = (pr[0].u + pr[1].u) * 0.5; fv = (pr[0].v + pr[1].v) * 0.5;
                fw = (pr[0].w + pr[1].w) * 0.5; ft = (pr[0].t + pr[1].t) * 0.5;
            }
            double fc[CHARM_GPU_MAX_COMP];
            for (int i = 0; i < nc; i++) fc[i] = (pr[0].c[i] + pr[1].c[i]) * 0.5;
            double qq[9];
            grad_face_q(o, mu, kt, (pr[0].r + pr[1].r) * 0.5, ft, fu, fv, fw, fc, &o->dif[e * nc], n, qq);
            for (int k = 0; k < NB; k++) grad_add(o, acc, e, qq, base_func(gp[q], k, g->c, g->dh) * gwj[q], k);
        }
    }
    /* A^-1 (_charm_model_ns_diff_grad_update_quad_iter_fn, :462-476) */
    for (int64_t e = 0; e < E; e++)
        for (int f = 0; f < 9; f++)
            for (int i = 0; i < NB; i++) {
                double r = 0.;
                for (int k = 0; k < NB; k++) r += o->g[e].a_inv[i][k] * acc[(e * 9 + f) * NB + k];
                o->vis[(e * 9 + f) * NB + i] = r;
            }
    free(acc);
}

/* charm_model_ns_timestep_diff_integrals (src/models/ns/charm_model_ns_diff_integrals.c) */
static void visc_integrals(oracle_t *o, const double *u, double *res)
{
    const int64_t E = o->E;
    /* volume (:21-55) */
    for (int64_t e = 0; e < E; e++) {
        const elem_geom_t *g = &o->g[e];
        for (int q = 0; q < NQ; q++) {
            const double *x = g->qgp[q];
            prim_t p;
            double t[9];
            prim_at(o, u, e, g->c, x, &p);
            vis_at(o, e, g->c, x, t);
            for (int k = 0; k < NB; k++) {
                const double px = base_func_grad(x, k, g->c, g->dh, 0) * g->qgj[q],
                             py = base_func_grad(x, k, g->c, g->dh, 1) * g->qgj[q],
                             pz = base_func_grad(x, k, g->c, g->dh, 2) * g->qgj[q], phi = base_func(x, k, g->c, g->dh) * g->qgj[q];
                res[(0 * NB + k) * E + e] += (t[0] * px + t[3] * py + t[4] * pz);
                res[(1 * NB + k) * E + e] += (t[3] * px + t[1] * py + t[5] * pz);
                res[(2 * NB + k) * E + e] += (t[4] * px + t[5] * py + t[2] * pz);
                double *re = &res[(3 * NB + k) * E + e];
                *re += (t[0] * p.u + t[3] * p.v + t[4] * p.w) * px;
                *re += (t[3] * p.u + t[1] * p.v + t[5] * p.w) * py;
                *re += (t[4] * p.u + t[5] * p.v + t[2] * p.w) * pz;
                *re += o->chem_rhs[e] * phi;
            }
        }
    }
    /* interior faces (:200-392) */
    for (int64_t f = 0; f < o->F; f++) {
        const int32_t e[2] = {o->face_elem[f], o->face_elem[o->F + f]};
        const int d = o->face_info[f] & 3, kind = (o->face_info[f] >> 2) & 3;
        double c1[3];
        side1_center(o, f, c1);
        const double *cs[2] = {o->g[e[0]].c, c1};
        const int hs = (kind == 2) ? 1 : 0;
        elem_geom_t pg = o->g[e[hs]];
        memcpy(pg.c, cs[hs], sizeof(double) * 3);
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        face_points(o, &pg, hs ? 2 * d : 2 * d + 1, gp, gwj);
        outward_normal(2 * d + 1, n);
        for (int q = 0; q < NFQ; q++) {
            double ft6[6] = {0., 0., 0., 0., 0., 0.}, fu = 0., fv = 0., fw = 0., ft = 0.;
            for (int s = 0; s < 2; s++) {
                prim_t p;
                double t[9];
                prim_at(o, u, e[s], cs[s], gp[q], &p);
                vis_at(o, e[s], cs[s], gp[q], t);
                for (int c = 0; c < 6; c++) ft6[c] += t[c];
                fu += p.u * t[0] + p.v * t[3] + p.w * t[4];
                fv += p.u * t[3] + p.v * t[1] + p.w * t[5];
                fw += p.u * t[4] + p.v * t[5] + p.w * t[2];
                ft += t[6] * n[0] + t[7] * n[1] + t[8] * n[2];
            }
            for (int c = 0; c < 6; c++) ft6[c] *= 0.5;
            fu *= 0.5; fv *= 0.5; fw *= 0.5; ft *= 0.5;
            const double qu = ft6[0] * n[0] + ft6[3] * n[1] + ft6[4] * n[2];
            const double qv = ft6[3] * n[0] + ft6[1] * n[1] + ft6[5] * n[2];
            const double qw = ft6[4] * n[0] + ft6[5] * n[1] + ft6[2] * n[2];
            const double qe = fu * n[0] + fv * n[1] + fw * n[2] - ft;
            for (int k = 0; k < NB; k++)
                for (int s = 0; s < 2; s++) {
                    double bfv = (s ? -1. : 1.) * base_func(gp[q], k, cs[s], o->g[e[s]].dh) * gwj[q];
                    res[(0 * NB + k) * E + e[s]] -= qu * bfv;
                    res[(1 * NB + k) * E + e[s]] -= qv * bfv;
                    res[(2 * NB + k) * E + e[s]] -= qw * bfv;
                    res[(3 * NB + k) * E + e[s]] -= qe * bfv;
                }
        }
    }
    /* no-slip walls: one point at the face centre (:58-126) */
    for (int64_t j = 0; j < o->Fb; j++) {
        const int bid = o->bface_bnd[j];
        if (o->cfg.bnd[bid].type != CHARM_GPU_BND_WALL_NO_SLIP) continue;
        const int32_t e = o->bface_elem[j];
        const int f = o->bface_face[j], dd = f / 2;
        const elem_geom_t *g = &o->g[e];
        double n[3], x[3], U[MAXV], t[9];
        outward_normal(f, n);
        memcpy(x, g->c, sizeof(x));
        x[dd] += ((f & 1) ? 0.5 : -0.5) * g->dh[dd];
        const double area = g->dh[(dd + 1) % 3] * g->dh[(dd + 2) % 3];
        prim_t px, pr[2];
        prim_at(o, u, e, g->c, x, &px);
        const double mu = visc_mu(o, &px);
        get_fields_avg(o, u, e, U);
        cons_to_prim(o, U, &pr[0]);
        vis_at(o, e, g->c, x, t);
        bnd_cond(o, bid, &pr[0], &pr[1], n);
        const double vv[3] = {pr[0].u, pr[0].v, pr[0].w};
        const double un = vv[0] * n[0] + vv[1] * n[1] + vv[2] * n[2];
        const double vt[3] = {vv[0] - un * n[0], vv[1] - un * n[1], vv[2] - un * n[2]};
        const double ll = 0.5 * g->dh[dd];
        const double qu = -mu * vt[0] / ll, qv = -mu * vt[1] / ll, qw = -mu * vt[2] / ll;
        const double qe = -t[6] * n[0] - t[7] * n[1] - t[8] * n[2];
        for (int k = 0; k < NB; k++) {
            double bfv = base_func(x, k, g->c, g->dh) * 1. * area;
            res[(0 * NB + k) * E + e] -= qu * bfv;
            res[(1 * NB + k) * E + e] -= qv * bfv;
            res[(2 * NB + k) * E + e] -= qw * bfv;
            res[(3 * NB + k) * E + e] -= qe * bfv;
        }
    }
}

/* ---- chemistry on cell means (src/models/ns/charm_model_ns_chem.c) --------- */

/* _charm_model_ns_chem_rhs (:18-63): rates at concentrations cc -> phi, psi */
static void chem_rates(const oracle_t *o, double t, const double *cc, double *k, double *w, double *phi, double *psi)
{
    const int nr = o->cfg.n_react, nc = o->cfg.n_comp;
    for (int n = 0; n < nr; n++) {
        const charm_gpu_reaction_t *r = &o->cfg.react[n];
        k[n] = r->a * pow(t, r->n) * exp(-r->e / t / gR);
        w[n] = k[n];
        for (int m = 0; m < 3; m++) { int i = r->left[m]; w[n] *= (i < 0 ? 1. : cc[i]); }
    }
    if (!phi) return;
    for (int i = 0; i < nc; i++) {
        phi[i] = 0.;
        psi[i] = 0.;
        for (int n = 0; n < nr; n++) {
            const charm_gpu_reaction_t *r = &o->cfg.react[n];
            for (int m = 0; m < 3; m++) {
                if (i == r->left[m]) {
                    double x = k[n];
                    for (int j = 1; j < 3; j++) { int ic = r->left[(m + j) % 3]; x *= (ic < 0 ? 1. : cc[ic]); }
                    phi[i] += x;
                }
                if (i == r->right[m]) psi[i] += w[n];
            }
        }
    }
}

/* _charm_model_ns_chem_iter_fn (:111-156): two semi-implicit passes on the
 * molar concentrations of the cell mean, dt = the configured TAU (not the
 * stage dt, as in the reference); the species coefficients are replaced by
 * their new means (higher moments zeroed) and chem_rhs keeps the heat release
 * (_charm_model_ns_chem_rhs_save, :66-108, including its w -= chem_w[i]). */
static void chemistry(oracle_t *o, double *u)
{
    const int nc = o->cfg.n_comp, nr = o->cfg.n_react;
    const int64_t E = o->E;
    const double dt = o->cfg.tau;
    for (int64_t e = 0; e < E; e++) {
        o->chem_rhs[e] = 0.;
        if (!nr) continue;
        double U[MAXV], c[CHARM_GPU_MAX_COMP], ch[CHARM_GPU_MAX_COMP], c_[CHARM_GPU_MAX_COMP];
        double k[CHARM_GPU_MAX_REACT], w[CHARM_GPU_MAX_REACT], phi[CHARM_GPU_MAX_COMP], psi[CHARM_GPU_MAX_COMP];
        prim_t p;
        get_fields_avg(o, u, e, U);
        cons_to_prim(o, U, &p);
        for (int i = 0; i < nc; i++) { c[i] = U[4 + i] / o->cfg.comp[i].m; ch[i] = c[i]; }
        for (int j = 0; j < 2; j++) {
            for (int i = 0; i < nc; i++) c_[i] = (ch[i] + c[i]) * 0.5;
            chem_rates(o, p.t, c_, k, w, phi, psi);
            for (int i = 0; i < nc; i++) {
                ch[i] = (c[i] + dt * psi[i] * (1. + dt * phi[i] * 0.5));
                ch[i] /= (1. + dt * phi[i] + (dt * phi[i]) * (dt * phi[i]) * 0.5);
            }
        }
        chem_rates(o, p.t, ch, k, w, NULL, NULL);
        double rhs = 0.;
        for (int i = 0; i < nc; i++) {
            double ww = 0.;
            for (int n = 0; n < nr; n++) {
                const charm_gpu_reaction_t *r = &o->cfg.react[n];
                for (int m = 0; m < 3; m++) {
                    if (i == r->left[m]) ww -= w[i];   /* indexed by species, as the reference */
                    if (i == r->right[m]) ww += w[n];
                }
            }
            rhs += ww * comp_h(o, &o->cfg.comp[i], p.t);
        }
        o->chem_rhs[e] = rhs;
        for (int i = 0; i < nc; i++) {
            for (int kk = 0; kk < NB; kk++) u[((4 + i) * NB + kk) * E + e] = 0.;
            u[((4 + i) * NB) * E + e] = ch[i] * o->cfg.comp[i].m;
        }
    }
}

/* u -= dt * A^-1 * int (src/models/ns/charm_model.c:68-99) */
static void update(oracle_t *o, double *u, const double *res, double dt)
{
    for (int64_t e = 0; e < o->E; e++)
        for (int v = 0; v < o->V; v++) {
            double rhs[NBMAX];
            for (int i = 0; i < NB; i++) {
                rhs[i] = 0.;
                for (int j = 0; j < NB; j++) rhs[i] += o->g[e].a_inv[i][j] * res[(v * NB + j) * o->E + e];
            }
            for (int i = 0; i < NB; i++) u[(v * NB + i) * o->E + e] -= dt * rhs[i];
        }
}

/* ---- Barth-Jespersen limiter (src/limiters/charm_limiter_bj.c) ------------- */

static void limiter(oracle_t *o, double *u)
{
    const int64_t E = o->E;
    const int V = o->V;
    /* neighbour values per (element, face) */
    double *self = (double *) malloc(sizeof(double) * (size_t) V * (size_t) E);
    for (int64_t e = 0; e < E; e++) get_fields_avg(o, u, e, &self[e * V]);   /* init (:11-27) */
    /* boundary (:30-92) */
    for (int64_t j = 0; j < o->Fb; j++) {
        const int32_t e = o->bface_elem[j];
        const int f = o->bface_face[j];
        double n[3];
        prim_t pr[2];
        elem_normal(o, e, f, n);
        cons_to_prim(o, &self[e * V], &pr[0]);
        bnd_cond(o, o->bface_bnd[j], &pr[0], &pr[1], n);
        prim_to_cons(o, &pr[1], &o->lim_nb[(e * 6 + f) * V]);
    }
    /* interior (:95-223) */
    for (int64_t f = 0; f < o->F; f++) {
        const int32_t e0 = o->face_elem[f], e1 = o->face_elem[o->F + f];
        const int d = o->face_info[f] & 3, kind = (o->face_info[f] >> 2) & 3;
        const int f0 = o->hex ? o->face_face[f] : 2 * d + 1, f1 = o->hex ? o->face_face[o->F + f] : 2 * d;
        if (kind == 0) {
            memcpy(&o->lim_nb[(e0 * 6 + f0) * V], &self[e1 * V], sizeof(double) * V);
            memcpy(&o->lim_nb[(e1 * 6 + f1) * V], &self[e0 * V], sizeof(double) * V);
            continue;
        }
        /* hanging: each of the 4 records; the big side is done once (sub 0) */
        const int32_t small = (kind == 1) ? e0 : e1, big = (kind == 1) ? e1 : e0;
        const int fs = (kind == 1) ? f0 : f1, fbig = (kind == 1) ? f1 : f0;
        double cb[MAXV];
        get_fields(o, u, big, o->g[big].c, o->g[big].dh, o->g[big].c, cb);   /* value at the big centre */
        memcpy(&o->lim_nb[(small * 6 + fs) * V], cb, sizeof(double) * V);
        if (((o->face_info[f] >> 4) & 3) == 0) {
            double acc[MAXV], svol = 0.;
            for (int v = 0; v < V; v++) acc[v] = 0.;
            for (int k = 0; k < 4; k++) {
                const int64_t fk = f + k;
                const int32_t sk = (((o->face_info[fk] >> 2) & 3) == 1) ? o->face_elem[fk] : o->face_elem[o->F + fk];
                double cj[MAXV];
                get_fields(o, u, sk, o->g[sk].c, o->g[sk].dh, o->g[sk].c, cj);
                double vol = o->g[sk].vol;
                svol += vol;
                for (int v = 0; v < V; v++) acc[v] += cj[v] * vol;
            }
            for (int v = 0; v < V; v++) acc[v] /= svol;
            memcpy(&o->lim_nb[(big * 6 + fbig) * V], acc, sizeof(double) * V);
        }
    }
    /* calc (:241-315) */
    for (int64_t e = 0; e < E; e++) {
        const elem_geom_t *g = &o->g[e];
        double umin[MAXV], umax[MAXV], psi[MAXV], v8[8][3];
        const double *u0 = &self[e * V];
        for (int v = 0; v < V; v++) {
            umin[v] = umax[v] = u0[v];
            for (int f = 0; f < 6; f++) {
                double x = o->lim_nb[(e * 6 + f) * V + v];
                if (umin[v] > x) umin[v] = x;
                if (umax[v] < x) umax[v] = x;
            }
            psi[v] = 1.;
        }
        if (o->hex) memcpy(v8, g->v, sizeof(v8));
        else elem_vertices(g, v8);
        for (int i = 0; i < 8; i++) {
            double fv[MAXV];
            get_fields(o, u, e, g->c, g->dh, v8[i], fv);
            for (int v = 0; v < V; v++) {
                double pt = 1.;
                if (fabs(fv[v] - u0[v]) > EPS) {
                    if (fv[v] - u0[v] > 0) { double r = (umax[v] - u0[v]) / (fv[v] - u0[v]); pt = r < 1 ? r : 1; }
                    else if (fv[v] - u0[v] < 0) { double r = (umin[v] - u0[v]) / (fv[v] - u0[v]); pt = r < 1 ? r : 1; }
                }
                if (pt < psi[v]) psi[v] = pt;
            }
        }
        for (int k = 1; k < NB; k++)
            for (int v = 0; v < V; v++) u[(v * NB + k) * E + e] *= psi[v];
    }
    free(self);
}

/* ---- API --------------------------------------------------------------------- */

void oracle_free(oracle_t *o)
{
    if (!o) return;
    free(o->g); free(o->face_elem); free(o->face_info); free(o->bface_elem); free(o->bface_face); free(o->bface_bnd);
    free(o->face_face);
    free(o->u); free(o->u_old); free(o->res); free(o->lim_nb); free(o->vis); free(o->dif); free(o->chem_rhs);
    free(o);
}

oracle_t *oracle_new(const charm_gpu_config_t *cfg, const charm_gpu_mesh_t *m)
{
    oracle_t *o = (oracle_t *) calloc(1, sizeof(oracle_t));
    if (!o) return NULL;
    o->cfg = *cfg;
    o->nb = (cfg->p_order == 2) ? 10 : 4;
    o->nq = (cfg->p_order == 2) ? 27 : 8;
    o->nfq = (cfg->p_order == 2) ? 9 : 6;
    o->E = m->n_elem; o->F = m->n_face; o->Fb = m->n_bface;
    o->V = 4 + cfg->n_comp;
    const size_t st = sizeof(double) * (size_t) o->V * NB * (size_t) o->E;
    o->g = (elem_geom_t *) malloc(sizeof(elem_geom_t) * (size_t) o->E);
    o->face_elem = (int32_t *) malloc(sizeof(int32_t) * 2 * (size_t) (o->F + 1));
    o->face_info = (uint8_t *) malloc((size_t) o->F + 1);
    o->bface_elem = (int32_t *) malloc(sizeof(int32_t) * (size_t) (o->Fb + 1));
    o->bface_face = (int8_t *) malloc((size_t) o->Fb + 1);
    o->bface_bnd = (int8_t *) malloc((size_t) o->Fb + 1);
    o->u = (double *) calloc(1, st);
    o->u_old = (double *) calloc(1, st);
    o->res = (double *) calloc(1, st);
    o->lim_nb = (double *) calloc((size_t) o->E * 6 * (size_t) o->V, sizeof(double));
    o->vis = (double *) calloc((size_t) o->E * 9 * NB, sizeof(double));
    o->dif = (double *) calloc((size_t) o->E * (size_t) cfg->n_comp, sizeof(double));
    o->chem_rhs = (double *) calloc((size_t) o->E, sizeof(double));
    if (!o->g || !o->face_elem || !o->face_info || !o->bface_elem || !o->bface_face || !o->bface_bnd || !o->u ||
        !o->u_old || !o->res || !o->lim_nb || !o->vis || !o->dif || !o->chem_rhs) {
        oracle_free(o);
        return NULL;
    }
    for (int64_t e = 0; e < o->E; e++) {
        double c[3] = {m->center[e], m->center[o->E + e], m->center[2 * o->E + e]}, h[3];
        for (int d = 0; d < 3; d++) h[d] = ldexp(m->tree_len[d], -m->level[e]);
        elem_geom(o, &o->g[e], c, h);
    }
    memcpy(o->face_elem, m->face_elem, sizeof(int32_t) * 2 * (size_t) o->F);
    memcpy(o->face_info, m->face_info, (size_t) o->F);
    memcpy(o->bface_elem, m->bface_elem, sizeof(int32_t) * (size_t) o->Fb);
    memcpy(o->bface_face, m->bface_face, (size_t) o->Fb);
    memcpy(o->bface_bnd, m->bface_bnd, (size_t) o->Fb);
    return o;
}

/* The oracle on general hexahedra (charm_gpu_hex_t): every element's
 * geometry from its corners; p1, convective terms.  NULL for a
 * non-positive Jacobian or an unsupported configuration. */
oracle_t *oracle_new_hex(const charm_gpu_config_t *cfg, const charm_gpu_mesh_t *m, const charm_gpu_hex_t *x)
{
    if (cfg->p_order == 2 || cfg->use_visc || cfg->n_react) return NULL;
    oracle_t *o = oracle_new(cfg, m);
    if (!o) return NULL;
    o->hex = 1;
    o->face_face = (int8_t *) malloc(2 * (size_t) (o->F + 1));
    if (!o->face_face) { oracle_free(o); return NULL; }
    memcpy(o->face_face, x->face_face, 2 * (size_t) o->F);
    for (int64_t e = 0; e < o->E; e++) {
        double v[8][3];
        for (int k = 0; k < 8; k++)
            for (int d = 0; d < 3; d++) v[k][d] = x->vertex[(int64_t) (3 * k + d) * o->E + e];
        if (hex_elem_geom(o, &o->g[e], v)) { oracle_free(o); return NULL; }
    }
    return o;
}

int oracle_set_state(oracle_t *o, const double *u)
{
    memcpy(o->u, u, sizeof(double) * (size_t) o->V * NB * (size_t) o->E);
    return 0;
}

int oracle_get_state(oracle_t *o, double *u)
{
    memcpy(u, o->u, sizeof(double) * (size_t) o->V * NB * (size_t) o->E);
    return 0;
}

int oracle_residual(oracle_t *o, double *res)
{
    memset(o->chem_rhs, 0, sizeof(double) * (size_t) o->E);   /* no chemistry outside a step */
    residual(o, o->u, res);
    return 0;
}

int oracle_limit(oracle_t *o)
{
    if (o->cfg.limiter == CHARM_GPU_LIM_BJ) limiter(o, o->u);
    return 0;
}

/* One time step, as charm_model_ns_timestep_single / ..._euler_... */
int oracle_step(oracle_t *o, double dt)
{
    const size_t n = (size_t) o->V * NB * (size_t) o->E;
    const int lim = o->cfg.limiter == CHARM_GPU_LIM_BJ;
    if (o->cfg.model == CHARM_GPU_MODEL_EULER) {
        residual(o, o->u, o->res);
        update(o, o->u, o->res, dt);
        if (lim) limiter(o, o->u);
        return 0;
    }
    memcpy(o->u_old, o->u, sizeof(double) * n);             /* rk_0 (:119-133) */
    for (int s = 0; s < 3; s++) {
        chemistry(o, o->u);                                   /* charm_model_ns_timestep_chem */
        residual(o, o->u, o->res);
        update(o, o->u, o->res, dt);
        if (lim) limiter(o, o->u);
        if (s == 1)                                           /* rk_1 (:136-157) */
            for (size_t i = 0; i < n; i++) { o->u[i] *= 0.25; o->u[i] += 0.75 * o->u_old[i]; }
        if (s == 2)                                           /* rk_2 (:160-184) */
            for (size_t i = 0; i < n; i++) { o->u[i] *= 2.; o->u[i] /= 3.; o->u[i] += o->u_old[i] / 3.; }
    }
    return 0;
}

int oracle_run(oracle_t *o, int nsteps, double dt)
{
    for (int s = 0; s < nsteps; s++) oracle_step(o, dt);
    return 0;
}

/* Density-gradient estimate of charm_adapt (src/charm_amr.c:350-573):
 * grad[3][E] = (1/vol) * sum over faces of 0.5*(r_L + r_R) * n * gw * gj,
 * n pointing out of side 0, side 0 adding and side 1 subtracting; on
 * boundary faces the right state is the boundary condition's ghost. */
int oracle_amr_grad(oracle_t *o, double *grad)
{
    const int64_t E = o->E;
    memset(grad, 0, sizeof(double) * 3 * (size_t) E);
    for (int64_t j = 0; j < o->Fb; j++) {   /* _charm_amr_par_calc_face_iter_bnd (:362-423) */
        const int32_t e = o->bface_elem[j];
        const int f = o->bface_face[j];
        const elem_geom_t *g = &o->g[e];
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        face_points(o, g, f, gp, gwj);
        elem_normal(o, e, f, n);
        for (int q = 0; q < NFQ; q++) {
            double U[MAXV];
            prim_t pr[2];
            get_fields(o, o->u, e, g->c, g->dh, gp[q], U);
            cons_to_prim(o, U, &pr[0]);
            bnd_cond(o, o->bface_bnd[j], &pr[0], &pr[1], n);
            double qr = 0.5 * (pr[0].r + pr[1].r);
            for (int k = 0; k < 3; k++) grad[k * E + e] += qr * gwj[q] * n[k];
        }
    }
    for (int64_t f = 0; f < o->F; f++) {    /* _charm_amr_par_calc_face_iter_inner (:426-549) */
        const int32_t e[2] = {o->face_elem[f], o->face_elem[o->F + f]};
        const int d = o->face_info[f] & 3, kind = (o->face_info[f] >> 2) & 3;
        double c1[3];
        if (o->hex) memcpy(c1, o->g[e[1]].c, sizeof(c1));
        else side1_center(o, f, c1);
        const double *cs[2] = {o->g[e[0]].c, c1};
        const int hs = (kind == 2) ? 1 : 0;
        elem_geom_t pg = o->g[e[hs]];
        memcpy(pg.c, cs[hs], sizeof(double) * 3);
        double gp[NFQMAX][3], gwj[NFQMAX], n[3];
        if (o->hex) {
            face_points(o, &pg, o->face_face[hs ? o->F + f : f], gp, gwj);
            hex_normal(&o->g[e[0]], o->face_face[f], n);
        } else {
            face_points(o, &pg, hs ? 2 * d : 2 * d + 1, gp, gwj);
            outward_normal(2 * d + 1, n);
        }
        for (int q = 0; q < NFQ; q++) {
            prim_t pr[2];
            for (int s = 0; s < 2; s++) {
                double U[MAXV];
                get_fields(o, o->u, e[s], cs[s], o->g[e[s]].dh, gp[q], U);
                cons_to_prim(o, U, &pr[s]);
            }
            double qr = 0.5 * (pr[0].r + pr[1].r);
            for (int k = 0; k < 3; k++)
                for (int s = 0; s < 2; s++) grad[k * E + e[s]] += (s ? -1. : 1.) * gwj[q] * qr * n[k];
        }
    }
    for (int64_t e = 0; e < E; e++)          /* _charm_amr_par_calc_quad_iter_fn (:564-573) */
        for (int k = 0; k < 3; k++) grad[k * E + e] /= o->g[e].vol;
    return 0;
}

/* charm_replace_quads (src/charm_amr.c:206-307) for one family of general
 * hexahedra, p1: parent corners vp [8][3] and child corners vc [8][8][3]
 * (child ids in Morton order).  down != 0: the 8 children [8][V][4] from
 * the parent's coefficients [V][4] (refinement); down == 0: the parent
 * from the children's (coarsening).  ar[m][n] = sum over the target's (or
 * each source's) Gauss points of gw gj phi_m phi_n, then A^-1 (ar u).
 * Returns -1 for a non-positive Jacobian. */
int oracle_hex_project(const charm_gpu_config_t *cfg, const double *vp, const double *vc, int down, const double *src,
                       double *dst)
{
    oracle_t o;
    memset(&o, 0, sizeof(o));
    o.cfg = *cfg;
    o.nb = 4; o.nq = 8; o.nfq = 6;
    o.V = 4 + cfg->n_comp;
    oracle_t *op = &o;
    elem_geom_t P, C[8];
    double v[8][3];
    memcpy(v, vp, sizeof(v));
    if (hex_elem_geom(op, &P, v)) return -1;
    for (int i = 0; i < 8; i++) {
        memcpy(v, vc + 24 * i, sizeof(v));
        if (hex_elem_geom(op, &C[i], v)) return -1;
    }
    const int V = o.V;
#define NB_ 4
    if (down) {
        for (int i = 0; i < 8; i++) {
            double ar[NB_][NB_];
            for (int m = 0; m < NB_; m++)
                for (int n = 0; n < NB_; n++) {
                    ar[m][n] = 0.;
                    for (int q = 0; q < 8; q++)
                        ar[m][n] += C[i].qgj[q] * base_func(C[i].qgp[q], m, C[i].c, C[i].dh) *
                                    base_func(C[i].qgp[q], n, P.c, P.dh);
                }
            for (int vv = 0; vv < V; vv++) {
                double rhs[NB_];
                for (int m = 0; m < NB_; m++) {
                    rhs[m] = 0.;
                    for (int n = 0; n < NB_; n++) rhs[m] += ar[m][n] * src[vv * NB_ + n];
                }
                for (int k = 0; k < NB_; k++) {
                    double x = 0.;
                    for (int m = 0; m < NB_; m++) x += C[i].a_inv[k][m] * rhs[m];
                    dst[(i * V + vv) * NB_ + k] = x;
                }
            }
        }
    } else {
        for (int vv = 0; vv < V; vv++) {
            double rhs[NB_] = {0., 0., 0., 0.};
            for (int i = 0; i < 8; i++) {
                double ar[NB_][NB_];
                for (int m = 0; m < NB_; m++)
                    for (int n = 0; n < NB_; n++) {
                        ar[m][n] = 0.;
                        for (int q = 0; q < 8; q++)
                            ar[m][n] += C[i].qgj[q] * base_func(C[i].qgp[q], m, P.c, P.dh) *
                                        base_func(C[i].qgp[q], n, C[i].c, C[i].dh);
                    }
                for (int m = 0; m < NB_; m++)
                    for (int n = 0; n < NB_; n++) rhs[m] += ar[m][n] * src[(i * V + vv) * NB_ + n];
            }
            for (int k = 0; k < NB_; k++) {
                double x = 0.;
                for (int m = 0; m < NB_; m++) x += P.a_inv[k][m] * rhs[m];
                dst[vv * NB_ + k] = x;
            }
        }
    }
#undef NB_
    return 0;
}

/* The CFL time step of the reference's get_dt (src/models/ns/charm_model.c:
 * 21-36, 50-59; unreachable there after `return ctx->dt`): the minimum over
 * the cells of CFL * volume / (|u| + c) with the fields at the cell centre,
 * starting from TAU. */
int oracle_cfl_dt(oracle_t *o, double *dt)
{
    double d = o->cfg.tau;
    for (int64_t e = 0; e < o->E; e++) {
        const elem_geom_t *g = &o->g[e];
        double U[MAXV];
        prim_t p;
        get_fields(o, o->u, e, g->c, g->dh, g->c, U);
        cons_to_prim(o, U, &p);
        const double loc = o->cfg.cfl * g->vol / (sqrt(p.u * p.u + p.v * p.v + p.w * p.w) + p.cz);
        if (loc < d) d = loc;
    }
    *dt = d;
    return 0;
}

/* rim_orig above on n inputs (rL pL uL vL wL rR pR uR vR wR gam each) ->
 * (r e p u v w), for the pin against the reference's own rim_orig. */
int oracle_rim(int64_t n, const double *in, double *out)
{
    for (int64_t i = 0; i < n; i++) {
        const double *a = in + 11 * i;
        double *o = out + 6 * i;
        rim_orig(&o[0], &o[1], &o[2], &o[3], &o[4], &o[5], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9],
                 a[10]);
    }
    return 0;
}

/* Point flux on two primitive states (r u v w p each), for unit tests. */
int oracle_point_flux(oracle_t *o, const double *prim2, const double n[3], double *q)
{
    prim_t pr[2];
    for (int s = 0; s < 2; s++) {
        prim_t p;
        double U[MAXV];
        memset(&p, 0, sizeof(p));
        p.r = prim2[5 * s]; p.u = prim2[5 * s + 1]; p.v = prim2[5 * s + 2]; p.w = prim2[5 * s + 3]; p.p = prim2[5 * s + 4];
        for (int i = 0; i < o->cfg.n_comp; i++) p.c[i] = i == 0 ? 1. : 0.;
        eos(o, &p, 1);
        p.e_tot = p.e + 0.5 * (p.u * p.u + p.v * p.v + p.w * p.w);
        prim_to_cons(o, &p, U);
        cons_to_prim(o, U, &pr[s]);
    }
    num_flux(o, pr, n, q);
    return 0;
}

/* Point fluxes on conserved states (U = ru rv rw re rc_i), for the
 * derivative tests of the adjoint: interior (two states), boundary (one
 * state and the ghost of boundary bid) and the volume fluxes F[3][V]. */
int oracle_point_flux_cons(oracle_t *o, const double *U2, const double n[3], double *q)
{
    prim_t pr[2];
    for (int s = 0; s < 2; s++) cons_to_prim(o, U2 + s * o->V, &pr[s]);
    num_flux(o, pr, n, q);
    return 0;
}

int oracle_point_bflux_cons(oracle_t *o, int bid, const double *U, const double n[3], double *q)
{
    prim_t pr[2];
    cons_to_prim(o, U, &pr[0]);
    bnd_cond(o, bid, &pr[0], &pr[1], n);
    num_flux(o, pr, n, q);
    return 0;
}

int oracle_point_vflux(oracle_t *o, const double *U, double *F)
{   /* the volume fluxes of residual() above (src/models/ns/charm_model_ns_conv.c:45-65) */
    const int V = o->V;
    prim_t p;
    cons_to_prim(o, U, &p);
    const double vel[3] = {p.u, p.v, p.w};
    for (int d = 0; d < 3; d++) {
        for (int j = 0; j < 3; j++) F[d * V + j] = U[d] * vel[j] + (j == d ? p.p : 0.);
        F[d * V + 3] = U[d] * p.e_tot + p.p * vel[d];
        for (int i = 0; i < o->cfg.n_comp; i++) F[d * V + 4 + i] = U[d] * p.c[i];
    }
    return 0;
}
