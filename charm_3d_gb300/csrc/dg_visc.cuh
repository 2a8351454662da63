// Viscous and heat-conduction terms (BR1-like lifting) and chemistry of the
// NS model on sm_103a, FP64.
//
// Reference: charm_model_ns_timestep_diff (src/models/ns/charm_model_ns_diff.c:83-90):
//   1. species diffusion coefficients per element from the centre state
//      (:18-71; only with use_diffusion and >= 2 species)
//   2. lifting (charm_model_ns_diff_grad.c): the stress tensor tau (6) and
//      the heat flux q (3) as p1 fields per element, from central face
//      values and the volume term, times A^-1
//   3. viscous integrals (charm_model_ns_diff_integrals.c): volume terms of
//      tau and tau.u, central face fluxes, a one-point flux on no-slip walls
// and charm_model_ns_timestep_chem (charm_model_ns_chem.c:111-202): two
// semi-implicit passes on the molar concentrations of the cell mean.
//
// Kernels (per RK stage, in this order):
//   chem_kernel         u -> u' (species means replaced), chem_rhs
//   diffcoef_kernel     d[n_comp][E]
//   vgrad_face_kernel   the 9 lifted fields' face terms of every (face, side) -> slots9
//   vgrad_cell_kernel   volume term + gather of slots9 + A^-1 -> vis [9][B][E]
//   vflux_face_kernel   viscous face fluxes added into the convective slots
//   vvol_kernel         viscous volume terms (+ chem_rhs) -> radd [4][B][E],
//                       added by cell_kernel
// Slot layout, gather lists and face records are those of the convective
// face kernel; no atomics.
#pragma once

namespace charm {

// Sutherland factor sqrt((t/t0)^3) (t0 + ts) / (t + ts) of component i
// (charm_comp_calc_ml / _kp, src/charm_globals.c:651-676; (t/t0)^1.5 as
// x sqrt(x), without pow).  T = float reads the FP32 mirrors.
template <typename T>
__device__ __forceinline__ T sutherland(int i, T t)
{
    const T t0 = cfgv<T>(c_cfg.comp_t0[i], c_cfg.comp_t0_f[i]), ts = cfgv<T>(c_cfg.comp_ts[i], c_cfg.comp_ts_f[i]);
    const T x = qdiv<T>(t, t0);
    return qdiv<T>(x * qsqrt<T>(x) * (t0 + ts), t + ts);
}

// charm_comp_calc_enthalpy (:679-694): h0 + integral of the cp polynomial
// from t_ref, here as h0 - H(t_ref) + H(t) with H(t) = sum cp_k t^(k+1)/(k+1)
// by Horner (coefficients cp_k/(k+1) and H(t_ref) prepared on the host;
// in FP32 h0 - H(t_ref) is one constant)
template <typename T>
__device__ __forceinline__ T comp_h(int i, T t)
{
    T x = T(0);
    for (int k = c_cfg.comp_ncp[i] - 1; k >= 0; k--) x = x * t + cfgv<T>(c_cfg.comp_hc[i][k], c_cfg.comp_hc_f[i][k]);
    if constexpr (sizeof(T) == sizeof(float)) return c_cfg.comp_hoff_f[i] + x * t;
    else return c_cfg.comp_h0[i] + (x * t - c_cfg.comp_href[i]);
}

// charm_get_visc_mu and charm_get_heat_k (:515-558) at one point, with one
// Sutherland factor per component shared by mu and kappa (both laws use the
// component's t0 and ts)
template <int NC, typename T>
__device__ __forceinline__ void transport(const Prim<T, NC> &p, T &mu, T &kt)
{
    T s = T(0), m = T(0), k = T(0);
#pragma unroll
    for (int i = 0; i < NC; i++) {
        const bool sm = c_cfg.comp_ml_type[i] == CHARM_GPU_LAW_SUTHERLAND;
        const bool sk = c_cfg.comp_kp_type[i] == CHARM_GPU_LAW_SUTHERLAND;
        const T f = (sm || sk) ? sutherland<T>(i, p.t) : T(1);
        const T ml0 = cfgv<T>(c_cfg.comp_ml0[i], c_cfg.comp_ml0_f[i]), kp0 = cfgv<T>(c_cfg.comp_kp0[i], c_cfg.comp_kp0_f[i]);
        const T cm = p.c[i] * cfgv<T>(c_cfg.comp_inv_m[i], c_cfg.comp_inv_m_f[i]);
        s += cm;
        m += cm * (sm ? ml0 * f : ml0);
        k += p.c[i] * (sk ? kp0 * f : kp0);
    }
    mu = qdiv<T>(m, s);
    kt = k;
}

template <int NC>
__device__ __forceinline__ double visc_mu(const Prim<double, NC> &p)
{
    double mu, kt;
    transport<NC>(p, mu, kt);
    return mu;
}

// The 9 lifted fields' face values (diff_grad.c:150-176, 266-305): tau
// rows xx yy zz xy xz yz from the central velocity, heat flux from the
// central temperature and the species enthalpy-diffusion term.
template <int NC, typename T>
__device__ __forceinline__ void vgrad_q(T mu, T kt, T fr, T ft, T fu, T fv, T fw, const T *fc, const T *dm,
                                        const T n[3], T q[9])
{
    const T lambda = T(0);   // charm_get_visc_lambda (src/charm_globals.c:509-512)
    // 4 mu / 3 and 2 mu / 3 as products with 1/3 (within 1 ulp; a quotient
    // by 3 would be a full division at every face point)
    const T third = T(1.0 / 3.0);
    const T lp = (lambda + T(4) * mu * third), lm = (lambda - T(2) * mu * third);
    q[0] = lp * fu * n[0] + lm * fv * n[1] + lm * fw * n[2];
    q[1] = lm * fu * n[0] + lp * fv * n[1] + lm * fw * n[2];
    q[2] = lm * fu * n[0] + lm * fv * n[1] + lp * fw * n[2];
    q[3] = mu * (fu * n[1] + fv * n[0]);
    q[4] = mu * (fw * n[0] + fu * n[2]);
    q[5] = mu * (fw * n[1] + fv * n[2]);
    q[6] = kt * ft * n[0];
    q[7] = kt * ft * n[1];
    q[8] = kt * ft * n[2];
#pragma unroll
    for (int i = 0; i < NC; i++) {
        const T h = comp_h<T>(i, ft);
        q[6] += h * fr * dm[i] * fc[i] * n[0];
        q[7] += h * fr * dm[i] * fc[i] * n[1];
        q[8] += h * fr * dm[i] * fc[i] * n[2];
    }
}

// ---------------------------------------------------------------------------
// chemistry on cell means
// ---------------------------------------------------------------------------

// Arrhenius rate constants k_n = A t^n exp(-E / (t R)).  The reference
// recomputes them on every call of its rate function at the same cell
// temperature; here they are computed once per cell (same values).  t^0 is 1.
__device__ __forceinline__ void rate_consts(double t, double *k)
{
    for (int n = 0; n < c_cfg.n_react; n++) {
        const double tn = (c_cfg.react_n[n] == 0.0) ? 1.0 : pow(t, c_cfg.react_n[n]);
        k[n] = c_cfg.react_a[n] * tn * exp(-c_cfg.react_e[n] / t / kGasR);
    }
}

// rates w and, when phi != nullptr, the semi-implicit split phi, psi at the
// molar concentrations cc, from the rate constants k
template <int NC>
__device__ __forceinline__ void chem_rates(const double *k, const double *cc, double *w, double *phi, double *psi)
{   // _charm_model_ns_chem_rhs (charm_model_ns_chem.c:18-63)
    const int nr = c_cfg.n_react;
    for (int n = 0; n < nr; n++) {
        w[n] = k[n];
        for (int m = 0; m < 3; m++) {
            const int i = c_cfg.react_l[n][m];
            w[n] *= (i < 0 ? 1. : cc[i]);
        }
    }
    if (!phi) return;
    for (int i = 0; i < NC; i++) {
        phi[i] = 0.;
        psi[i] = 0.;
        for (int n = 0; n < nr; n++)
            for (int m = 0; m < 3; m++) {
                if (i == c_cfg.react_l[n][m]) {
                    double x = k[n];
                    for (int j = 1; j < 3; j++) {
                        const int ic = c_cfg.react_l[n][(m + j) % 3];
                        x *= (ic < 0 ? 1. : cc[ic]);
                    }
                    phi[i] += x;
                }
                if (i == c_cfg.react_r[n][m]) psi[i] += w[n];
            }
    }
}

// _charm_model_ns_chem_iter_fn (:111-156) + _charm_model_ns_chem_rhs_save
// (:66-108): dt is the configured TAU (as the reference's ctx->dt); the
// species coefficients become their new means (higher moments zeroed);
// chem_rhs keeps the heat release, including the reference's w -= w[i]
// (reaction rate indexed by the species).  out may not alias u.
template <int NC>
__global__ void __launch_bounds__(128)
chem_kernel(MeshDev m, const double *__restrict__ u, double *__restrict__ out, double *__restrict__ chem_rhs)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double U[V];
#pragma unroll
    for (int v = 0; v < V; v++) U[v] = __ldg(u + (int64_t) (v * kNB) * E + e);
    Prim<double, NC> p;
    cons_to_prim<double, NC>(U, p);
    const double dt = c_cfg.tau;
    double c[NC], ch[NC], c_[NC], phi[NC], psi[NC];
    double k[CHARM_GPU_MAX_REACT], w[CHARM_GPU_MAX_REACT];
#pragma unroll
    for (int i = 0; i < NC; i++) {
        c[i] = U[4 + i] / c_cfg.comp_m[i];
        ch[i] = c[i];
    }
    rate_consts(p.t, k);
    for (int j = 0; j < 2; j++) {
#pragma unroll
        for (int i = 0; i < NC; i++) c_[i] = (ch[i] + c[i]) * 0.5;
        chem_rates<NC>(k, c_, w, phi, psi);
#pragma unroll
        for (int i = 0; i < NC; i++) {
            ch[i] = (c[i] + dt * psi[i] * (1. + dt * phi[i] * 0.5));
            ch[i] /= (1. + dt * phi[i] + (dt * phi[i]) * (dt * phi[i]) * 0.5);
        }
    }
    chem_rates<NC>(k, ch, w, nullptr, nullptr);
    double rhs = 0.;
#pragma unroll
    for (int i = 0; i < NC; i++) {
        double ww = 0.;
        for (int n = 0; n < c_cfg.n_react; n++)
            for (int mm = 0; mm < 3; mm++) {
                if (i == c_cfg.react_l[n][mm]) ww -= w[i];
                if (i == c_cfg.react_r[n][mm]) ww += w[n];
            }
        rhs += ww * comp_h(i, p.t);
    }
    chem_rhs[e] = rhs;
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int kk = 0; kk < kNB; kk++) out[(int64_t) (v * kNB + kk) * E + e] = __ldg(u + (int64_t) (v * kNB + kk) * E + e);
#pragma unroll
    for (int i = 0; i < NC; i++) {
        out[(int64_t) ((4 + i) * kNB) * E + e] = ch[i] * c_cfg.comp_m[i];
#pragma unroll
        for (int kk = 1; kk < kNB; kk++) out[(int64_t) ((4 + i) * kNB + kk) * E + e] = 0.;
    }
}

// ---------------------------------------------------------------------------
// state access in FP64 for the per-element kernels that stay FP64 in the
// mixed form (chemistry, diffusion coefficients): a double plane, or the
// FP32 hi/lo planes of the mixed form (hi + lo is exact in double)
// ---------------------------------------------------------------------------

template <typename S> struct StIn;
template <> struct StIn<double> {
    const double *u;
    __device__ __forceinline__ double at(int64_t i) const { return __ldg(u + i); }
};
template <> struct StIn<float> {
    const float *h, *l;
    __device__ __forceinline__ double at(int64_t i) const { return (double) __ldg(h + i) + (double) __ldg(l + i); }
};

template <typename S> struct StOut;
template <> struct StOut<double> {
    double *u;
    __device__ __forceinline__ void put(int64_t i, double x) const { u[i] = x; }
    __device__ __forceinline__ void copy(int64_t i, const StIn<double> &in) const { u[i] = __ldg(in.u + i); }
};
template <> struct StOut<float> {
    float *h, *l;
    __device__ __forceinline__ void put(int64_t i, double x) const
    {
        const float a = __double2float_rn(x);
        h[i] = a;
        l[i] = __double2float_rn(x - (double) a);
    }
    __device__ __forceinline__ void copy(int64_t i, const StIn<float> &in) const
    {
        h[i] = __ldg(in.h + i);
        l[i] = __ldg(in.l + i);
    }
};

// ---------------------------------------------------------------------------
// species diffusion coefficients (charm_model_ns_diff.c:18-71)
// ---------------------------------------------------------------------------
// NBK: basis functions per variable (4 or 10); the centre value is c_0 for
// both.  The state, mass and mole fractions and the pure-species test are
// FP64 (a fraction within 1e-12 of 1 is not resolvable in FP32); the
// collision integrals and the binary coefficients are computed and stored
// in TD: double for the FP64 form, float for the mixed form (whose kernels
// read them as float; the transport coefficients there are FP32 too).
template <int NC, int NBK, typename S, typename TD>
__global__ void __launch_bounds__(128) diffcoef_kernel(MeshDev m, StIn<S> u, TD *__restrict__ dif)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double U[V];
#pragma unroll
    for (int v = 0; v < V; v++) U[v] = u.at((int64_t) (v * NBK) * E + e);   // centre value = c_0
    Prim<double, NC> p;
    cons_to_prim<double, NC>(U, p);
    const TD pabs = TD(p.p / 101325.0), t = TD(p.t);
    double x[NC], s = 0.;
#pragma unroll
    for (int i = 0; i < NC; i++) {
        x[i] = p.c[i] / c_cfg.comp_m[i];
        s += x[i];
    }
#pragma unroll
    for (int i = 0; i < NC; i++) x[i] /= s;
#pragma unroll
    for (int i = 0; i < NC; i++) {
        TD d = TD(0);
        if (!(fabs(p.c[i] - 1.) <= kEps)) {
            TD s_xd = TD(0);
#pragma unroll
            for (int j = 0; j < NC; j++) {
                const TD td = t / TD(sqrt(c_cfg.comp_ek[i] * c_cfg.comp_ek[j]));
                const TD wd = TD(1.06036) / pow(td, TD(0.1561)) + TD(0.1930) / exp(TD(0.47635) * td) +
                              TD(1.03587) / exp(TD(1.52996) * td) + TD(1.76474) / exp(TD(3.89411) * td);
                const TD sg = TD(0.5 * (c_cfg.comp_sig[i] + c_cfg.comp_sig[j]));
                const TD dij = TD(2.628e-7) *
                               TD(sqrt(0.5 * (1.0 / (1000.0 * c_cfg.comp_m[i]) + 1.0 / (1000.0 * c_cfg.comp_m[j])))) *
                               sqrt(t * t * t) / (pabs * (sg * sg) * wd);
                s_xd += i == j ? TD(0) : TD(x[j]) / dij;
            }
            if constexpr (sizeof(TD) == sizeof(float)) d = (s_xd > 0.f) ? TD(1. - x[i]) / s_xd : 0.f;   // FP32 underflow
            else d = (1. - x[i]) / s_xd;
        }
        dif[(int64_t) i * E + e] = d;
    }
}

// ---------------------------------------------------------------------------
// lifting: face terms -> slots9 [9*B][S], sign of the heat rows included
// ---------------------------------------------------------------------------

template <int NC, int D>
__device__ __forceinline__ void vgrad_interior(const MeshDev &m, const double *__restrict__ u,
                                               const double *__restrict__ dif, double *__restrict__ s9, int64_t i)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e0 = m.face_elem[i], e1 = m.face_elem[m.n_face + i];
    const unsigned info = m.face_info[i];
    const int kind = (info >> 2) & 3, sub = (info >> 4) & 3;
    const int lev = m.level[(kind == 2) ? e1 : e0];
    const double w = level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0);
    const double os = (sub & 1) ? 0.25 : -0.25, ot = (sub & 2) ? 0.25 : -0.25;
    const double g0 = (kind == 2) ? 0.5 : 1.0, g1 = (kind == 1) ? 0.5 : 1.0;
    const double hs0 = (kind == 2) ? os : 0.0, ht0 = (kind == 2) ? ot : 0.0;
    const double hs1 = (kind == 1) ? os : 0.0, ht1 = (kind == 1) ? ot : 0.0;
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = 1.0;
    double dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = (dif[(int64_t) c * E + e0] + dif[(int64_t) c * E + e1]) * 0.5;
    double S0[9], Ss[9], St[9];
#pragma unroll
    for (int f = 0; f < 9; f++) S0[f] = Ss[f] = St[f] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const double ps = face_ps<double>(g), pt = face_pt<double>(g);
        const double ps0 = g0 * ps + hs0, pt0 = g0 * pt + ht0, ps1 = g1 * ps + hs1, pt1 = g1 * pt + ht1;
        double Ua[V], Ub[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            const int64_t p0 = (int64_t) (v * kNB) * E;
            Ua[v] = __ldg(u + p0 + e0) + 0.5 * __ldg(u + p0 + (int64_t) (1 + D) * E + e0) +
                    ps0 * __ldg(u + p0 + (int64_t) (1 + s) * E + e0) + pt0 * __ldg(u + p0 + (int64_t) (1 + t) * E + e0);
            Ub[v] = __ldg(u + p0 + e1) - 0.5 * __ldg(u + p0 + (int64_t) (1 + D) * E + e1) +
                    ps1 * __ldg(u + p0 + (int64_t) (1 + s) * E + e1) + pt1 * __ldg(u + p0 + (int64_t) (1 + t) * E + e1);
        }
        Prim<double, NC> pa, pb;
        cons_to_prim<double, NC>(Ua, pa);
        cons_to_prim<double, NC>(Ub, pb);
        double mua, kta, mub, ktb;
        transport<NC>(pa, mua, kta);
        transport<NC>(pb, mub, ktb);
        const double fmu = 0.5 * (mua + mub);
        const double kt = (kta + ktb) * 0.5;
        double fc[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) fc[c] = (pa.c[c] + pb.c[c]) * 0.5;
        double q[9];
        vgrad_q<NC>(fmu, kt, (pa.r + pb.r) * 0.5, (pa.t + pb.t) * 0.5, (pa.u + pb.u) * 0.5, (pa.v + pb.v) * 0.5,
                    (pa.w + pb.w) * 0.5, fc, dm, n, q);
#pragma unroll
        for (int f = 0; f < 9; f++) {
            S0[f] += q[f];
            Ss[f] += q[f] * ps;
            St[f] += q[f] * pt;
        }
    }
    // side 0: + phi0 * w; side 1: - phi1 * w; heat rows enter with the opposite sign
    const int64_t base = 2 * i;
#pragma unroll
    for (int f = 0; f < 9; f++) {
        const double sg = (f < 6) ? w : -w;
        const double a0 = sg * S0[f], as = sg * Ss[f], at = sg * St[f];
        store_pair<double>(s9, (int64_t) (f * kNB + 0) * S + base, a0, -a0);
        store_pair<double>(s9, (int64_t) (f * kNB + 1 + D) * S + base, 0.5 * a0, 0.5 * a0);
        store_pair<double>(s9, (int64_t) (f * kNB + 1 + s) * S + base, g0 * as + hs0 * a0, -(g1 * as + hs1 * a0));
        store_pair<double>(s9, (int64_t) (f * kNB + 1 + t) * S + base, g0 * at + ht0 * a0, -(g1 * at + ht1 * a0));
    }
}

template <int NC, int D>
__device__ __forceinline__ void vgrad_boundary(const MeshDev &m, const double *__restrict__ u,
                                               const double *__restrict__ dif, double *__restrict__ s9, int64_t j)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
    const double sg = (f & 1) ? 1.0 : -1.0;
    const int lev = m.level[e];
    const double w = level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0);
    const bool noslip = c_cfg.bnd_type[bid] == CHARM_GPU_BND_WALL_NO_SLIP;
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = sg;
    double c[V][kNB], dm[NC];
    load_coef<double, V>(u, E, e, c);
#pragma unroll
    for (int k = 0; k < NC; k++) dm[k] = dif[(int64_t) k * E + e];
    double S0[9], Ss[9], St[9];
#pragma unroll
    for (int q = 0; q < 9; q++) S0[q] = Ss[q] = St[q] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const double ps = face_ps<double>(g), pt = face_pt<double>(g);
        double U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + 0.5 * sg * c[v][1 + D] + ps * c[v][1 + s] + pt * c[v][1 + t];
        Prim<double, NC> pin, pout;
        cons_to_prim<double, NC>(U, pin);
        double mu, kt;
        transport<NC>(pin, mu, kt);
        bnd_cond<double, NC>(bid, pin, pout, n);
        double fu, fv, fw, ft;
        if (noslip) {
            fu = fv = fw = 0.;
            ft = c_cfg.bnd_par[bid][0];
        } else {
            fu = (pin.u + pout.u) * 0.5; fv = (pin.v + pout.v) * 0.5;
            fw = (pin.w + pout.w) * 0.5; ft = (pin.t + pout.t) * 0.5;
        }
        double fc[NC];
#pragma unroll
        for (int k = 0; k < NC; k++) fc[k] = (pin.c[k] + pout.c[k]) * 0.5;
        double q[9];
        vgrad_q<NC>(mu, kt, (pin.r + pout.r) * 0.5, ft, fu, fv, fw, fc, dm, n, q);
#pragma unroll
        for (int r = 0; r < 9; r++) {
            S0[r] += q[r];
            Ss[r] += q[r] * ps;
            St[r] += q[r] * pt;
        }
    }
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int r = 0; r < 9; r++) {
        const double wr = (r < 6) ? w : -w;
        s9[(int64_t) (r * kNB + 0) * S + slot] = wr * S0[r];
        s9[(int64_t) (r * kNB + 1 + D) * S + slot] = 0.5 * sg * wr * S0[r];
        s9[(int64_t) (r * kNB + 1 + s) * S + slot] = wr * Ss[r];
        s9[(int64_t) (r * kNB + 1 + t) * S + slot] = wr * St[r];
    }
}

template <int NC>
__global__ void __launch_bounds__(128)
vgrad_face_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ dif, double *__restrict__ s9,
                  int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: vgrad_interior<NC, 0>(m, u, dif, s9, i); break;
        case 1: vgrad_interior<NC, 1>(m, u, dif, s9, i); break;
        default: vgrad_interior<NC, 2>(m, u, dif, s9, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        switch (m.bface_face[j] >> 1) {
        case 0: vgrad_boundary<NC, 0>(m, u, dif, s9, j); break;
        case 1: vgrad_boundary<NC, 1>(m, u, dif, s9, j); break;
        default: vgrad_boundary<NC, 2>(m, u, dif, s9, j); break;
        }
    }
}

// volume term (diff_grad.c:21-77) + gather + A^-1 -> vis [9][B][E]
template <int NC>
__global__ void __launch_bounds__(128)
vgrad_cell_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ dif,
                  const double *__restrict__ s9, double *__restrict__ vis)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double vol = hx * hy * hz, w8 = vol * 0.125;
    double c[V][kNB], dm[NC];
    load_coef<double, V>(u, E, e, c);
#pragma unroll
    for (int k = 0; k < NC; k++) dm[k] = dif[(int64_t) k * E + e];
    double a[9][kNB];
#pragma unroll
    for (int f = 0; f < 9; f++)
#pragma unroll
        for (int k = 0; k < kNB; k++) a[f][k] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 8; g++) {
        const double px = (g & 1) ? kGaussPhi : -kGaussPhi;
        const double py = (g & 2) ? kGaussPhi : -kGaussPhi;
        const double pz = (g & 4) ? kGaussPhi : -kGaussPhi;
        double U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        double kt, mu;
        transport<NC>(p, mu, kt);
        const double lp = 4. * mu / 3., lm = -2. * mu / 3.;
        double hq = kt * p.t;
#pragma unroll
        for (int i = 0; i < NC; i++) hq += comp_h(i, p.t) * p.r * dm[i] * p.c[i];
        // basis derivatives are 1/h_d on coefficient 1+d, zero elsewhere
        const double dx = w8 / hx, dy = w8 / hy, dz = w8 / hz;
        a[0][1] -= lp * p.u * dx; a[0][2] -= lm * p.v * dy; a[0][3] -= lm * p.w * dz;
        a[1][1] -= lm * p.u * dx; a[1][2] -= lp * p.v * dy; a[1][3] -= lm * p.w * dz;
        a[2][1] -= lm * p.u * dx; a[2][2] -= lm * p.v * dy; a[2][3] -= lp * p.w * dz;
        a[3][1] -= mu * p.v * dx; a[3][2] -= mu * p.u * dy;
        a[4][1] -= mu * p.w * dx; a[4][3] -= mu * p.u * dz;
        a[5][2] -= mu * p.w * dy; a[5][3] -= mu * p.v * dz;
        a[6][1] += hq * dx;
        a[7][2] += hq * dy;
        a[8][3] += hq * dz;
    }
    const int32_t g0 = m.gather_ptr[e], g1 = m.gather_ptr[e + 1];
    const int64_t S = m.n_slot;
    for (int32_t j = g0; j < g1; j++) {
        const int64_t sl = m.gather_slot[j];
#pragma unroll
        for (int f = 0; f < 9; f++)
#pragma unroll
            for (int k = 0; k < kNB; k++) a[f][k] += s9[(int64_t) (f * kNB + k) * S + sl];
    }
    const double minv0 = 1.0 / vol, minv1 = 12.0 / vol;
#pragma unroll
    for (int f = 0; f < 9; f++)
#pragma unroll
        for (int k = 0; k < kNB; k++) vis[(int64_t) (f * kNB + k) * E + e] = a[f][k] * (k ? minv1 : minv0);
}

// ---------------------------------------------------------------------------
// viscous integrals
// ---------------------------------------------------------------------------

// tau (6) and q (3) at the basis values phi of element e
__device__ __forceinline__ void vis_at(const double *__restrict__ vis, int64_t E, int64_t e, const double phi[4],
                                       double t[9])
{
#pragma unroll
    for (int f = 0; f < 9; f++) {
        double x = 0.0;
#pragma unroll
        for (int k = 0; k < kNB; k++) x += __ldg(vis + (int64_t) (f * kNB + k) * E + e) * phi[k];
        t[f] = x;
    }
}

template <int NC, int D>
__device__ __forceinline__ void vflux_interior(const MeshDev &m, const double *__restrict__ u,
                                               const double *__restrict__ vis, double *__restrict__ slots, int64_t i)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e[2] = {m.face_elem[i], m.face_elem[m.n_face + i]};
    const unsigned info = m.face_info[i];
    const int kind = (info >> 2) & 3, sub = (info >> 4) & 3;
    const int lev = m.level[(kind == 2) ? e[1] : e[0]];
    const double w = level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0);
    const double os = (sub & 1) ? 0.25 : -0.25, ot = (sub & 2) ? 0.25 : -0.25;
    const double gg[2] = {(kind == 2) ? 0.5 : 1.0, (kind == 1) ? 0.5 : 1.0};
    const double hs[2] = {(kind == 2) ? os : 0.0, (kind == 1) ? os : 0.0};
    const double ht[2] = {(kind == 2) ? ot : 0.0, (kind == 1) ? ot : 0.0};
    double S0[4], Ss[4], St[4];
#pragma unroll
    for (int v = 0; v < 4; v++) S0[v] = Ss[v] = St[v] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const double ps = face_ps<double>(g), pt = face_pt<double>(g);
        double t6[6] = {0., 0., 0., 0., 0., 0.}, fu = 0., fv = 0., fw = 0., ft = 0.;
#pragma unroll
        for (int sd = 0; sd < 2; sd++) {
            const double phi[4] = {1.0, 0.0, 0.0, 0.0};
            double ph[4] = {phi[0], 0.0, 0.0, 0.0};
            ph[1 + D] = sd ? -0.5 : 0.5;
            ph[1 + s] = gg[sd] * ps + hs[sd];
            ph[1 + t] = gg[sd] * pt + ht[sd];
            double U[V];
#pragma unroll
            for (int v = 0; v < V; v++) {
                double x = 0.0;
#pragma unroll
                for (int k = 0; k < kNB; k++) x += __ldg(u + (int64_t) (v * kNB + k) * E + e[sd]) * ph[k];
                U[v] = x;
            }
            Prim<double, NC> p;
            cons_to_prim<double, NC>(U, p);
            double tq[9];
            vis_at(vis, E, e[sd], ph, tq);
#pragma unroll
            for (int c = 0; c < 6; c++) t6[c] += tq[c];
            fu += p.u * tq[0] + p.v * tq[3] + p.w * tq[4];
            fv += p.u * tq[3] + p.v * tq[1] + p.w * tq[5];
            fw += p.u * tq[4] + p.v * tq[5] + p.w * tq[2];
            ft += tq[6 + D];   // q . n with n = e_D
        }
#pragma unroll
        for (int c = 0; c < 6; c++) t6[c] *= 0.5;
        fu *= 0.5; fv *= 0.5; fw *= 0.5; ft *= 0.5;
        // rows of tau along n = e_D: xx xy xz / xy yy yz / xz yz zz
        constexpr int r0 = (D == 0) ? 0 : (D == 1) ? 3 : 4;
        constexpr int r1 = (D == 0) ? 3 : (D == 1) ? 1 : 5;
        constexpr int r2 = (D == 0) ? 4 : (D == 1) ? 5 : 2;
        const double fl[4] = {t6[r0], t6[r1], t6[r2], ((D == 0) ? fu : (D == 1) ? fv : fw) - ft};
#pragma unroll
        for (int v = 0; v < 4; v++) {
            S0[v] += fl[v];
            Ss[v] += fl[v] * ps;
            St[v] += fl[v] * pt;
        }
    }
    // the residual gets -flux * phi * w on side 0 and +flux * phi * w on side 1
    const int64_t base = 2 * i;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        const double a0 = w * S0[v], as = w * Ss[v], at = w * St[v];
        double2 *p;
        p = reinterpret_cast<double2 *>(slots + (int64_t) (v * kNB + 0) * S + base);
        p->x -= a0; p->y += a0;
        p = reinterpret_cast<double2 *>(slots + (int64_t) (v * kNB + 1 + D) * S + base);
        p->x -= 0.5 * a0; p->y -= 0.5 * a0;
        p = reinterpret_cast<double2 *>(slots + (int64_t) (v * kNB + 1 + s) * S + base);
        p->x -= gg[0] * as + hs[0] * a0; p->y += gg[1] * as + hs[1] * a0;
        p = reinterpret_cast<double2 *>(slots + (int64_t) (v * kNB + 1 + t) * S + base);
        p->x -= gg[0] * at + ht[0] * a0; p->y += gg[1] * at + ht[1] * a0;
    }
}

// no-slip wall: one point at the face centre (diff_integrals.c:58-126)
template <int NC>
__device__ __forceinline__ void vflux_noslip(const MeshDev &m, const double *__restrict__ u,
                                             const double *__restrict__ vis, double *__restrict__ slots, int64_t j)
{
    constexpr int V = 4 + NC;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j];
    const int d = f >> 1;
    const double sg = (f & 1) ? 1.0 : -1.0;
    const int lev = m.level[e];
    const double hd = level_h(m, lev, d);
    const double area = level_h(m, lev, (d + 1) % 3) * level_h(m, lev, (d + 2) % 3);
    double ph[4] = {1.0, 0.0, 0.0, 0.0};
    ph[1 + d] = 0.5 * sg;
    double U[V], Um[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
        Um[v] = __ldg(u + (int64_t) (v * kNB) * E + e);
        U[v] = Um[v] + ph[1 + d] * __ldg(u + (int64_t) (v * kNB + 1 + d) * E + e);
    }
    Prim<double, NC> px, pm;
    cons_to_prim<double, NC>(U, px);
    cons_to_prim<double, NC>(Um, pm);
    const double mu = visc_mu<NC>(px);
    double tq[9];
    vis_at(vis, E, e, ph, tq);
    const double vv[3] = {pm.u, pm.v, pm.w};
    const double un = vv[d] * sg;
    double vt[3] = {vv[0], vv[1], vv[2]};
    vt[d] -= un * sg;
    const double ll = 0.5 * hd;
    const double fl[4] = {-mu * vt[0] / ll, -mu * vt[1] / ll, -mu * vt[2] / ll, -tq[6 + d] * sg};
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        slots[(int64_t) (v * kNB + 0) * S + slot] -= fl[v] * area;
        slots[(int64_t) (v * kNB + 1 + d) * S + slot] -= fl[v] * ph[1 + d] * area;
    }
}

template <int NC>
__global__ void __launch_bounds__(128)
vflux_face_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ vis, double *__restrict__ slots,
                  int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: vflux_interior<NC, 0>(m, u, vis, slots, i); break;
        case 1: vflux_interior<NC, 1>(m, u, vis, slots, i); break;
        default: vflux_interior<NC, 2>(m, u, vis, slots, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        if (c_cfg.bnd_type[m.bface_bnd[j]] == CHARM_GPU_BND_WALL_NO_SLIP) vflux_noslip<NC>(m, u, vis, slots, j);
    }
}

// viscous volume terms (diff_integrals.c:21-55) -> radd [4][B][E]
template <int NC>
__global__ void __launch_bounds__(128)
vvol_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ vis,
            const double *__restrict__ chem_rhs, double *__restrict__ radd)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double w8 = hx * hy * hz * 0.125;
    const double dx = w8 / hx, dy = w8 / hy, dz = w8 / hz;
    const double cr = chem_rhs ? chem_rhs[e] : 0.0;
    double c[V][kNB];
    load_coef<double, V>(u, E, e, c);
    double R[4][kNB];
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) R[v][k] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 8; g++) {
        const double ph[4] = {1.0, (g & 1) ? kGaussPhi : -kGaussPhi, (g & 2) ? kGaussPhi : -kGaussPhi,
                              (g & 4) ? kGaussPhi : -kGaussPhi};
        double U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + ph[1] * c[v][1] + ph[2] * c[v][2] + ph[3] * c[v][3];
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        double tq[9];
        vis_at(vis, E, e, ph, tq);
        R[0][1] += tq[0] * dx; R[0][2] += tq[3] * dy; R[0][3] += tq[4] * dz;
        R[1][1] += tq[3] * dx; R[1][2] += tq[1] * dy; R[1][3] += tq[5] * dz;
        R[2][1] += tq[4] * dx; R[2][2] += tq[5] * dy; R[2][3] += tq[2] * dz;
        R[3][1] += (tq[0] * p.u + tq[3] * p.v + tq[4] * p.w) * dx;
        R[3][2] += (tq[3] * p.u + tq[1] * p.v + tq[5] * p.w) * dy;
        R[3][3] += (tq[4] * p.u + tq[5] * p.v + tq[2] * p.w) * dz;
#pragma unroll
        for (int k = 0; k < kNB; k++) R[3][k] += cr * ph[k] * w8;
    }
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) radd[(int64_t) (v * kNB + k) * E + e] = R[v][k];
}

}  // namespace charm
