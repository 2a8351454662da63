// p2 path (FP64): the 10-function Taylor basis of charm_base_func
// (src/charm_base_func.c:8-125 with CHARM_BASE_FN_COUNT = 10) on boxes,
// with a 27-point (3x3x3 Gauss) cell rule and a 9-point (3x3 Gauss) face
// rule: the reference's 8/6-point rules under-integrate p2.  Uniform
// (conforming) meshes; convective, viscous and chemistry terms.
//
// State [V][10][E]; slots [V*10][S] with the p1 face-record layout.  The
// kernels mirror the p1 ones (face pass into per-side slots, element-owned
// gather, no atomics); basis values come from the rule tables in c_p2 and
// the closed-form basis below, the mass matrix is the reference element's
// (the same for every box up to its volume), inverted once on the host.
#pragma once

namespace charm {

constexpr int kNB2 = 10;

struct P2Tab {
    double cxi[27][3];        // cell points in reference coordinates, [-1/2, 1/2]^3, x fastest
    double cw[27];            // cell weights, sum 1
    double fxi[9][2];         // face points (lower, upper tangential axis), [-1/2, 1/2]^2
    double fw[9];             // face weights, sum 1
    double minv[kNB2][kNB2];  // inverse mass matrix of the reference box (volume 1)
    double mean[kNB2];        // cell mean of each basis function
};

__constant__ P2Tab c_p2;

// basis values at reference coordinates (x, y, z) = (x - c) / h
__device__ __forceinline__ void basis10(double x, double y, double z, double phi[kNB2])
{
    phi[0] = 1.0; phi[1] = x; phi[2] = y; phi[3] = z;
    phi[4] = x * x; phi[5] = y * y; phi[6] = z * z;
    phi[7] = x * y; phi[8] = x * z; phi[9] = y * z;
}

// d phi / d(reference coordinate a)
__device__ __forceinline__ void grad10(double x, double y, double z, double g[3][kNB2])
{
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) g[a][k] = 0.0;
    g[0][1] = 1.0; g[1][2] = 1.0; g[2][3] = 1.0;
    g[0][4] = 2.0 * x; g[1][5] = 2.0 * y; g[2][6] = 2.0 * z;
    g[0][7] = y; g[1][7] = x;
    g[0][8] = z; g[2][8] = x;
    g[1][9] = z; g[2][9] = y;
}

// point on face D of a box: the normal coordinate xd, tangential (xs, xt)
template <int D>
__device__ __forceinline__ void face_basis10(double xd, double xs, double xt, double phi[kNB2])
{
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    double r[3];
    r[D] = xd; r[s] = xs; r[t] = xt;
    basis10(r[0], r[1], r[2], phi);
}

template <int V>
__device__ __forceinline__ void eval10(const double *__restrict__ u, int64_t E, int64_t e, const double phi[kNB2],
                                       double U[V])
{
#pragma unroll
    for (int v = 0; v < V; v++) {
        double x = 0.0;
#pragma unroll
        for (int k = 0; k < kNB2; k++) x += __ldg(u + (int64_t) (v * kNB2 + k) * E + e) * phi[k];
        U[v] = x;
    }
}

// ---------------------------------------------------------------------------
// convective face pass
// ---------------------------------------------------------------------------

template <int NC, int FLUX, int D>
__device__ __forceinline__ void p2_interior(const MeshDev &m, const double *__restrict__ u, double *__restrict__ slots,
                                            int64_t i, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e0 = m.face_elem[i], e1 = m.face_elem[m.n_face + i];
    const int lev = m.level[e0];
    const double area = level_h(m, lev, s) * level_h(m, lev, t);
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = 1.0;
    double q9[9][V];
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        double p0[kNB2], p1[kNB2], U0[V], U1[V];
        face_basis10<D>(0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p0);
        face_basis10<D>(-0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p1);
        eval10<V>(u, E, e0, p0, U0);
        eval10<V>(u, E, e1, p1, U1);
        Prim<double, NC> pa, pb;
        cons_to_prim<double, NC>(U0, pa);
        cons_to_prim<double, NC>(U1, pb);
        double q[V];
        num_flux<FLUX, double, NC, D>(pa, pb, n, q, err);
        const double w = area * c_p2.fw[g];
#pragma unroll
        for (int v = 0; v < V; v++) q9[g][v] = q[v] * w;
    }
    const int64_t base = 2 * i;
#pragma unroll 1
    for (int k = 0; k < kNB2; k++) {
        double a0[V], a1[V];
#pragma unroll
        for (int v = 0; v < V; v++) a0[v] = a1[v] = 0.0;
#pragma unroll 1
        for (int g = 0; g < 9; g++) {
            double p0[kNB2], p1[kNB2];
            face_basis10<D>(0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p0);
            face_basis10<D>(-0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p1);
#pragma unroll
            for (int v = 0; v < V; v++) {
                a0[v] += q9[g][v] * p0[k];
                a1[v] -= q9[g][v] * p1[k];
            }
        }
#pragma unroll
        for (int v = 0; v < V; v++) store_pair<double>(slots, (int64_t) (v * kNB2 + k) * S + base, a0[v], a1[v]);
    }
}

template <int NC, int FLUX, int D>
__device__ __forceinline__ void p2_boundary(const MeshDev &m, const double *__restrict__ u, double *__restrict__ slots,
                                            int64_t j, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
    const double sg = (f & 1) ? 1.0 : -1.0;
    const int lev = m.level[e];
    const double area = level_h(m, lev, s) * level_h(m, lev, t);
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = sg;
    double q9[9][V];
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        double ph[kNB2], U[V];
        face_basis10<D>(0.5 * sg, c_p2.fxi[g][0], c_p2.fxi[g][1], ph);
        eval10<V>(u, E, e, ph, U);
        Prim<double, NC> pin, pout;
        cons_to_prim<double, NC>(U, pin);
        bnd_cond<double, NC>(bid, pin, pout, n);
        double q[V];
        num_flux<FLUX, double, NC, D>(pin, pout, n, q, err);
        const double w = area * c_p2.fw[g];
#pragma unroll
        for (int v = 0; v < V; v++) q9[g][v] = q[v] * w;
    }
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll 1
    for (int k = 0; k < kNB2; k++) {
        double a[V];
#pragma unroll
        for (int v = 0; v < V; v++) a[v] = 0.0;
#pragma unroll 1
        for (int g = 0; g < 9; g++) {
            double ph[kNB2];
            face_basis10<D>(0.5 * sg, c_p2.fxi[g][0], c_p2.fxi[g][1], ph);
#pragma unroll
            for (int v = 0; v < V; v++) a[v] += q9[g][v] * ph[k];
        }
#pragma unroll
        for (int v = 0; v < V; v++) slots[(int64_t) (v * kNB2 + k) * S + slot] = a[v];
    }
}

template <int NC, int FLUX>
__global__ void __launch_bounds__(128)
p2_face_kernel(MeshDev m, const double *__restrict__ u, double *__restrict__ slots, int64_t n_int_blocks, unsigned *err)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: p2_interior<NC, FLUX, 0>(m, u, slots, i, err); break;
        case 1: p2_interior<NC, FLUX, 1>(m, u, slots, i, err); break;
        default: p2_interior<NC, FLUX, 2>(m, u, slots, i, err); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        switch (m.bface_face[j] >> 1) {
        case 0: p2_boundary<NC, FLUX, 0>(m, u, slots, j, err); break;
        case 1: p2_boundary<NC, FLUX, 1>(m, u, slots, j, err); break;
        default: p2_boundary<NC, FLUX, 2>(m, u, slots, j, err); break;
        }
    }
}

// ---------------------------------------------------------------------------
// cell pass: volume integral (27 points), gather, M^-1, update
// ---------------------------------------------------------------------------
// mode kCellUpdate:   out = a_new*(u - dt*M^-1*(R + radd)) + a_old*u0
// mode kCellResidual: out = R + radd
template <int NC>
__global__ void __launch_bounds__(128)
p2_cell_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ slots, const double *u0,
               double *out, double dt, const double *__restrict__ dt_dev, double a_new, double a_old, int mode,
               unsigned *err, const double *__restrict__ radd)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double vol = hx * hy * hz;
    const bool grav = c_cfg.has_grav != 0;
    double R[V][kNB2];
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) R[v][k] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 27; g++) {
        const double x = c_p2.cxi[g][0], y = c_p2.cxi[g][1], z = c_p2.cxi[g][2];
        double ph[kNB2], gr[3][kNB2], U[V];
        basis10(x, y, z, ph);
        grad10(x, y, z, gr);
        eval10<V>(u, E, e, ph, U);
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        if (!(p.r > 0.0) || !(p.p > 0.0)) set_error(err, isfinite(p.r) && isfinite(p.p) ? kErrNegative : kErrNonFinite);
        double F[V], G[V], H[V];
        F[0] = U[0] * p.u + p.p; F[1] = U[0] * p.v; F[2] = U[0] * p.w; F[3] = U[0] * p.e_tot + p.p * p.u;
        G[0] = U[1] * p.u; G[1] = U[1] * p.v + p.p; G[2] = U[1] * p.w; G[3] = U[1] * p.e_tot + p.p * p.v;
        H[0] = U[2] * p.u; H[1] = U[2] * p.v; H[2] = U[2] * p.w + p.p; H[3] = U[2] * p.e_tot + p.p * p.w;
#pragma unroll
        for (int c = 0; c < NC; c++) { F[4 + c] = U[0] * p.c[c]; G[4 + c] = U[1] * p.c[c]; H[4 + c] = U[2] * p.c[c]; }
        const double w = vol * c_p2.cw[g];
        const double wx = w / hx, wy = w / hy, wz = w / hz;
#pragma unroll
        for (int k = 1; k < kNB2; k++) {
            const double dx = gr[0][k] * wx, dy = gr[1][k] * wy, dz = gr[2][k] * wz;
#pragma unroll
            for (int v = 0; v < V; v++) R[v][k] -= F[v] * dx + G[v] * dy + H[v] * dz;
        }
        if (grav) {
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int k = 0; k < kNB2; k++) R[a][k] -= p.r * c_cfg.grav[a] * ph[k] * w;
        }
    }
    const int32_t g0 = m.gather_ptr[e], g1 = m.gather_ptr[e + 1];
    const int64_t S = m.n_slot;
    for (int32_t j = g0; j < g1; j++) {
        const int64_t sl = m.gather_slot[j];
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB2; k++) R[v][k] += slots[(int64_t) (v * kNB2 + k) * S + sl];
    }
    if (radd) {
#pragma unroll
        for (int v = 0; v < 4; v++)
#pragma unroll
            for (int k = 0; k < kNB2; k++) R[v][k] += __ldg(radd + (int64_t) (v * kNB2 + k) * E + e);
    }
    if (mode == kCellResidual) {
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB2; k++) out[(int64_t) (v * kNB2 + k) * E + e] = R[v][k];
        return;
    }
    const double step = dt_dev ? *dt_dev : dt;
    const bool comb = (a_old != 0.0);
    const double iv = 1.0 / vol;
#pragma unroll 1
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int i = 0; i < kNB2; i++) {
            double r = 0.0;
#pragma unroll
            for (int j = 0; j < kNB2; j++) r += c_p2.minv[i][j] * R[v][j];
            const int64_t idx = (int64_t) (v * kNB2 + i) * E + e;
            double x = __ldg(u + idx) - step * (r * iv);
            if (comb) x = a_new * x + a_old * u0[idx];
            out[idx] = x;
        }
    }
}

// ---------------------------------------------------------------------------
// chemistry and diffusion coefficients (cell means of the p2 field)
// ---------------------------------------------------------------------------

template <int NC>
__global__ void __launch_bounds__(128)
p2_chem_kernel(MeshDev m, const double *__restrict__ u, double *__restrict__ out, double *__restrict__ chem_rhs)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double U[V];
    eval10<V>(u, E, e, c_p2.mean, U);   // charm_get_fields_avg
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
    for (int j = 0; j < 2; j++) {
#pragma unroll
        for (int i = 0; i < NC; i++) c_[i] = (ch[i] + c[i]) * 0.5;
        chem_rates<NC>(p.t, c_, k, w, phi, psi);
#pragma unroll
        for (int i = 0; i < NC; i++) {
            ch[i] = (c[i] + dt * psi[i] * (1. + dt * phi[i] * 0.5));
            ch[i] /= (1. + dt * phi[i] + (dt * phi[i]) * (dt * phi[i]) * 0.5);
        }
    }
    chem_rates<NC>(p.t, ch, k, w, nullptr, nullptr);
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
        for (int kk = 0; kk < kNB2; kk++)
            out[(int64_t) (v * kNB2 + kk) * E + e] = __ldg(u + (int64_t) (v * kNB2 + kk) * E + e);
#pragma unroll
    for (int i = 0; i < NC; i++) {
        out[(int64_t) ((4 + i) * kNB2) * E + e] = ch[i] * c_cfg.comp_m[i];
#pragma unroll
        for (int kk = 1; kk < kNB2; kk++) out[(int64_t) ((4 + i) * kNB2 + kk) * E + e] = 0.;
    }
}

// ---------------------------------------------------------------------------
// viscous terms (the p1 kernels' arithmetic on the p2 basis)
// ---------------------------------------------------------------------------

template <int NC, int D>
__device__ __forceinline__ void p2_vgrad_interior(const MeshDev &m, const double *__restrict__ u,
                                                  const double *__restrict__ dif, double *__restrict__ s9, int64_t i)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e0 = m.face_elem[i], e1 = m.face_elem[m.n_face + i];
    const int lev = m.level[e0];
    const double area = level_h(m, lev, s) * level_h(m, lev, t);
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = 1.0;
    double dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = (dif[(int64_t) c * E + e0] + dif[(int64_t) c * E + e1]) * 0.5;
    double q9[9][9];   // [point][field], weight included, heat rows negated
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        double p0[kNB2], p1[kNB2], Ua[V], Ub[V];
        face_basis10<D>(0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p0);
        face_basis10<D>(-0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p1);
        eval10<V>(u, E, e0, p0, Ua);
        eval10<V>(u, E, e1, p1, Ub);
        Prim<double, NC> pa, pb;
        cons_to_prim<double, NC>(Ua, pa);
        cons_to_prim<double, NC>(Ub, pb);
        double mua, kta, mub, ktb;
        transport<NC>(pa, mua, kta);
        transport<NC>(pb, mub, ktb);
        double fc[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) fc[c] = (pa.c[c] + pb.c[c]) * 0.5;
        double q[9];
        vgrad_q<NC>(0.5 * (mua + mub), (kta + ktb) * 0.5, (pa.r + pb.r) * 0.5, (pa.t + pb.t) * 0.5,
                    (pa.u + pb.u) * 0.5, (pa.v + pb.v) * 0.5, (pa.w + pb.w) * 0.5, fc, dm, n, q);
        const double w = area * c_p2.fw[g];
#pragma unroll
        for (int f = 0; f < 9; f++) q9[g][f] = (f < 6 ? w : -w) * q[f];
    }
    const int64_t base = 2 * i;
#pragma unroll 1
    for (int k = 0; k < kNB2; k++) {
        double a0[9], a1[9];
#pragma unroll
        for (int f = 0; f < 9; f++) a0[f] = a1[f] = 0.0;
#pragma unroll 1
        for (int g = 0; g < 9; g++) {
            double p0[kNB2], p1[kNB2];
            face_basis10<D>(0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p0);
            face_basis10<D>(-0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p1);
#pragma unroll
            for (int f = 0; f < 9; f++) {
                a0[f] += q9[g][f] * p0[k];
                a1[f] -= q9[g][f] * p1[k];
            }
        }
#pragma unroll
        for (int f = 0; f < 9; f++) store_pair<double>(s9, (int64_t) (f * kNB2 + k) * S + base, a0[f], a1[f]);
    }
}

template <int NC, int D>
__device__ __forceinline__ void p2_vgrad_boundary(const MeshDev &m, const double *__restrict__ u,
                                                  const double *__restrict__ dif, double *__restrict__ s9, int64_t j)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
    const double sg = (f & 1) ? 1.0 : -1.0;
    const int lev = m.level[e];
    const double area = level_h(m, lev, s) * level_h(m, lev, t);
    const bool noslip = c_cfg.bnd_type[bid] == CHARM_GPU_BND_WALL_NO_SLIP;
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = sg;
    double dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = dif[(int64_t) c * E + e];
    double q9[9][9];
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        double ph[kNB2], U[V];
        face_basis10<D>(0.5 * sg, c_p2.fxi[g][0], c_p2.fxi[g][1], ph);
        eval10<V>(u, E, e, ph, U);
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
        for (int c = 0; c < NC; c++) fc[c] = (pin.c[c] + pout.c[c]) * 0.5;
        double q[9];
        vgrad_q<NC>(mu, kt, (pin.r + pout.r) * 0.5, ft, fu, fv, fw, fc, dm, n, q);
        const double w = area * c_p2.fw[g];
#pragma unroll
        for (int r = 0; r < 9; r++) q9[g][r] = (r < 6 ? w : -w) * q[r];
    }
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll 1
    for (int k = 0; k < kNB2; k++) {
        double a[9];
#pragma unroll
        for (int r = 0; r < 9; r++) a[r] = 0.0;
#pragma unroll 1
        for (int g = 0; g < 9; g++) {
            double ph[kNB2];
            face_basis10<D>(0.5 * sg, c_p2.fxi[g][0], c_p2.fxi[g][1], ph);
#pragma unroll
            for (int r = 0; r < 9; r++) a[r] += q9[g][r] * ph[k];
        }
#pragma unroll
        for (int r = 0; r < 9; r++) s9[(int64_t) (r * kNB2 + k) * S + slot] = a[r];
    }
}

template <int NC>
__global__ void __launch_bounds__(128)
p2_vgrad_face_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ dif, double *__restrict__ s9,
                     int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: p2_vgrad_interior<NC, 0>(m, u, dif, s9, i); break;
        case 1: p2_vgrad_interior<NC, 1>(m, u, dif, s9, i); break;
        default: p2_vgrad_interior<NC, 2>(m, u, dif, s9, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        switch (m.bface_face[j] >> 1) {
        case 0: p2_vgrad_boundary<NC, 0>(m, u, dif, s9, j); break;
        case 1: p2_vgrad_boundary<NC, 1>(m, u, dif, s9, j); break;
        default: p2_vgrad_boundary<NC, 2>(m, u, dif, s9, j); break;
        }
    }
}

// lifting volume term + gather + M^-1 -> vis [9][10][E]
template <int NC>
__global__ void __launch_bounds__(128)
p2_vgrad_cell_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ dif,
                     const double *__restrict__ s9, double *__restrict__ vis)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double vol = hx * hy * hz;
    double dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = dif[(int64_t) c * E + e];
    double a[9][kNB2];
#pragma unroll
    for (int f = 0; f < 9; f++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) a[f][k] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 27; g++) {
        const double x = c_p2.cxi[g][0], y = c_p2.cxi[g][1], z = c_p2.cxi[g][2];
        double ph[kNB2], gr[3][kNB2], U[V];
        basis10(x, y, z, ph);
        grad10(x, y, z, gr);
        eval10<V>(u, E, e, ph, U);
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        double kt, mu;
        transport<NC>(p, mu, kt);
        const double lp = 4. * mu / 3., lm = -2. * mu / 3.;
        double hq = kt * p.t;
#pragma unroll
        for (int c = 0; c < NC; c++) hq += comp_h(c, p.t) * p.r * dm[c] * p.c[c];
        const double w = vol * c_p2.cw[g];
#pragma unroll
        for (int k = 1; k < kNB2; k++) {
            const double px = gr[0][k] * w / hx, py = gr[1][k] * w / hy, pz = gr[2][k] * w / hz;
            a[0][k] -= (lp * p.u * px + lm * p.v * py + lm * p.w * pz);
            a[1][k] -= (lm * p.u * px + lp * p.v * py + lm * p.w * pz);
            a[2][k] -= (lm * p.u * px + lm * p.v * py + lp * p.w * pz);
            a[3][k] -= mu * (p.u * py + p.v * px);
            a[4][k] -= mu * (p.w * px + p.u * pz);
            a[5][k] -= mu * (p.w * py + p.v * pz);
            a[6][k] += hq * px;
            a[7][k] += hq * py;
            a[8][k] += hq * pz;
        }
    }
    const int32_t g0 = m.gather_ptr[e], g1 = m.gather_ptr[e + 1];
    const int64_t S = m.n_slot;
    for (int32_t j = g0; j < g1; j++) {
        const int64_t sl = m.gather_slot[j];
#pragma unroll
        for (int f = 0; f < 9; f++)
#pragma unroll
            for (int k = 0; k < kNB2; k++) a[f][k] += s9[(int64_t) (f * kNB2 + k) * S + sl];
    }
    const double iv = 1.0 / vol;
#pragma unroll 1
    for (int f = 0; f < 9; f++)
#pragma unroll
        for (int i = 0; i < kNB2; i++) {
            double r = 0.0;
#pragma unroll
            for (int j = 0; j < kNB2; j++) r += c_p2.minv[i][j] * a[f][j];
            vis[(int64_t) (f * kNB2 + i) * E + e] = r * iv;
        }
}

__device__ __forceinline__ void vis_at10(const double *__restrict__ vis, int64_t E, int64_t e, const double phi[kNB2],
                                         double t[9])
{
#pragma unroll
    for (int f = 0; f < 9; f++) {
        double x = 0.0;
#pragma unroll
        for (int k = 0; k < kNB2; k++) x += __ldg(vis + (int64_t) (f * kNB2 + k) * E + e) * phi[k];
        t[f] = x;
    }
}

template <int NC, int D>
__device__ __forceinline__ void p2_vflux_interior(const MeshDev &m, const double *__restrict__ u,
                                                  const double *__restrict__ vis, double *__restrict__ slots, int64_t i)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e[2] = {m.face_elem[i], m.face_elem[m.n_face + i]};
    const int lev = m.level[e[0]];
    const double area = level_h(m, lev, s) * level_h(m, lev, t);
    constexpr int r0 = (D == 0) ? 0 : (D == 1) ? 3 : 4;
    constexpr int r1 = (D == 0) ? 3 : (D == 1) ? 1 : 5;
    constexpr int r2 = (D == 0) ? 4 : (D == 1) ? 5 : 2;
    double q9[9][4];
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        double t6[6] = {0., 0., 0., 0., 0., 0.}, fu = 0., fv = 0., fw = 0., ft = 0.;
#pragma unroll
        for (int sd = 0; sd < 2; sd++) {
            double ph[kNB2], U[V], tq[9];
            face_basis10<D>(sd ? -0.5 : 0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], ph);
            eval10<V>(u, E, e[sd], ph, U);
            Prim<double, NC> p;
            cons_to_prim<double, NC>(U, p);
            vis_at10(vis, E, e[sd], ph, tq);
#pragma unroll
            for (int c = 0; c < 6; c++) t6[c] += tq[c];
            fu += p.u * tq[0] + p.v * tq[3] + p.w * tq[4];
            fv += p.u * tq[3] + p.v * tq[1] + p.w * tq[5];
            fw += p.u * tq[4] + p.v * tq[5] + p.w * tq[2];
            ft += tq[6 + D];
        }
        const double w = area * c_p2.fw[g];
        q9[g][0] = 0.5 * t6[r0] * w;
        q9[g][1] = 0.5 * t6[r1] * w;
        q9[g][2] = 0.5 * t6[r2] * w;
        q9[g][3] = (0.5 * ((D == 0) ? fu : (D == 1) ? fv : fw) - 0.5 * ft) * w;
    }
    const int64_t base = 2 * i;
#pragma unroll 1
    for (int k = 0; k < kNB2; k++) {
        double a0[4] = {0., 0., 0., 0.}, a1[4] = {0., 0., 0., 0.};
#pragma unroll 1
        for (int g = 0; g < 9; g++) {
            double p0[kNB2], p1[kNB2];
            face_basis10<D>(0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p0);
            face_basis10<D>(-0.5, c_p2.fxi[g][0], c_p2.fxi[g][1], p1);
#pragma unroll
            for (int v = 0; v < 4; v++) {
                a0[v] += q9[g][v] * p0[k];
                a1[v] += q9[g][v] * p1[k];
            }
        }
        // the residual gets -flux phi0 on side 0 and +flux phi1 on side 1
#pragma unroll
        for (int v = 0; v < 4; v++) {
            double2 *p = reinterpret_cast<double2 *>(slots + (int64_t) (v * kNB2 + k) * S + base);
            p->x -= a0[v];
            p->y += a1[v];
        }
    }
}

template <int NC>
__device__ __forceinline__ void p2_vflux_noslip(const MeshDev &m, const double *__restrict__ u,
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
    double r[3] = {0.0, 0.0, 0.0};
    r[d] = 0.5 * sg;
    double ph[kNB2], U[V], Um[V], tq[9];
    basis10(r[0], r[1], r[2], ph);
    eval10<V>(u, E, e, ph, U);
    eval10<V>(u, E, e, c_p2.mean, Um);
    Prim<double, NC> px, pm;
    cons_to_prim<double, NC>(U, px);
    cons_to_prim<double, NC>(Um, pm);
    double mu, kt;
    transport<NC>(px, mu, kt);
    vis_at10(vis, E, e, ph, tq);
    const double vv[3] = {pm.u, pm.v, pm.w};
    const double un = vv[d] * sg;
    double vt[3] = {vv[0], vv[1], vv[2]};
    vt[d] -= un * sg;
    const double ll = 0.5 * hd;
    const double fl[4] = {-mu * vt[0] / ll, -mu * vt[1] / ll, -mu * vt[2] / ll, -tq[6 + d] * sg};
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) slots[(int64_t) (v * kNB2 + k) * S + slot] -= fl[v] * ph[k] * area;
}

template <int NC>
__global__ void __launch_bounds__(128)
p2_vflux_face_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ vis,
                     double *__restrict__ slots, int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: p2_vflux_interior<NC, 0>(m, u, vis, slots, i); break;
        case 1: p2_vflux_interior<NC, 1>(m, u, vis, slots, i); break;
        default: p2_vflux_interior<NC, 2>(m, u, vis, slots, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        if (c_cfg.bnd_type[m.bface_bnd[j]] == CHARM_GPU_BND_WALL_NO_SLIP) p2_vflux_noslip<NC>(m, u, vis, slots, j);
    }
}

// viscous volume terms (27 points) + chem_rhs -> radd [4][10][E]
template <int NC>
__global__ void __launch_bounds__(128)
p2_vvol_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ vis,
               const double *__restrict__ chem_rhs, double *__restrict__ radd)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double vol = hx * hy * hz;
    const double cr = chem_rhs ? chem_rhs[e] : 0.0;
    double R[4][kNB2];
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) R[v][k] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 27; g++) {
        const double x = c_p2.cxi[g][0], y = c_p2.cxi[g][1], z = c_p2.cxi[g][2];
        double ph[kNB2], gr[3][kNB2], U[V], tq[9];
        basis10(x, y, z, ph);
        grad10(x, y, z, gr);
        eval10<V>(u, E, e, ph, U);
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        vis_at10(vis, E, e, ph, tq);
        const double w = vol * c_p2.cw[g];
        const double ex = tq[0] * p.u + tq[3] * p.v + tq[4] * p.w;
        const double ey = tq[3] * p.u + tq[1] * p.v + tq[5] * p.w;
        const double ez = tq[4] * p.u + tq[5] * p.v + tq[2] * p.w;
#pragma unroll
        for (int k = 0; k < kNB2; k++) {
            const double px = gr[0][k] * w / hx, py = gr[1][k] * w / hy, pz = gr[2][k] * w / hz;
            R[0][k] += tq[0] * px + tq[3] * py + tq[4] * pz;
            R[1][k] += tq[3] * px + tq[1] * py + tq[5] * pz;
            R[2][k] += tq[4] * px + tq[5] * py + tq[2] * pz;
            R[3][k] += ex * px + ey * py + ez * pz + cr * ph[k] * w;
        }
    }
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) radd[(int64_t) (v * kNB2 + k) * E + e] = R[v][k];
}

}  // namespace charm
