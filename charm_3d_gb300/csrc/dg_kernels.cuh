// Kernels of the DG time step on sm_103a.
//
// Data layout in HBM (E = elements, V = 4 + n_comp, B = 4):
//   state      double [V][B][E]   one coalesced plane per (variable, coefficient)
//   center     double [3][E], level int8 [E]; h = tree_len * 2^-level
//   faces      int32 [2][F] (side 0 lower, side 1 upper), uint8 info [F]
//   bfaces     int32 elem, int8 face, int8 bnd
//   slots      T [V*B][S]: one flux projection per (face, side); S = 2F + Fb
//              (rounded up to even).  Side 0 and side 1 of interior face i
//              are slots 2i, 2i+1, written as one 2-vector store.
//   gather     CSR over elements listing the slots that belong to each one
//
// The three kernels of one RK stage:
//   face_kernel   : Riemann flux at the 6 face points of every interior
//                   face / mortar sub-face / boundary face, projected on the
//                   basis of each side -> slots (no atomics).
//   cell_kernel   : volume integral at the 8 Gauss points, gather of the
//                   element's slots, M^-1 and the RK update (and the SSP
//                   combination when no limiter follows).
//   limit_kernel  : Barth-Jespersen limiter on the updated state, fused with
//                   the SSP combination.
//
// Geometry on this path is axis-aligned boxes, so the basis values at every
// quadrature point are the constants below; the reference computes them
// from trilinear-mapped points (src/charm_geom.c:40-172, 443-494), which
// agrees to rounding.
#pragma once

#include "dg_device.cuh"

namespace charm {

// Face quadrature: two triangles x 3 points, weights 1/6, jacobian
// 2*area(triangle) (reference src/charm_geom.c:443-494).  In face-local
// coordinates (s, t) on [0,1]^2, s = the lower tangential axis:
__constant__ double c_face_s[6] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0, 5.0 / 6.0};
__constant__ double c_face_t[6] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0, 5.0 / 6.0, 5.0 / 6.0};

// Cell quadrature: 2x2x2 Gauss points at +-1/sqrt(3) of the half edge, x
// fastest (reference src/charm_geom.c:139-155).  Taylor basis value there:
// (x - c)/dh = +-1/(2 sqrt 3).
constexpr double kGaussPhi = 0.28867513459481288225;   // 1/(2*sqrt(3))

struct MeshDev {
    int64_t n_elem, n_face, n_bface, n_slot;
    const double  *center;       // [3][E]
    const int8_t  *level;        // [E]
    const int32_t *face_elem;    // [2][F]
    const uint8_t *face_info;    // [F]
    const int32_t *bface_elem;
    const int8_t  *bface_face;
    const int8_t  *bface_bnd;
    const int32_t *gather_ptr;   // [E+1]
    const int32_t *gather_slot;  // [gather_ptr[E]]
    const int32_t *lim_idx;      // [6][E]
    const int8_t  *lim_kind;     // [6][E]  0 same, 1 boundary, 2 big side of mortar, 3 small side
    double tree_len[3];
};

__device__ __forceinline__ double level_h(const MeshDev &m, int lev, int d)
{
    return ldexp(m.tree_len[d], -lev);
}

template <typename T>
__device__ __forceinline__ T ld_state(const double *u, int64_t plane, int64_t E, int64_t e)
{
    return T(__ldg(u + plane * E + e));
}

// ---------------------------------------------------------------------------
// face kernel
// ---------------------------------------------------------------------------

// Load the V x 4 coefficients of element e.
template <typename T, int V>
__device__ __forceinline__ void load_coef(const double *u, int64_t E, int64_t e, T c[V][kNB])
{
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) c[v][k] = ld_state<T>(u, v * kNB + k, E, e);
}

template <typename T>
__device__ __forceinline__ void store_pair(T *slots, int64_t idx, T a, T b);
template <>
__device__ __forceinline__ void store_pair<double>(double *slots, int64_t idx, double a, double b)
{
    *reinterpret_cast<double2 *>(slots + idx) = make_double2(a, b);
}
template <>
__device__ __forceinline__ void store_pair<float>(float *slots, int64_t idx, float a, float b)
{
    *reinterpret_cast<float2 *>(slots + idx) = make_float2(a, b);
}

// Interior face i along axis D (compile-time, so that the coefficient arrays
// stay in registers).
template <typename T, int NC, int FLUX, int D>
__device__ __forceinline__ void interior_face(const MeshDev &m, const double *__restrict__ u, T *__restrict__ slots,
                                              int64_t i, int e0, int e1, unsigned info, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot;
    const int kind = (info >> 2) & 3, sub = (info >> 4) & 3;
    // the leaf that owns the quadrature points: side 0 unless side 1 is
    // the small leaf of a mortar (src/models/euler/charm_model.c:282-285)
    const int ep = (kind == 2) ? e1 : e0;
    const int lev = m.level[ep];
    const T w = T(level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0));
    // tangential offsets of the big side in a mortar
    const T os = T((sub & 1) ? 0.25 : -0.25), ot = T((sub & 2) ? 0.25 : -0.25);

    T c0[V][kNB], c1[V][kNB];
    load_coef<T, V>(u, m.n_elem, e0, c0);
    load_coef<T, V>(u, m.n_elem, e1, c1);

    // n points from side 0 to side 1 (+e_D), as the reference's flipped
    // side-0 face normal (src/models/euler/charm_model.c:268-280)
    T n[3] = {T(0), T(0), T(0)};
    n[D] = T(1);

    T S0[V], Ss[V], St[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = T(0);

#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const T ps = T(c_face_s[g] - 0.5), pt = T(c_face_t[g] - 0.5);
        // tangential basis values on each side
        T ps0 = ps, pt0 = pt, ps1 = ps, pt1 = pt;
        if (kind == 1) { ps1 = T(0.5) * ps + os; pt1 = T(0.5) * pt + ot; }
        if (kind == 2) { ps0 = T(0.5) * ps + os; pt0 = T(0.5) * pt + ot; }
        T U0[V], U1[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            U0[v] = c0[v][0] + T(0.5) * c0[v][1 + D] + ps0 * c0[v][1 + s] + pt0 * c0[v][1 + t];
            U1[v] = c1[v][0] - T(0.5) * c1[v][1 + D] + ps1 * c1[v][1 + s] + pt1 * c1[v][1 + t];
        }
        Prim<T, NC> p0, p1;
        cons_to_prim<T, NC>(U0, p0);
        cons_to_prim<T, NC>(U1, p1);
        T q[V];
        num_flux<FLUX, T, NC>(p0, p1, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
    // project: side 0 gets +w*sum(q*phi), side 1 gets -w*sum(q*phi)
    const int64_t base = 2 * i;
#pragma unroll
    for (int v = 0; v < V; v++) {
        T a0 = w * S0[v];
        T as = w * Ss[v], at = w * St[v];
        T as0 = as, at0 = at, as1 = as, at1 = at;
        if (kind == 1) { as1 = T(0.5) * as + os * a0; at1 = T(0.5) * at + ot * a0; }
        if (kind == 2) { as0 = T(0.5) * as + os * a0; at0 = T(0.5) * at + ot * a0; }
        store_pair<T>(slots, (int64_t) (v * kNB + 0) * S + base, a0, -a0);
        store_pair<T>(slots, (int64_t) (v * kNB + 1 + D) * S + base, T(0.5) * a0, T(0.5) * a0);
        store_pair<T>(slots, (int64_t) (v * kNB + 1 + s) * S + base, as0, -as1);
        store_pair<T>(slots, (int64_t) (v * kNB + 1 + t) * S + base, at0, -at1);
    }
}

// Boundary face j on axis D; sg = -1 for the lower face, +1 for the upper.
template <typename T, int NC, int FLUX, int D>
__device__ __forceinline__ void boundary_face(const MeshDev &m, const double *__restrict__ u, T *__restrict__ slots,
                                              int64_t j, int e, T sg, int bid, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot;
    const int lev = m.level[e];
    const T w = T(level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0));
    T c[V][kNB];
    load_coef<T, V>(u, m.n_elem, e, c);
    // outward normal (src/models/euler/charm_model.c:175-187)
    T n[3] = {T(0), T(0), T(0)};
    n[D] = sg;
    T S0[V], Ss[V], St[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = T(0);
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const T ps = T(c_face_s[g] - 0.5), pt = T(c_face_t[g] - 0.5);
        T U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + T(0.5) * sg * c[v][1 + D] + ps * c[v][1 + s] + pt * c[v][1 + t];
        Prim<T, NC> pin, pout;
        cons_to_prim<T, NC>(U, pin);
        bnd_cond<T, NC>(bid, pin, pout, n);
        T q[V];
        num_flux<FLUX, T, NC>(pin, pout, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int v = 0; v < V; v++) {
        T a0 = w * S0[v];
        slots[(int64_t) (v * kNB + 0) * S + slot] = a0;
        slots[(int64_t) (v * kNB + 1 + D) * S + slot] = T(0.5) * sg * a0;
        slots[(int64_t) (v * kNB + 1 + s) * S + slot] = w * Ss[v];
        slots[(int64_t) (v * kNB + 1 + t) * S + slot] = w * St[v];
    }
}

// Blocks [0, n_int_blocks) take interior faces, the rest boundary faces
// (a block-uniform split).  Faces are stored grouped by axis, so the switch
// on the axis is warp-uniform almost everywhere.
template <typename T, int NC, int FLUX>
__global__ void __launch_bounds__(128)
face_kernel(MeshDev m, const double *__restrict__ u, T *__restrict__ slots, int64_t n_int_blocks,
            unsigned *err)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        const int e0 = m.face_elem[i], e1 = m.face_elem[m.n_face + i];
        const unsigned info = m.face_info[i];
        switch (info & 3) {
        case 0: interior_face<T, NC, FLUX, 0>(m, u, slots, i, e0, e1, info, err); break;
        case 1: interior_face<T, NC, FLUX, 1>(m, u, slots, i, e0, e1, info, err); break;
        default: interior_face<T, NC, FLUX, 2>(m, u, slots, i, e0, e1, info, err); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        const int e = m.bface_elem[j];
        const int f = m.bface_face[j], bid = m.bface_bnd[j];
        const T sg = (f & 1) ? T(1) : T(-1);
        switch (f >> 1) {
        case 0: boundary_face<T, NC, FLUX, 0>(m, u, slots, j, e, sg, bid, err); break;
        case 1: boundary_face<T, NC, FLUX, 1>(m, u, slots, j, e, sg, bid, err); break;
        default: boundary_face<T, NC, FLUX, 2>(m, u, slots, j, e, sg, bid, err); break;
        }
    }
}

// ---------------------------------------------------------------------------
// cell kernel: volume integral + gather + M^-1 + update
// ---------------------------------------------------------------------------

enum { kCellUpdate = 0, kCellResidual = 1 };

// mode kCellUpdate:   out = a_new*(u - dt*M^-1*R(u)) + a_old*u0
// mode kCellResidual: out = R(u)  (the reference's int_* arrays)
template <typename T, int NC>
__global__ void __launch_bounds__(128)
cell_kernel(MeshDev m, const double *__restrict__ u, const T *__restrict__ slots, const double *u0,
            double *out, double dt, const double *__restrict__ dt_dev, double a_new, double a_old,
            int mode, unsigned *err)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double vol = hx * hy * hz;

    T c[V][kNB];
    load_coef<T, V>(u, E, e, c);

    // ---- volume integral (src/models/ns/charm_model_ns_conv.c:23-89) ----
    // int[v][1+a] -= (vol/8)/h_a * sum_gp F_a,v(gp); gravity adds to all k.
    T F[V], G[V], H[V];
#pragma unroll
    for (int v = 0; v < V; v++) F[v] = G[v] = H[v] = T(0);
    T gr[3][kNB];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int k = 0; k < kNB; k++) gr[a][k] = T(0);
    const bool grav = c_cfg.has_grav != 0;

#pragma unroll 1
    for (int g = 0; g < 8; g++) {
        const T px = T((g & 1) ? kGaussPhi : -kGaussPhi);
        const T py = T((g & 2) ? kGaussPhi : -kGaussPhi);
        const T pz = T((g & 4) ? kGaussPhi : -kGaussPhi);
        T U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
        Prim<T, NC> p;
        cons_to_prim<T, NC>(U, p);
        if (!(p.r > T(0)) || !(p.p > T(0))) set_error(err, isfinite((double) p.r) && isfinite((double) p.p) ? kErrNegative : kErrNonFinite);
        // Euler fluxes (src/models/ns/charm_model_ns_conv.c:45-65)
        F[0] += U[0] * p.u + p.p; F[1] += U[0] * p.v; F[2] += U[0] * p.w; F[3] += U[0] * p.e_tot + p.p * p.u;
        G[0] += U[1] * p.u; G[1] += U[1] * p.v + p.p; G[2] += U[1] * p.w; G[3] += U[1] * p.e_tot + p.p * p.v;
        H[0] += U[2] * p.u; H[1] += U[2] * p.v; H[2] += U[2] * p.w + p.p; H[3] += U[2] * p.e_tot + p.p * p.w;
#pragma unroll
        for (int i = 0; i < NC; i++) {
            F[4 + i] += U[0] * p.c[i];
            G[4 + i] += U[1] * p.c[i];
            H[4 + i] += U[2] * p.c[i];
        }
        if (grav) {
            const T phi[4] = {T(1), px, py, pz};
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int k = 0; k < kNB; k++) gr[a][k] += p.r * T(c_cfg.grav[a]) * phi[k];
        }
    }
    const double w8 = vol * 0.125;
    double R[V][kNB];
#pragma unroll
    for (int v = 0; v < V; v++) {
        R[v][0] = 0.0;
        R[v][1] = -(double) F[v] * (w8 / hx);
        R[v][2] = -(double) G[v] * (w8 / hy);
        R[v][3] = -(double) H[v] * (w8 / hz);
    }
    if (grav) {
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int k = 0; k < kNB; k++) R[a][k] -= (double) gr[a][k] * w8;
    }

    // ---- element-owned gather of face contributions ----
    const int32_t g0 = m.gather_ptr[e], g1 = m.gather_ptr[e + 1];
    const int64_t S = m.n_slot;
    T acc[V][kNB];
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) acc[v][k] = T(0);
    for (int32_t j = g0; j < g1; j++) {
        const int64_t sl = m.gather_slot[j];
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) acc[v][k] += slots[(int64_t) (v * kNB + k) * S + sl];
    }
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) R[v][k] += (double) acc[v][k];

    if (mode == kCellResidual) {
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) out[(int64_t) (v * kNB + k) * E + e] = R[v][k];
        return;
    }

    // ---- M^-1 (diagonal for the p1 Taylor basis on a box: vol, vol/12 x3)
    //      and update (src/models/ns/charm_model.c:68-99) ----
    const double step = dt_dev ? *dt_dev : dt;
    const double minv0 = 1.0 / vol, minv1 = 12.0 / vol;
    const bool comb = (a_old != 0.0);
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            const double cu = __ldg(u + idx);
            double x = cu - step * (R[v][k] * (k == 0 ? minv0 : minv1));
            if (comb) x = a_new * x + a_old * u0[idx];
            out[idx] = x;
        }
    }
}

// ---------------------------------------------------------------------------
// Barth-Jespersen limiter (src/limiters/charm_limiter_bj.c) + SSP combination
// ---------------------------------------------------------------------------
//
// Per element: bounds from its own mean and the six neighbour values
// (conforming: neighbour mean; boundary: BC ghost of the own mean; big side
// of a mortar: volume-weighted mean of the 4 small leaves' centre values;
// small side: the big leaf's centre value), psi = min over the 8 vertices,
// higher coefficients scaled by psi; then out = a_new*lim + a_old*u0.
// Means are the constant coefficient: the reference's 8-point quadrature
// mean equals c_0 up to rounding.  Species get the same treatment as the
// other variables at hanging faces (the reference leaves those slots stale,
// src/limiters/charm_limiter_bj.c:174-193).
template <int NC>
__global__ void __launch_bounds__(128)
limit_kernel(MeshDev m, const double *__restrict__ ua, const double *u0, double *out,
             double a_new, double a_old)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;

    double c[V][kNB];
    load_coef<double, V>(ua, E, e, c);
    double umin[V], umax[V];
#pragma unroll
    for (int v = 0; v < V; v++) umin[v] = umax[v] = c[v][0];

#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        const int kind = m.lim_kind[(int64_t) f * E + e];
        const int idx = m.lim_idx[(int64_t) f * E + e];
        double nbv[V];
        if (kind == 0 || kind == 3) {
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = __ldg(ua + (int64_t) (v * kNB) * E + idx);
        } else if (kind == 2) {
            // idx = first of the 4 sub-face records of this big face
            double svol = 0.0;
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = 0.0;
            for (int k = 0; k < 4; k++) {
                const int64_t fi = idx + k;
                const unsigned info = m.face_info[fi];
                const int small = (((info >> 2) & 3) == 1) ? m.face_elem[fi] : m.face_elem[m.n_face + fi];
                const int ls = m.level[small];
                const double vs = level_h(m, ls, 0) * level_h(m, ls, 1) * level_h(m, ls, 2);
                svol += vs;
#pragma unroll
                for (int v = 0; v < V; v++) nbv[v] += __ldg(ua + (int64_t) (v * kNB) * E + small) * vs;
            }
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] /= svol;
        } else {
            // boundary: ghost state of the own mean (charm_limiter_bj.c:79-91)
            const int fb = m.bface_face[idx], bid = m.bface_bnd[idx];
            double n[3] = {0.0, 0.0, 0.0};
            n[fb >> 1] = (fb & 1) ? 1.0 : -1.0;
            double U[V];
#pragma unroll
            for (int v = 0; v < V; v++) U[v] = c[v][0];
            Prim<double, NC> pin, pout;
            cons_to_prim<double, NC>(U, pin);
            bnd_cond<double, NC>(bid, pin, pout, n);
            prim_to_cons<double, NC>(pout, nbv);
        }
#pragma unroll
        for (int v = 0; v < V; v++) {
            if (umin[v] > nbv[v]) umin[v] = nbv[v];
            if (umax[v] < nbv[v]) umax[v] = nbv[v];
        }
    }

    // psi over the 8 vertices (charm_limiter_bj.c:275-299); basis = +-1/2
    double psi[V];
#pragma unroll
    for (int v = 0; v < V; v++) psi[v] = 1.0;
#pragma unroll
    for (int vx = 0; vx < 8; vx++) {
        const double sx = (vx & 1) ? 0.5 : -0.5, sy = (vx & 2) ? 0.5 : -0.5, sz = (vx & 4) ? 0.5 : -0.5;
#pragma unroll
        for (int v = 0; v < V; v++) {
            const double f = c[v][0] + sx * c[v][1] + sy * c[v][2] + sz * c[v][3];
            const double df = f - c[v][0];
            double pt = 1.0;
            if (fabs(df) > kEps) {
                if (df > 0) pt = fmin(1.0, (umax[v] - c[v][0]) / df);
                else if (df < 0) pt = fmin(1.0, (umin[v] - c[v][0]) / df);
            }
            if (pt < psi[v]) psi[v] = pt;
        }
    }
    const bool comb = (a_old != 0.0);
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            double x = (k == 0) ? c[v][0] : c[v][k] * psi[v];
            if (comb) x = a_new * x + a_old * u0[idx];
            out[idx] = x;
        }
    }
}

// ---------------------------------------------------------------------------
// CFL time step: min over cells of CFL*vol/(|u|+c) at the cell centre (the
// reference's unreachable get_dt code, src/models/ns/charm_model.c:21-36,
// 50-59).  Warp-shuffle + block min, one 64-bit atomicMin per block (the bit
// pattern of positive doubles orders like the values).
// ---------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(256)
cfl_dt_kernel(MeshDev m, const double *__restrict__ u, double cfl, unsigned long long *dt_bits)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    double dtl = 1.0e300;
    if (e < m.n_elem) {
        double U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = __ldg(u + (int64_t) (v * kNB) * m.n_elem + e);
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        const int lev = m.level[e];
        const double vol = level_h(m, lev, 0) * level_h(m, lev, 1) * level_h(m, lev, 2);
        dtl = cfl * vol / (sqrt(p.u * p.u + p.v * p.v + p.w * p.w) + p.cz);
        if (!(dtl > 0.0)) dtl = 1.0e300;
    }
    for (int o = 16; o > 0; o >>= 1) dtl = fmin(dtl, __shfl_xor_sync(0xffffffffu, dtl, o));
    __shared__ double red[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = dtl;
    __syncthreads();
    if (wid == 0) {
        dtl = (lane < (int) (blockDim.x >> 5)) ? red[lane] : 1.0e300;
        for (int o = 16; o > 0; o >>= 1) dtl = fmin(dtl, __shfl_xor_sync(0xffffffffu, dtl, o));
        if (lane == 0) atomicMin(dt_bits, (unsigned long long) __double_as_longlong(dtl));
    }
}

// ---------------------------------------------------------------------------
// Arithmetic peak probe: kPeakChains independent FMA chains per thread, the
// result stored so the compiler keeps them.  Used only to measure the
// roofline denominator of the CUDA-core pipes on the running GPU.
// ---------------------------------------------------------------------------
constexpr int kPeakChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T *out, int iters)
{
    T a[kPeakChains];
    const T x = T(1) + T(threadIdx.x) * T(1e-7), y = T(0.999999);
#pragma unroll
    for (int k = 0; k < kPeakChains; k++) a[k] = T(k) * T(1e-3);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kPeakChains; k++) a[k] = fma(a[k], y, x);
    }
    T s = T(0);
#pragma unroll
    for (int k = 0; k < kPeakChains; k++) s += a[k];
    out[(size_t) blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace charm
