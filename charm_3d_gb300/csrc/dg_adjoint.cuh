// Discrete adjoint of the DG time step on sm_103a (FP64).
//
// One forward stage is  s = u - dt M^-1 R(u),  u' = a L(s) + b u^n  (L the
// limiter, identity without one).  Its reverse, for a given adjoint s^ of s,
// is  u^ = s^ + (dR/du)^T r^  with  r^ = -dt M^-1 s^,  which the two kernels
// below compute in the layout of the forward ones:
//
//   adj_face_kernel : for every interior face / mortar sub-face / boundary
//                     face, the adjoint trace q^ = w (sum_k r^_k phi_k) of
//                     both sides at the 6 face points, the flux VJP (dq/dU)^T
//                     q^ at each point, projected on the basis of each side
//                     -> slots (the forward kernel's slot layout, no atomics)
//   adj_cell_kernel : the volume-flux VJP at the 8 Gauss points, the gather
//                     of the element's slots, + s^, then the combination with
//                     the previous stage (limiter scaling frozen at the
//                     forward psi: the active set is not differentiated)
//
// The pointwise derivatives are in adjoint_math.h (tested on the host
// against differences of the oracle's fluxes).
#pragma once

#include "adjoint_math.h"

namespace charm {

__device__ __forceinline__ adj::Gas adj_gas()
{
    return adj::Gas{c_cfg.ideal_gam, c_cfg.ideal_inv_cv, c_cfg.ideal_m, kGasR, kEps};
}

// r^ of element e: coef * M^-1 (when scale_minv) * s^
template <int V>
__device__ __forceinline__ void adj_rbar(const MeshDev &m, const double *__restrict__ sh, int64_t e, double coef,
                                         int scale_minv, double rb[V][kNB])
{
    const int64_t E = m.n_elem;
    double s0 = coef, s1 = coef;
    if (scale_minv) {
        const int lev = m.level[e];
        const double vol = level_h(m, lev, 0) * level_h(m, lev, 1) * level_h(m, lev, 2);
        const double iv = rcp_nr(vol);   // the flux path's reciprocal: no division per element side
        s0 = coef * iv;
        s1 = coef * 12.0 * iv;
    }
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) rb[v][k] = __ldg(sh + (int64_t) (v * kNB + k) * E + e) * (k ? s1 : s0);
}

template <int NC, int FLUX, int D>
__device__ __forceinline__ void adj_interior(const MeshDev &m, const double *__restrict__ u,
                                             const double *__restrict__ sh, double coef, int scale_minv,
                                             double *__restrict__ slots, int64_t i)
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
    // tangential scale/offset of each side's basis: phi_s = gs * ps + hs
    const double g0 = (kind == 2) ? 0.5 : 1.0, g1 = (kind == 1) ? 0.5 : 1.0;
    const double hs0 = (kind == 2) ? os : 0.0, ht0 = (kind == 2) ? ot : 0.0;
    const double hs1 = (kind == 1) ? os : 0.0, ht1 = (kind == 1) ? ot : 0.0;
    // adjoint trace q^(ps, pt) = A + B ps + C pt
    double A[V], B[V], C[V];
    {
        double r0[V][kNB], r1[V][kNB];
        adj_rbar<V>(m, sh, e0, coef, scale_minv, r0);
        adj_rbar<V>(m, sh, e1, coef, scale_minv, r1);
#pragma unroll
        for (int v = 0; v < V; v++) {
            A[v] = w * ((r0[v][0] + 0.5 * r0[v][1 + D] + hs0 * r0[v][1 + s] + ht0 * r0[v][1 + t]) -
                        (r1[v][0] - 0.5 * r1[v][1 + D] + hs1 * r1[v][1 + s] + ht1 * r1[v][1 + t]));
            B[v] = w * (g0 * r0[v][1 + s] - g1 * r1[v][1 + s]);
            C[v] = w * (g0 * r0[v][1 + t] - g1 * r1[v][1 + t]);
        }
    }
    const int64_t base = 2 * i;
    {
        // outside the support of the adjoint the trace is exactly zero, and so
        // is the contribution (linear in q^): skip the face
        bool live = false;
#pragma unroll
        for (int v = 0; v < V; v++) live |= (A[v] != 0.0) | (B[v] != 0.0) | (C[v] != 0.0);
        if (!live) {
#pragma unroll
            for (int v = 0; v < V; v++)
#pragma unroll
                for (int k = 0; k < kNB; k++) store_pair<double>(slots, (int64_t) (v * kNB + k) * S + base, 0.0, 0.0);
            return;
        }
    }
    const adj::Gas gas = adj_gas();
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = 1.0;
    double S0a[V], Ssa[V], Sta[V], S0b[V], Ssb[V], Stb[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0a[v] = Ssa[v] = Sta[v] = S0b[v] = Ssb[v] = Stb[v] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const double ps = face_ps<double>(g), pt = face_pt<double>(g);
        const double ps0 = g0 * ps + hs0, pt0 = g0 * pt + ht0, ps1 = g1 * ps + hs1, pt1 = g1 * pt + ht1;
        double Ua[V], Ub[V], qb[V], Uab[V], Ubb[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            const int64_t p0 = (int64_t) (v * kNB) * E;
            Ua[v] = __ldg(u + p0 + e0) + 0.5 * __ldg(u + p0 + (int64_t) (1 + D) * E + e0) +
                    ps0 * __ldg(u + p0 + (int64_t) (1 + s) * E + e0) + pt0 * __ldg(u + p0 + (int64_t) (1 + t) * E + e0);
            Ub[v] = __ldg(u + p0 + e1) - 0.5 * __ldg(u + p0 + (int64_t) (1 + D) * E + e1) +
                    ps1 * __ldg(u + p0 + (int64_t) (1 + s) * E + e1) + pt1 * __ldg(u + p0 + (int64_t) (1 + t) * E + e1);
            qb[v] = A[v] + B[v] * ps + C[v] * pt;
        }
        adj::point_vjp<NC, D>(FLUX, Ua, Ub, n, gas, qb, Uab, Ubb, nullptr);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0a[v] += Uab[v]; Ssa[v] += Uab[v] * ps; Sta[v] += Uab[v] * pt;
            S0b[v] += Ubb[v]; Ssb[v] += Ubb[v] * ps; Stb[v] += Ubb[v] * pt;
        }
    }
#pragma unroll
    for (int v = 0; v < V; v++) {
        store_pair<double>(slots, (int64_t) (v * kNB + 0) * S + base, S0a[v], S0b[v]);
        store_pair<double>(slots, (int64_t) (v * kNB + 1 + D) * S + base, 0.5 * S0a[v], -0.5 * S0b[v]);
        store_pair<double>(slots, (int64_t) (v * kNB + 1 + s) * S + base, g0 * Ssa[v] + hs0 * S0a[v],
                           g1 * Ssb[v] + hs1 * S0b[v]);
        store_pair<double>(slots, (int64_t) (v * kNB + 1 + t) * S + base, g0 * Sta[v] + ht0 * S0a[v],
                           g1 * Stb[v] + ht1 * S0b[v]);
    }
}

template <int NC, int FLUX, int D>
__device__ __forceinline__ void adj_boundary(const MeshDev &m, const double *__restrict__ u,
                                             const double *__restrict__ sh, double coef, int scale_minv,
                                             double *__restrict__ slots, int64_t j)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
    const double sg = (f & 1) ? 1.0 : -1.0;
    const int lev = m.level[e];
    const double w = level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0);
    double A[V], B[V], C[V], c[V][kNB];
    {
        double r[V][kNB];
        adj_rbar<V>(m, sh, e, coef, scale_minv, r);
#pragma unroll
        for (int v = 0; v < V; v++) {
            A[v] = w * (r[v][0] + 0.5 * sg * r[v][1 + D]);
            B[v] = w * r[v][1 + s];
            C[v] = w * r[v][1 + t];
        }
    }
    const int64_t slot = 2 * m.n_face + j;
    {
        bool live = false;
#pragma unroll
        for (int v = 0; v < V; v++) live |= (A[v] != 0.0) | (B[v] != 0.0) | (C[v] != 0.0);
        if (!live) {
#pragma unroll
            for (int v = 0; v < V; v++)
#pragma unroll
                for (int k = 0; k < kNB; k++) slots[(int64_t) (v * kNB + k) * S + slot] = 0.0;
            return;
        }
    }
    load_coef<double, V>(u, E, e, c);
    const adj::Gas gas = adj_gas();
    double n[3] = {0.0, 0.0, 0.0};
    n[D] = sg;
    const int type = c_cfg.bnd_type[bid];
    const double *par = c_cfg.bnd_par[bid];
    double S0[V], Ss[V], St[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const double ps = face_ps<double>(g), pt = face_pt<double>(g);
        double U[V], qb[V], Ub[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            U[v] = c[v][0] + 0.5 * sg * c[v][1 + D] + ps * c[v][1 + s] + pt * c[v][1 + t];
            qb[v] = A[v] + B[v] * ps + C[v] * pt;
        }
        adj::bpoint_vjp<NC, D>(FLUX, type, par, U, n, gas, qb, Ub, nullptr);
#pragma unroll
        for (int v = 0; v < V; v++) { S0[v] += Ub[v]; Ss[v] += Ub[v] * ps; St[v] += Ub[v] * pt; }
    }
#pragma unroll
    for (int v = 0; v < V; v++) {
        slots[(int64_t) (v * kNB + 0) * S + slot] = S0[v];
        slots[(int64_t) (v * kNB + 1 + D) * S + slot] = 0.5 * sg * S0[v];
        slots[(int64_t) (v * kNB + 1 + s) * S + slot] = Ss[v];
        slots[(int64_t) (v * kNB + 1 + t) * S + slot] = St[v];
    }
}

// Blocks [0, n_int_blocks) take interior faces, the rest boundary faces.
template <int NC, int FLUX>
__global__ void __launch_bounds__(128)
adj_face_kernel(MeshDev m, const double *__restrict__ u, const double *__restrict__ sh, double coef, int scale_minv,
                double *__restrict__ slots, int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: adj_interior<NC, FLUX, 0>(m, u, sh, coef, scale_minv, slots, i); break;
        case 1: adj_interior<NC, FLUX, 1>(m, u, sh, coef, scale_minv, slots, i); break;
        default: adj_interior<NC, FLUX, 2>(m, u, sh, coef, scale_minv, slots, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        switch (m.bface_face[j] >> 1) {
        case 0: adj_boundary<NC, FLUX, 0>(m, u, sh, coef, scale_minv, slots, j); break;
        case 1: adj_boundary<NC, FLUX, 1>(m, u, sh, coef, scale_minv, slots, j); break;
        default: adj_boundary<NC, FLUX, 2>(m, u, sh, coef, scale_minv, slots, j); break;
        }
    }
}

enum { kAdjResidual = 0, kAdjStage = 1, kAdjFinal = 2 };

// lam = base * s^ + (dR/du)^T r^ for element e, then
//   kAdjResidual: out = lam
//   kAdjStage:    out = psi (.) (a_next * lam)  (psi scales coefficients 1..3;
//                 none when psi is null);  acc += b_next * lam  (when b_next != 0)
//   kAdjFinal:    out = lam + acc  (acc may be null)
// out may be sh itself (each element reads only its own s^ before writing).
template <int NC>
__global__ void __launch_bounds__(128)
adj_cell_kernel(MeshDev m, const double *__restrict__ u, const double *sh, double coef, int scale_minv,
                const double *__restrict__ slots, double base, int mode, const double *__restrict__ psi,
                double a_next, double b_next, double *acc, double *out)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double w8 = hx * hy * hz * 0.125;
    double lam[V][kNB];
    double a[3][V];
    double grb[kNB];   // gravity: -w8 * sum_a g_a * r^[a][k] per basis function k
    {
        double rb[V][kNB];
        adj_rbar<V>(m, sh, e, coef, scale_minv, rb);
#pragma unroll
        for (int v = 0; v < V; v++) {
            a[0][v] = -(hy * hz * 0.125) * rb[v][1];   // (vol / 8) / h_a as a product
            a[1][v] = -(hx * hz * 0.125) * rb[v][2];
            a[2][v] = -(hx * hy * 0.125) * rb[v][3];
#pragma unroll
            for (int k = 0; k < kNB; k++) lam[v][k] = base * __ldg(sh + (int64_t) (v * kNB + k) * E + e);
        }
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            double x = 0.0;
#pragma unroll
            for (int d = 0; d < 3; d++) x += c_cfg.grav[d] * rb[d][k];
            grb[k] = -w8 * x;
        }
    }
    const bool grav = c_cfg.has_grav != 0;
    bool live = false;   // r^ = 0: the volume term contributes exactly zero
#pragma unroll
    for (int v = 0; v < V; v++) live |= (a[0][v] != 0.0) | (a[1][v] != 0.0) | (a[2][v] != 0.0);
#pragma unroll
    for (int k = 0; k < kNB; k++) live |= grav && (grb[k] != 0.0);
    const adj::Gas gas = adj_gas();
    double c[V][kNB];
    if (live) load_coef<double, V>(u, E, e, c);
#pragma unroll 1
    for (int g = 0; g < (live ? 8 : 0); g++) {
        const double px = (g & 1) ? kGaussPhi : -kGaussPhi;
        const double py = (g & 2) ? kGaussPhi : -kGaussPhi;
        const double pz = (g & 4) ? kGaussPhi : -kGaussPhi;
        double U[V], Ub[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
            Ub[v] = 0.0;
        }
        adj::vpoint_vjp<NC>(U, gas, a, Ub);
        if (grav) {
            // R[a][k] -= w8 rho g_a phi_k,  rho = sum_i U[4+i]
            const double x = grb[0] + grb[1] * px + grb[2] * py + grb[3] * pz;
#pragma unroll
            for (int i = 0; i < NC; i++) Ub[4 + i] += x;
        }
#pragma unroll
        for (int v = 0; v < V; v++) {
            lam[v][0] += Ub[v];
            lam[v][1] += px * Ub[v];
            lam[v][2] += py * Ub[v];
            lam[v][3] += pz * Ub[v];
        }
    }
    const int32_t s0 = m.gather_ptr[e], s1 = m.gather_ptr[e + 1];
    const int64_t S = m.n_slot;
    for (int32_t j = s0; j < s1; j++) {
        const int64_t sl = m.gather_slot[j];
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) lam[v][k] += slots[(int64_t) (v * kNB + k) * S + sl];
    }
#pragma unroll
    for (int v = 0; v < V; v++) {
        const double ps = (mode == kAdjStage && psi) ? psi[(int64_t) v * E + e] : 1.0;
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            const double x = lam[v][k];
            if (mode == kAdjResidual) {
                out[idx] = x;
            } else if (mode == kAdjStage) {
                if (b_next != 0.0) acc[idx] += b_next * x;
                out[idx] = (k ? ps : 1.0) * (a_next * x);
            } else {
                out[idx] = acc ? x + acc[idx] : x;
            }
        }
    }
}

// s^ = psi (.) (a * lam), acc = b * lam  (the adjoint of the last stage's
// combination u' = a L(s) + b u^n).  psi may be null.
__global__ void __launch_bounds__(256)
adj_init_kernel(const double *__restrict__ lam, const double *__restrict__ psi, double a, double b, int V, int64_t E,
                double *__restrict__ sh, double *__restrict__ acc)
{
    const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t) V * kNB * E) return;
    const int64_t plane = i / E, e = i - plane * E;
    const int v = (int) (plane / kNB), k = (int) (plane % kNB);
    const double x = lam[i];
    const double ps = (psi && k) ? psi[(int64_t) v * E + e] : 1.0;
    sh[i] = ps * (a * x);
    if (acc) acc[i] = b * x;
}

// Objective J = integral of the pressure over the elements whose centre lies
// in [lo, hi) (8-point Gauss rule), and its gradient dJ/du.  One partial sum
// per block (fixed order), summed on the host.
template <int NC>
__global__ void __launch_bounds__(128)
adj_objective_kernel(MeshDev m, const double *__restrict__ u, double lo0, double lo1, double lo2, double hi0,
                     double hi1, double hi2, double *__restrict__ partial, double *__restrict__ grad)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    double Je = 0.0;
    if (e < E) {
        const double cx = m.center[e], cy = m.center[E + e], cz = m.center[2 * E + e];
        const bool in = cx >= lo0 && cx < hi0 && cy >= lo1 && cy < hi1 && cz >= lo2 && cz < hi2;
        double lam[V][kNB];
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) lam[v][k] = 0.0;
        if (in) {
            const int lev = m.level[e];
            const double w8 = level_h(m, lev, 0) * level_h(m, lev, 1) * level_h(m, lev, 2) * 0.125;
            const adj::Gas gas = adj_gas();
            double c[V][kNB];
            load_coef<double, V>(u, E, e, c);
            for (int g = 0; g < 8; g++) {
                const double px = (g & 1) ? kGaussPhi : -kGaussPhi;
                const double py = (g & 2) ? kGaussPhi : -kGaussPhi;
                const double pz = (g & 4) ? kGaussPhi : -kGaussPhi;
                double U[V], Ub[V];
#pragma unroll
                for (int v = 0; v < V; v++) {
                    U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
                    Ub[v] = 0.0;
                }
                adj::Pr<NC> p;
                adj::prim<NC, 0>(U, gas, p);
                Je += w8 * p.p;
                adj::PrBar<NC> b;
                adj::zero<NC>(b);
                b.p = w8;
                adj::prim_vjp<NC, 0>(U, p, gas, b, Ub);
#pragma unroll
                for (int v = 0; v < V; v++) {
                    lam[v][0] += Ub[v];
                    lam[v][1] += px * Ub[v];
                    lam[v][2] += py * Ub[v];
                    lam[v][3] += pz * Ub[v];
                }
            }
        }
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) grad[(int64_t) (v * kNB + k) * E + e] = lam[v][k];
    }
    __shared__ double red[128];
    red[threadIdx.x] = Je;
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if ((int) threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Weight of the adjoint-weighted refinement indicator: |dJ/d(density mean)|
// per unit volume, w[e] = |sum_i lam[rc_i][0][e]| / vol_e.
__global__ void __launch_bounds__(256)
adj_weight_kernel(MeshDev m, const double *__restrict__ lam, int n_comp, double *__restrict__ w)
{
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double x = 0.0;
    for (int i = 0; i < n_comp; i++) x += lam[(int64_t) ((4 + i) * kNB) * E + e];
    const int lev = m.level[e];
    w[e] = fabs(x) / (level_h(m, lev, 0) * level_h(m, lev, 1) * level_h(m, lev, 2));
}

}  // namespace charm
