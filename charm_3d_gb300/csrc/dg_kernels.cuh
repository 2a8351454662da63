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
static __constant__ double c_face_s[6] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0, 5.0 / 6.0};
static __constant__ double c_face_t[6] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0, 5.0 / 6.0, 5.0 / 6.0};
// the same points as float basis values s - 1/2, t - 1/2 (FP32 paths)
static __constant__ float c_face_psf[6] = {(float) (1.0 / 6.0 - 0.5), (float) (2.0 / 3.0 - 0.5), (float) (1.0 / 6.0 - 0.5),
                                    (float) (5.0 / 6.0 - 0.5), (float) (1.0 / 3.0 - 0.5), (float) (5.0 / 6.0 - 0.5)};
static __constant__ float c_face_ptf[6] = {(float) (1.0 / 6.0 - 0.5), (float) (1.0 / 6.0 - 0.5), (float) (2.0 / 3.0 - 0.5),
                                    (float) (1.0 / 3.0 - 0.5), (float) (5.0 / 6.0 - 0.5), (float) (5.0 / 6.0 - 0.5)};

// and as double basis values (the same doubles as c_face_s[g] - 0.5)
static __constant__ double c_face_psd[6] = {1.0 / 6.0 - 0.5, 2.0 / 3.0 - 0.5, 1.0 / 6.0 - 0.5,
                                            5.0 / 6.0 - 0.5, 1.0 / 3.0 - 0.5, 5.0 / 6.0 - 0.5};
static __constant__ double c_face_ptd[6] = {1.0 / 6.0 - 0.5, 1.0 / 6.0 - 0.5, 2.0 / 3.0 - 0.5,
                                            1.0 / 3.0 - 0.5, 5.0 / 6.0 - 0.5, 5.0 / 6.0 - 0.5};

// and as double-word values (hi, lo of the doubles above)
static __constant__ dw c_face_psw[6] = {dw(1.0 / 6.0 - 0.5), dw(2.0 / 3.0 - 0.5), dw(1.0 / 6.0 - 0.5),
                                        dw(5.0 / 6.0 - 0.5), dw(1.0 / 3.0 - 0.5), dw(5.0 / 6.0 - 0.5)};
static __constant__ dw c_face_ptw[6] = {dw(1.0 / 6.0 - 0.5), dw(1.0 / 6.0 - 0.5), dw(2.0 / 3.0 - 0.5),
                                        dw(1.0 / 3.0 - 0.5), dw(5.0 / 6.0 - 0.5), dw(5.0 / 6.0 - 0.5)};

template <typename T>
__device__ __forceinline__ T face_ps(int g)
{
    if constexpr (is_dw<T>) return c_face_psw[g];
    else if constexpr (sizeof(T) == sizeof(float)) return c_face_psf[g];
    else return c_face_psd[g];
}
template <typename T>
__device__ __forceinline__ T face_pt(int g)
{
    if constexpr (is_dw<T>) return c_face_ptw[g];
    else if constexpr (sizeof(T) == sizeof(float)) return c_face_ptf[g];
    else return c_face_ptd[g];
}

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
    const int8_t  *lim_kind;     // [6][E]  bits 0-1: 0 same, 1 boundary, 2 big side of mortar,
                                 // 3 small side (bits 4-5: its position in the big face)
    double tree_len[3];
    float  tree_len_f[3];
};

__device__ __forceinline__ double level_h(const MeshDev &m, int lev, int d)
{
    return ldexp(m.tree_len[d], -lev);
}

// edge length in the arithmetic type T (exact scaling by 2^-lev in both)
template <typename T>
__device__ __forceinline__ T level_ht(const MeshDev &m, int lev, int d)
{
    if constexpr (is_dw<T>) return dw(ldexp(m.tree_len[d], -lev));
    else if constexpr (sizeof(T) == sizeof(float)) return ldexpf(m.tree_len_f[d], -lev);
    else return ldexp(m.tree_len[d], -lev);
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
template <>
__device__ __forceinline__ void store_pair<dw>(dw *slots, int64_t idx, dw a, dw b)
{
    *reinterpret_cast<float4 *>(slots + idx) = make_float4(a.h, a.l, b.h, b.l);
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
    const T w = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t) * (T(1) / T(6));
    // tangential offsets of the big side in a mortar
    const T os = (sub & 1) ? T(0.25) : T(-0.25), ot = (sub & 2) ? T(0.25) : T(-0.25);

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
        const T ps = face_ps<T>(g), pt = face_pt<T>(g);
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
        num_flux<FLUX, T, NC, D>(p0, p1, n, q, err);
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
// T: the arithmetic, S: the slot type (S = dw with T = double: the
// double-word form evaluates its boundary faces, a surface's worth, in FP64)
template <typename T, int NC, int FLUX, int D, typename S = T>
__device__ __forceinline__ void boundary_face(const MeshDev &m, const double *__restrict__ u, S *__restrict__ slots,
                                              int64_t j, int e, T sg, int bid, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int lev = m.level[e];
    const T w = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t) * (T(1) / T(6));
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
        const T ps = face_ps<T>(g), pt = face_pt<T>(g);
        T U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + T(0.5) * sg * c[v][1 + D] + ps * c[v][1 + s] + pt * c[v][1 + t];
        Prim<T, NC> pin, pout;
        cons_to_prim<T, NC>(U, pin);
        bnd_cond<T, NC>(bid, pin, pout, n);
        T q[V];
        num_flux<FLUX, T, NC, D>(pin, pout, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
    const int64_t slot = 2 * m.n_face + j;
    const int64_t NS = m.n_slot;
#pragma unroll
    for (int v = 0; v < V; v++) {
        T a0 = w * S0[v];
        slots[(int64_t) (v * kNB + 0) * NS + slot] = S(a0);
        slots[(int64_t) (v * kNB + 1 + D) * NS + slot] = S(T(0.5) * sg * a0);
        slots[(int64_t) (v * kNB + 1 + s) * NS + slot] = S(w * Ss[v]);
        slots[(int64_t) (v * kNB + 1 + t) * NS + slot] = S(w * St[v]);
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
        using TB = typename std::conditional<is_dw<T>, double, T>::type;
        const TB sg = (f & 1) ? TB(1) : TB(-1);
        switch (f >> 1) {
        case 0: boundary_face<TB, NC, FLUX, 0, T>(m, u, slots, j, e, sg, bid, err); break;
        case 1: boundary_face<TB, NC, FLUX, 1, T>(m, u, slots, j, e, sg, bid, err); break;
        default: boundary_face<TB, NC, FLUX, 2, T>(m, u, slots, j, e, sg, bid, err); break;
        }
    }
}

// ---------------------------------------------------------------------------
// CFL step of the state a stage kernel has just written (the reference's
// get_dt formula, src/models/ns/charm_model.c:21-36: CFL * volume / (|u| + c)
// from the fields at the cell centre, i.e. coefficient 0), folded into
// *dt_next by a warp reduction and one 64-bit atomicMin per warp (positive
// doubles order as their bit patterns).  Called by the threads still active
// in the warp (elements past the end have already left).
// ---------------------------------------------------------------------------
template <int NC>
__device__ __forceinline__ double cell_cfl_dt(const double U[4 + NC], double cfl, double vol)
{
    Prim<double, NC> p;
    cons_to_prim<double, NC>(U, p);
    const double d = cfl * vol / (sqrt(p.u * p.u + p.v * p.v + p.w * p.w) + p.cz);
    return (d > 0.0) ? d : 1.0e300;
}

__device__ __forceinline__ void warp_min_to(double d, unsigned long long *dst)
{
    const unsigned mask = __activemask();
    const unsigned long long b = (unsigned long long) __double_as_longlong(d);
    const unsigned hi = (unsigned) (b >> 32), lo = (unsigned) b;
    const unsigned mhi = __reduce_min_sync(mask, hi);
    const unsigned mlo = __reduce_min_sync(mask, (hi == mhi) ? lo : 0xffffffffu);
    if ((int) (threadIdx.x & 31) == __ffs(mask) - 1) atomicMin(dst, ((unsigned long long) mhi << 32) | mlo);
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
            int mode, unsigned *err, const double *__restrict__ radd, unsigned long long *dt_next, double cfl)
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
        const T px = (g & 1) ? T(kGaussPhi) : T(-kGaussPhi);
        const T py = (g & 2) ? T(kGaussPhi) : T(-kGaussPhi);
        const T pz = (g & 4) ? T(kGaussPhi) : T(-kGaussPhi);
        T U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
        Prim<T, NC> p;
        cons_to_prim<T, NC>(U, p);
        if (!(p.r > T(0)) || !(p.p > T(0))) set_error(err, isfinite((double) p.r) && isfinite((double) p.p) ? kErrNegative : kErrNonFinite);
        // Euler fluxes (src/models/ns/charm_model_ns_conv.c:45-65)
        const auto hp = U[3] + p.p;   // r e_tot + p: the energy fluxes are u hp, v hp, w hp
        F[0] += U[0] * p.u + p.p; F[1] += U[0] * p.v; F[2] += U[0] * p.w; F[3] += p.u * hp;
        G[0] += U[1] * p.u; G[1] += U[1] * p.v + p.p; G[2] += U[1] * p.w; G[3] += p.v * hp;
        H[0] += U[2] * p.u; H[1] += U[2] * p.v; H[2] += U[2] * p.w + p.p; H[3] += p.w * hp;
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
                for (int k = 0; k < kNB; k++) gr[a][k] += p.r * cfgv<T>(c_cfg.grav[a], c_cfg.grav_f[a]) * phi[k];
        }
    }
    const double w8 = vol * 0.125;
    double R[V][kNB];
#pragma unroll
    for (int v = 0; v < V; v++) {
        R[v][0] = 0.0;
        // (vol / 8) / h_a as the product of the other two edges / 8
        // (within 1.5 ulp of the quotient, without a division)
        R[v][1] = -(double) F[v] * (hy * hz * 0.125);
        R[v][2] = -(double) G[v] * (hx * hz * 0.125);
        R[v][3] = -(double) H[v] * (hx * hy * 0.125);
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
    if (radd) {   // viscous volume terms of the momentum and energy rows
#pragma unroll
        for (int v = 0; v < 4; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) R[v][k] += __ldg(radd + (int64_t) (v * kNB + k) * E + e);
    }

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
    const double minv0 = rcp_nr(vol), minv1 = 12.0 * minv0;   // within 1.5 ulp of 1/vol, 12/vol
    const bool comb = (a_old != 0.0);
    double cen[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            const double cu = __ldg(u + idx);
            double x = cu - step * (R[v][k] * (k == 0 ? minv0 : minv1));
            if (comb) x = a_new * x + a_old * u0[idx];
            out[idx] = x;
            if (k == 0) cen[v] = x;
        }
    }
    // last stage of a step in CFL mode: the next step's dt from this state
    if (dt_next) warp_min_to(cell_cfl_dt<NC>(cen, cfl, vol), dt_next);
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
// Barth-Jespersen scaling from the 8 vertex differences of each variable
// (bj_side_psi).
template <int V>
__device__ __forceinline__ void bj_psi8(const double c[V][kNB], const double umin[V], const double umax[V],
                                        double psi[V])
{
#pragma unroll
    for (int v = 0; v < V; v++) {
        double dmax = 0.0, dmin = 0.0;
#pragma unroll
        for (int vx = 0; vx < 8; vx++) {
            const double sx = (vx & 1) ? 0.5 : -0.5, sy = (vx & 2) ? 0.5 : -0.5, sz = (vx & 4) ? 0.5 : -0.5;
            const double f = c[v][0] + sx * c[v][1] + sy * c[v][2] + sz * c[v][3];
            const double df = f - c[v][0];
            dmax = fmax(dmax, df);
            dmin = fmin(dmin, df);
        }
        psi[v] = bj_side_psi(dmax, dmin, umin[v] - c[v][0], umax[v] - c[v][0]);
    }
}

template <int NC>
__global__ void __launch_bounds__(128)
limit_kernel(MeshDev m, const double *__restrict__ ua, const double *u0, double *out,
             double a_new, double a_old, double *__restrict__ psi_out, unsigned long long *dt_next, double cfl)
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
        const int kind = m.lim_kind[(int64_t) f * E + e] & 3;
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
    bj_psi8<V>(c, umin, umax, psi);
    if (psi_out) {   // the scaling, kept for the adjoint (frozen active set)
#pragma unroll
        for (int v = 0; v < V; v++) psi_out[(int64_t) v * E + e] = psi[v];
    }
    const bool comb = (a_old != 0.0);
    double cen[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            double x = (k == 0) ? c[v][0] : c[v][k] * psi[v];
            if (comb) x = a_new * x + a_old * u0[idx];
            out[idx] = x;
            if (k == 0) cen[v] = x;
        }
    }
    // last stage of a step in CFL mode: the next step's dt from this state
    if (dt_next) {
        const int lev = m.level[e];
        const double vol = level_h(m, lev, 0) * level_h(m, lev, 1) * level_h(m, lev, 2);
        warp_min_to(cell_cfl_dt<NC>(cen, cfl, vol), dt_next);
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


// ===========================================================================
// Mixed form: element-owned fused stage on an FP32 hi/lo state
// ===========================================================================
//
// The stage state of the mixed form is kept as two FP32 planes, u = hi + lo
// (same 8 bytes per coefficient as FP64, ~48-bit significand), so that the
// stage kernel issues no FP64 instruction: on GB300 the FP64 pipe is ~1/64
// of FP32, and conversions from a double state kept it 77-82 % busy.
// One thread per element computes the volume integral, the fluxes of all its
// faces (each face is computed by both of its owners, from the same operands
// at one code location, so the two contributions are exact negatives), the
// M^-1 scaling and the update, with error-free FP32 transformations for
// u - dt*M^-1*R and the SSP combinations.  No face buffer goes through HBM.

struct FF { float h, l; };

__device__ __forceinline__ FF ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ FF ff_renorm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

// x - (dh + dl) * r
__device__ __forceinline__ FF ff_sub_scaled(FF x, float r, float dh, float dl)
{
    const float ph = __fmul_rn(dh, r);
    float pl = __fmaf_rn(dh, r, -ph);
    pl = __fmaf_rn(dl, r, pl);
    const FF s = ff_two_sum(x.h, -ph);
    const float e = __fadd_rn(s.l, __fsub_rn(x.l, pl));
    return ff_renorm(s.h, e);
}

// (ah + al) * y + (bh + bl) * w
__device__ __forceinline__ FF ff_comb(FF y, FF w, float ah, float al, float bh, float bl)
{
    const float p = __fmul_rn(ah, y.h);
    float pe = __fmaf_rn(ah, y.h, -p);
    pe = __fmaf_rn(ah, y.l, pe);
    pe = __fmaf_rn(al, y.h, pe);
    const float q = __fmul_rn(bh, w.h);
    float qe = __fmaf_rn(bh, w.h, -q);
    qe = __fmaf_rn(bh, w.l, qe);
    qe = __fmaf_rn(bl, w.h, qe);
    const FF s = ff_two_sum(p, q);
    return ff_renorm(s.h, __fadd_rn(s.l, __fadd_rn(pe, qe)));
}

static __global__ void __launch_bounds__(256) ff_from_double_kernel(const double *__restrict__ u, float *__restrict__ hi,
                                                             float *__restrict__ lo, int64_t n)
{
    const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = u[i];
    const float h = __double2float_rn(x);
    hi[i] = h;
    lo[i] = __double2float_rn(x - (double) h);
}

static __global__ void __launch_bounds__(256) ff_to_double_kernel(const float *__restrict__ hi, const float *__restrict__ lo,
                                                           double *__restrict__ u, int64_t n)
{
    const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u[i] = (double) hi[i] + (double) lo[i];
}

template <int V>
__device__ __forceinline__ void load_coef_f(const float *__restrict__ u, int64_t E, int64_t e, float c[V][kNB])
{
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) c[v][k] = __ldg(u + (int64_t) (v * kNB + k) * E + e);
}

// Flux of one (sub-)face along axis D from the lower and upper leaves'
// coefficients, projected on the owner's basis and added to R.
//   kind: 0 conforming, 1 lower leaf is the small one, 2 upper leaf is small
//   sub : position of the small face in the big face
//   w   : gw*gj of one point of the (small) face
// R[v][0] += x with the rounding error kept in R0l[v] (two-sum), so that the
// mean coefficient's residual is the element's face contributions summed
// without loss: the two owners of a face add exact negatives, and the total
// mass change of a stage cancels to the float-float level.
__device__ __forceinline__ void acc0(float &hi, float &lo, float x)
{
    const FF s = ff_two_sum(hi, x);
    hi = s.h;
    lo = __fadd_rn(lo, s.l);
}

template <int NC, int FLUX, int D>
__device__ __forceinline__ void owned_face(const float cl[4 + NC][kNB], const float cu[4 + NC][kNB], int kind, int sub,
                                           bool own_lower, float w, float R[4 + NC][kNB], float R0l[4 + NC],
                                           unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const float os = (sub & 1) ? 0.25f : -0.25f, ot = (sub & 2) ? 0.25f : -0.25f;
    float n[3] = {0.f, 0.f, 0.f};
    n[D] = 1.f;
    float S0[V], Ss[V], St[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = 0.f;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const float ps = c_face_psf[g], pt = c_face_ptf[g];
        float psl = ps, ptl = pt, psu = ps, ptu = pt;
        if (kind == 2) { psl = 0.5f * ps + os; ptl = 0.5f * pt + ot; }
        if (kind == 1) { psu = 0.5f * ps + os; ptu = 0.5f * pt + ot; }
        float Ul[V], Uu[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            Ul[v] = cl[v][0] + 0.5f * cl[v][1 + D] + psl * cl[v][1 + s] + ptl * cl[v][1 + t];
            Uu[v] = cu[v][0] - 0.5f * cu[v][1 + D] + psu * cu[v][1 + s] + ptu * cu[v][1 + t];
        }
        Prim<float, NC> pl, pu;
        cons_to_prim<float, NC>(Ul, pl);
        cons_to_prim<float, NC>(Uu, pu);
        float q[V];
        num_flux<FLUX, float, NC, D>(pl, pu, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
    // projection on the owner's basis (lower side gets +, upper side -)
    const bool own_big = (own_lower && kind == 2) || (!own_lower && kind == 1);
#pragma unroll
    for (int v = 0; v < V; v++) {
        const float a0 = w * S0[v];
        float as = w * Ss[v], at = w * St[v];
        if (own_big) { as = 0.5f * as + os * a0; at = 0.5f * at + ot * a0; }
        const float sg = own_lower ? 1.f : -1.f;
        acc0(R[v][0], R0l[v], sg * a0);
        R[v][1 + D] += 0.5f * a0;
        R[v][1 + s] += sg * as;
        R[v][1 + t] += sg * at;
    }
}

template <int NC, int FLUX, int D>
__device__ __forceinline__ void owned_boundary(const MeshDev &m, const float c[4 + NC][kNB], int j, float w,
                                               float R[4 + NC][kNB], float R0l[4 + NC], unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int f = m.bface_face[j], bid = m.bface_bnd[j];
    const float sg = (f & 1) ? 1.f : -1.f;
    float n[3] = {0.f, 0.f, 0.f};
    n[D] = sg;
    float S0[V], Ss[V], St[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = 0.f;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const float ps = c_face_psf[g], pt = c_face_ptf[g];
        float U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + 0.5f * sg * c[v][1 + D] + ps * c[v][1 + s] + pt * c[v][1 + t];
        Prim<float, NC> pin, pout;
        cons_to_prim<float, NC>(U, pin);
        bnd_cond<float, NC>(bid, pin, pout, n);
        float q[V];
        num_flux<FLUX, float, NC, D>(pin, pout, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
#pragma unroll
    for (int v = 0; v < V; v++) {
        const float a0 = w * S0[v];
        acc0(R[v][0], R0l[v], a0);
        R[v][1 + D] += 0.5f * sg * a0;
        R[v][1 + s] += w * Ss[v];
        R[v][1 + t] += w * St[v];
    }
}

// The two faces of element e along axis D (lower face 2D, upper face 2D+1).
template <int NC, int FLUX, int D>
__device__ __forceinline__ void owned_axis(const MeshDev &m, const float *__restrict__ uh, int64_t e,
                                           const float c[4 + NC][kNB], int lev, float R[4 + NC][kNB],
                                           float R0l[4 + NC], unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t E = m.n_elem;
#pragma unroll 1
    for (int side = 0; side < 2; side++) {
        const int f = 2 * D + side;
        const int code = m.lim_kind[(int64_t) f * E + e];
        const int idx = m.lim_idx[(int64_t) f * E + e];
        const int kind = code & 3;
        if (kind == 1) {   // boundary
            const float w = level_ht<float>(m, lev, s) * level_ht<float>(m, lev, t) * (1.f / 6.f);
            owned_boundary<NC, FLUX, D>(m, c, idx, w, R, R0l, err);
            continue;
        }
        const bool own_lower = (side == 1);
        const int nsub = (kind == 2) ? 4 : 1;
#pragma unroll 1
        for (int k = 0; k < nsub; k++) {
            int nb, rec_kind, sub, small_lev;
            if (kind == 2) {   // we are the big leaf: record idx+k holds small leaf k
                const int64_t fi = idx + k;
                const unsigned info = m.face_info[fi];
                rec_kind = (info >> 2) & 3;
                nb = (rec_kind == 1) ? m.face_elem[fi] : m.face_elem[m.n_face + fi];
                sub = k;
                small_lev = m.level[nb];
            } else {
                nb = idx;
                sub = (code >> 4) & 3;
                rec_kind = (kind == 0) ? 0 : (own_lower ? 1 : 2);
                small_lev = lev;
            }
            float cn[V][kNB];
            load_coef_f<V>(uh, E, nb, cn);
            float cl[V][kNB], cu[V][kNB];
#pragma unroll
            for (int v = 0; v < V; v++)
#pragma unroll
                for (int b = 0; b < kNB; b++) {
                    cl[v][b] = own_lower ? c[v][b] : cn[v][b];
                    cu[v][b] = own_lower ? cn[v][b] : c[v][b];
                }
            const float w = level_ht<float>(m, small_lev, s) * level_ht<float>(m, small_lev, t) * (1.f / 6.f);
            owned_face<NC, FLUX, D>(cl, cu, rec_kind, sub, own_lower, w, R, R0l, err);
        }
    }
}

// One stage of the mixed form:
//   out = (ah+al) * (u - dt*M^-1*R(u)) + (bh+bl) * u0     (comb != 0)
//   out = u - dt*M^-1*R(u)                                 (comb == 0)
// all planes FP32 hi/lo; dt = dth + dtl (or *dt_dev when given).
template <int NC, int FLUX>
__global__ void __launch_bounds__(128)
ff_stage_kernel(MeshDev m, const float *__restrict__ uh, const float *__restrict__ ul, const float *u0h,
                const float *u0l, float *oh, float *ol, float dth, float dtl, const double *__restrict__ dt_dev,
                float ah, float al, float bh, float bl, int comb, unsigned *err)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const float hx = level_ht<float>(m, lev, 0), hy = level_ht<float>(m, lev, 1), hz = level_ht<float>(m, lev, 2);
    const float vol = hx * hy * hz;

    float c[V][kNB];
    load_coef_f<V>(uh, E, e, c);
    float R[V][kNB], R0l[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
        R0l[v] = 0.f;
#pragma unroll
        for (int k = 0; k < kNB; k++) R[v][k] = 0.f;
    }

    // volume integral (src/models/ns/charm_model_ns_conv.c:23-89)
    {
        float F[V], G[V], H[V];
#pragma unroll
        for (int v = 0; v < V; v++) F[v] = G[v] = H[v] = 0.f;
        const bool grav = c_cfg.has_grav != 0;
        float gr[3][kNB];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int k = 0; k < kNB; k++) gr[a][k] = 0.f;
#pragma unroll 1
        for (int g = 0; g < 8; g++) {
            const float px = (g & 1) ? (float) kGaussPhi : -(float) kGaussPhi;
            const float py = (g & 2) ? (float) kGaussPhi : -(float) kGaussPhi;
            const float pz = (g & 4) ? (float) kGaussPhi : -(float) kGaussPhi;
            float U[V];
#pragma unroll
            for (int v = 0; v < V; v++) U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
            Prim<float, NC> p;
            cons_to_prim<float, NC>(U, p);
            if (!(p.r > 0.f) || !(p.p > 0.f)) set_error(err, (isfinite(p.r) && isfinite(p.p)) ? kErrNegative : kErrNonFinite);
            const auto hp = U[3] + p.p;   // r e_tot + p: the energy fluxes are u hp, v hp, w hp
            F[0] += U[0] * p.u + p.p; F[1] += U[0] * p.v; F[2] += U[0] * p.w; F[3] += p.u * hp;
            G[0] += U[1] * p.u; G[1] += U[1] * p.v + p.p; G[2] += U[1] * p.w; G[3] += p.v * hp;
            H[0] += U[2] * p.u; H[1] += U[2] * p.v; H[2] += U[2] * p.w + p.p; H[3] += p.w * hp;
#pragma unroll
            for (int i = 0; i < NC; i++) {
                F[4 + i] += U[0] * p.c[i];
                G[4 + i] += U[1] * p.c[i];
                H[4 + i] += U[2] * p.c[i];
            }
            if (grav) {
                const float phi[4] = {1.f, px, py, pz};
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int k = 0; k < kNB; k++) gr[a][k] += p.r * c_cfg.grav_f[a] * phi[k];
            }
        }
        const float w8 = vol * 0.125f;
#pragma unroll
        for (int v = 0; v < V; v++) {
            R[v][1] -= F[v] * (w8 / hx);
            R[v][2] -= G[v] * (w8 / hy);
            R[v][3] -= H[v] * (w8 / hz);
        }
        if (grav) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                acc0(R[a][0], R0l[a], -gr[a][0] * w8);
#pragma unroll
                for (int k = 1; k < kNB; k++) R[a][k] -= gr[a][k] * w8;
            }
        }
    }
    // faces
    owned_axis<NC, FLUX, 0>(m, uh, e, c, lev, R, R0l, err);
    owned_axis<NC, FLUX, 1>(m, uh, e, c, lev, R, R0l, err);
    owned_axis<NC, FLUX, 2>(m, uh, e, c, lev, R, R0l, err);

    // update with diagonal M^-1 = (1/vol, 12/vol, 12/vol, 12/vol)
    if (dt_dev) {
        const double d = *dt_dev;
        dth = __double2float_rn(d);
        dtl = __double2float_rn(d - (double) dth);
    }
    const float minv0 = 1.f / vol, minv1 = 12.f / vol;
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            FF x = {uh[idx], ul[idx]};
            FF y;
            if (k == 0) {   // mean coefficient: (R + R0l) * minv0 kept as float-float
                const float rh = __fmul_rn(R[v][0], minv0);
                const float rl = __fmaf_rn(R0l[v], minv0, __fmaf_rn(R[v][0], minv0, -rh));
                y = ff_sub_scaled(x, rh, dth, dtl);
                y = ff_sub_scaled(y, rl, dth, dtl);
            } else {
                y = ff_sub_scaled(x, R[v][k] * minv1, dth, dtl);
            }
            if (comb) {
                const FF w0 = {u0h[idx], u0l[idx]};
                y = ff_comb(y, w0, ah, al, bh, bl);
            }
            oh[idx] = y.h;
            ol[idx] = y.l;
        }
    }
}

// Barth-Jespersen limiter of the mixed form on hi/lo planes (the same rules
// as limit_kernel; bounds and psi in FP32, coefficients scaled in hi/lo),
// fused with the SSP combination.
template <int NC>
__global__ void __launch_bounds__(128)
ff_limit_kernel(MeshDev m, const float *__restrict__ ah_, const float *__restrict__ al_, const float *u0h,
                const float *u0l, float *oh, float *ol, float ah, float al, float bh, float bl, int comb)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    float c[V][kNB];
    load_coef_f<V>(ah_, E, e, c);
    float umin[V], umax[V];
#pragma unroll
    for (int v = 0; v < V; v++) umin[v] = umax[v] = c[v][0];
#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        const int kind = m.lim_kind[(int64_t) f * E + e] & 3;
        const int idx = m.lim_idx[(int64_t) f * E + e];
        float nbv[V];
        if (kind == 0 || kind == 3) {
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = __ldg(ah_ + (int64_t) (v * kNB) * E + idx);
        } else if (kind == 2) {
            float svol = 0.f;
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = 0.f;
            for (int k = 0; k < 4; k++) {
                const int64_t fi = idx + k;
                const unsigned info = m.face_info[fi];
                const int small = (((info >> 2) & 3) == 1) ? m.face_elem[fi] : m.face_elem[m.n_face + fi];
                const int ls = m.level[small];
                const float vs = level_ht<float>(m, ls, 0) * level_ht<float>(m, ls, 1) * level_ht<float>(m, ls, 2);
                svol += vs;
#pragma unroll
                for (int v = 0; v < V; v++) nbv[v] += __ldg(ah_ + (int64_t) (v * kNB) * E + small) * vs;
            }
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] /= svol;
        } else {
            const int fb = m.bface_face[idx], bid = m.bface_bnd[idx];
            float n[3] = {0.f, 0.f, 0.f};
            n[fb >> 1] = (fb & 1) ? 1.f : -1.f;
            float U[V];
#pragma unroll
            for (int v = 0; v < V; v++) U[v] = c[v][0];
            Prim<float, NC> pin, pout;
            cons_to_prim<float, NC>(U, pin);
            bnd_cond<float, NC>(bid, pin, pout, n);
            prim_to_cons<float, NC>(pout, nbv);
        }
#pragma unroll
        for (int v = 0; v < V; v++) {
            umin[v] = fminf(umin[v], nbv[v]);
            umax[v] = fmaxf(umax[v], nbv[v]);
        }
    }
    // psi from the largest and the most negative vertex difference per
    // variable: two correctly rounded quotients, monotone in the
    // difference, give the per-vertex minimum (as bj_side_psi in FP64)
    float psi[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
        float dmax = 0.f, dmin = 0.f;
#pragma unroll
        for (int vx = 0; vx < 8; vx++) {
            const float sx = (vx & 1) ? 0.5f : -0.5f, sy = (vx & 2) ? 0.5f : -0.5f, sz = (vx & 4) ? 0.5f : -0.5f;
            const float df = sx * c[v][1] + sy * c[v][2] + sz * c[v][3];
            dmax = fmaxf(dmax, df);
            dmin = fminf(dmin, df);
        }
        float p = 1.f;
        if (dmax > (float) kEps) p = fminf(p, fminf(1.f, (umax[v] - c[v][0]) / dmax));
        if (dmin < -(float) kEps) p = fminf(p, fminf(1.f, (umin[v] - c[v][0]) / dmin));
        psi[v] = p;
    }
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            FF y = {ah_[idx], al_[idx]};
            if (k > 0) {   // psi * y, error-free product on the hi part
                const float p = __fmul_rn(psi[v], y.h);
                const float pe = __fmaf_rn(psi[v], y.l, __fmaf_rn(psi[v], y.h, -p));
                y = ff_renorm(p, pe);
            }
            if (comb) {
                const FF w0 = {u0h[idx], u0l[idx]};
                y = ff_comb(y, w0, ah, al, bh, bl);
            }
            oh[idx] = y.h;
            ol[idx] = y.l;
        }
    }
}


// ===========================================================================
// AMR indicator: density-gradient estimate of charm_adapt
// (src/charm_amr.c:350-573): grad = (1/vol) * sum over the element's faces
// of 0.5*(rho_L + rho_R) * n * gw*gj at the 6 face points, n pointing out of
// side 0 (side 0 adds, side 1 subtracts); boundary faces use the boundary
// condition's ghost density.  FP64, one thread per element.
// ===========================================================================

template <int NC>
__device__ __forceinline__ double point_density(const double c[4 + NC][kNB], double pd, int D, double ps, double pt)
{
    const int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < NC; i++)
        r += c[4 + i][0] + pd * c[4 + i][1 + D] + ps * c[4 + i][1 + s] + pt * c[4 + i][1 + t];
    return r < kEps ? kEps : r;   // prim.r after eos flag 4 (src/charm_eos.c:87)
}

template <int NC>
__global__ void __launch_bounds__(128) amr_grad_kernel(MeshDev m, const double *__restrict__ u, double *__restrict__ grad)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    double c[V][kNB];
    load_coef<double, V>(u, E, e, c);
    double g[3] = {0.0, 0.0, 0.0};
#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        const int D = f >> 1;
        const int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
        const int code = m.lim_kind[(int64_t) f * E + e];
        const int kind = code & 3, idx = m.lim_idx[(int64_t) f * E + e];
        if (kind == 1) {   // boundary
            const int fb = m.bface_face[idx], bid = m.bface_bnd[idx];
            const double sg = (fb & 1) ? 1.0 : -1.0;
            double n[3] = {0.0, 0.0, 0.0};
            n[D] = sg;
            const double w = level_h(m, lev, s) * level_h(m, lev, t) * (1.0 / 6.0);
            for (int q = 0; q < 6; q++) {
                const double ps = c_face_s[q] - 0.5, pt = c_face_t[q] - 0.5;
                double U[V];
#pragma unroll
                for (int v = 0; v < V; v++) {
                    double x = c[v][0] + 0.5 * sg * c[v][1 + D];
                    x += ps * c[v][1 + s];
                    x += pt * c[v][1 + t];
                    U[v] = x;
                }
                Prim<double, NC> pin, pout;
                cons_to_prim<double, NC>(U, pin);
                bnd_cond<double, NC>(bid, pin, pout, n);
                g[D] += 0.5 * (pin.r + pout.r) * w * sg;
            }
            continue;
        }
        const bool own_lower = (f & 1);
        const int nsub = (kind == 2) ? 4 : 1;
        for (int k = 0; k < nsub; k++) {
            int nb, rec_kind, sub, plev;
            if (kind == 2) {
                const unsigned info = m.face_info[idx + k];
                rec_kind = (info >> 2) & 3;
                nb = (rec_kind == 1) ? m.face_elem[idx + k] : m.face_elem[m.n_face + idx + k];
                sub = k;
                plev = m.level[nb];
            } else {
                nb = idx;
                sub = (code >> 4) & 3;
                rec_kind = (kind == 0) ? 0 : (own_lower ? 1 : 2);
                plev = lev;
            }
            double cn[V][kNB];
            load_coef<double, V>(u, E, nb, cn);
            const double os = (sub & 1) ? 0.25 : -0.25, ot = (sub & 2) ? 0.25 : -0.25;
            const double w = level_h(m, plev, s) * level_h(m, plev, t) * (1.0 / 6.0);
            double acc = 0.0;
            for (int q = 0; q < 6; q++) {
                const double ps = c_face_s[q] - 0.5, pt = c_face_t[q] - 0.5;
                double psl = ps, ptl = pt, psu = ps, ptu = pt;
                if (rec_kind == 2) { psl = 0.5 * ps + os; ptl = 0.5 * pt + ot; }
                if (rec_kind == 1) { psu = 0.5 * ps + os; ptu = 0.5 * pt + ot; }
                const double rl = own_lower ? point_density<NC>(c, 0.5, D, psl, ptl) : point_density<NC>(cn, 0.5, D, psl, ptl);
                const double ru = own_lower ? point_density<NC>(cn, -0.5, D, psu, ptu) : point_density<NC>(c, -0.5, D, psu, ptu);
                acc += 0.5 * (rl + ru) * w;
            }
            g[D] += own_lower ? acc : -acc;
        }
    }
    const double vol = level_h(m, lev, 0) * level_h(m, lev, 1) * level_h(m, lev, 2);
#pragma unroll
    for (int k = 0; k < 3; k++) grad[(int64_t) k * E + e] = g[k] / vol;
}


// ===========================================================================
// Mixed form, block-local: one CTA per tile of kTile Morton-consecutive
// elements.  Everything a tile's stage reads is staged in shared memory
// before any face is evaluated:
//   - the tile's hi coefficient planes (kTile consecutive floats per plane)
//     by bulk asynchronous copies (cp.async.bulk, completion on an
//     mbarrier) issued by one thread;
//   - the halo: the hi coefficients of every element outside the tile that
//     shares a face with it (a per-tile list built at upload), loaded by all
//     threads at once;
// so the face loop reads no global memory but one 16-byte record per face.
// Every face that touches the tile is evaluated once by the CTA (faces on
// the tile boundary once by each of the two tiles, from identical operands
// at one code location), its projections (a0, as, at per variable) kept in
// shared memory; then each thread gathers its element's faces, adds the
// volume integral and updates u in float-float.
// ===========================================================================
constexpr int kTile = 128;

struct TileDev {
    const int32_t *fptr;    // [n_tiles + 1] into rec
    const int4    *rec;     // one record per (tile, face), see tile_face_rec
    const int32_t *hptr;    // [n_tiles + 1] into halo
    const int32_t *halo;    // global element ids of each tile's halo
    const int32_t *slot;    // [6][E]: (position of the element face in its tile's records << 2) | kind
                            // (kind: 0 conforming, 1 boundary, 2 big side of a mortar, 3 small side)
    int ncol;               // shared-memory columns: kTile + the largest halo
    int bulk;               // 1: the tile planes are 16-byte aligned runs (E % 4 == 0): bulk copies
};

// Face record (int4), built by the host at upload:
//   x: shared-memory column of side 0 (interior) or of the element (boundary)
//   y: column of side 1 (interior), -1 (boundary)
//   z: interior: the face_info byte; boundary: face id | bnd id << 8 | 1 << 30
//   w: level of the leaf that owns the quadrature points
constexpr int kRecBoundary = 1 << 30;

template <int V>
__device__ __forceinline__ void col_coef(const float *s_u, int ncol, int col, float c[V][kNB])
{
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) c[v][k] = s_u[(v * kNB + k) * ncol + col];
}

// 6-point sums of one interior (sub-)face along D: S0 = sum q, Ss = sum q*ps,
// St = sum q*pt with the lower/upper leaves' coefficients.
template <int NC, int FLUX, int D>
__device__ __forceinline__ void face_sums(const float cl[4 + NC][kNB], const float cu[4 + NC][kNB], int kind, int sub,
                                          float S0[4 + NC], float Ss[4 + NC], float St[4 + NC], unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const float os = (sub & 1) ? 0.25f : -0.25f, ot = (sub & 2) ? 0.25f : -0.25f;
    float n[3] = {0.f, 0.f, 0.f};
    n[D] = 1.f;
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = 0.f;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const float ps = c_face_psf[g], pt = c_face_ptf[g];
        float psl = ps, ptl = pt, psu = ps, ptu = pt;
        if (kind == 2) { psl = 0.5f * ps + os; ptl = 0.5f * pt + ot; }
        if (kind == 1) { psu = 0.5f * ps + os; ptu = 0.5f * pt + ot; }
        float Ul[V], Uu[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            Ul[v] = cl[v][0] + 0.5f * cl[v][1 + D] + psl * cl[v][1 + s] + ptl * cl[v][1 + t];
            Uu[v] = cu[v][0] - 0.5f * cu[v][1 + D] + psu * cu[v][1 + s] + ptu * cu[v][1 + t];
        }
        Prim<float, NC> pl, pu;
        cons_to_prim<float, NC>(Ul, pl);
        cons_to_prim<float, NC>(Uu, pu);
        float q[V];
        num_flux<FLUX, float, NC, D>(pl, pu, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
}

// Momentum components (x, y, z) of a face along axis D into the face frame
// (normal, t1, t2) of the flux (frame_in of dg_device.cuh: D = 1 gives
// (y, -x, z), D = 2 gives (z, -y, x)) and back (frame_out): signed
// permutations, exact.
__device__ __forceinline__ void tile_rot_in(int D, float &a, float &b, float &c)
{
    const float x = a, y = b, z = c;
    a = (D == 0) ? x : (D == 1) ? y : z;
    b = (D == 0) ? y : (D == 1) ? -x : -y;
    c = (D == 2) ? x : z;
}

__device__ __forceinline__ void tile_rot_out(int D, float &a, float &b, float &c)
{
    const float fu = a, fv = b, fw = c;
    a = (D == 0) ? fu : (D == 1) ? -fv : fw;
    b = (D == 0) ? fv : (D == 1) ? fu : -fv;
    c = (D == 2) ? fu : fw;
}

// Interior (sub-)face of a tile, its axis D read at run time: the
// coefficients of both leaves reordered into the face frame (mean, slope
// along the normal, along s, along t) and their momentum components
// rotated by tile_rot_in, then the 6-point sums of a face along x, whose
// momentum components tile_rot_out turns back.  One inlined face path
// serves all three axes, which keeps the face loop of tile_stage_kernel
// within the instruction cache.
template <int NC, int FLUX>
__device__ __forceinline__ void tile_interior(const MeshDev &m, const float *s_u, int ncol, int4 r, float *out,
                                              unsigned *err)
{
    constexpr int V = 4 + NC;
    const unsigned info = (unsigned) r.z;
    const int D = info & 3, s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int kind = (info >> 2) & 3, sub = (info >> 4) & 3;
    float cl[V][kNB], cu[V][kNB];
#pragma unroll
    for (int v = 0; v < V; v++) {
        const int b = v * kNB;
        cl[v][0] = s_u[b * ncol + r.x];
        cl[v][1] = s_u[(b + 1 + D) * ncol + r.x];
        cl[v][2] = s_u[(b + 1 + s) * ncol + r.x];
        cl[v][3] = s_u[(b + 1 + t) * ncol + r.x];
        cu[v][0] = s_u[b * ncol + r.y];
        cu[v][1] = s_u[(b + 1 + D) * ncol + r.y];
        cu[v][2] = s_u[(b + 1 + s) * ncol + r.y];
        cu[v][3] = s_u[(b + 1 + t) * ncol + r.y];
    }
#pragma unroll
    for (int k = 0; k < kNB; k++) {
        tile_rot_in(D, cl[0][k], cl[1][k], cl[2][k]);
        tile_rot_in(D, cu[0][k], cu[1][k], cu[2][k]);
    }
    float S0[V], Ss[V], St[V];
    face_sums<NC, FLUX, 0>(cl, cu, kind, sub, S0, Ss, St, err);
    tile_rot_out(D, S0[0], S0[1], S0[2]);
    tile_rot_out(D, Ss[0], Ss[1], Ss[2]);
    tile_rot_out(D, St[0], St[1], St[2]);
    // the tangential edges (s is axis 0 or 1, t axis 1 or 2), chosen by
    // value: no run-time index into the kernel's parameters
    const float Ls = (s == 0) ? m.tree_len_f[0] : m.tree_len_f[1];
    const float Lt = (t == 1) ? m.tree_len_f[1] : m.tree_len_f[2];
    const float w = ldexpf(Ls, -r.w) * ldexpf(Lt, -r.w) * (1.f / 6.f);
#pragma unroll
    for (int v = 0; v < V; v++) {
        out[v] = w * S0[v];
        out[V + v] = w * Ss[v];
        out[2 * V + v] = w * St[v];
    }
}

template <int NC, int FLUX, int D>
__device__ __forceinline__ void tile_boundary(const MeshDev &m, const float *s_u, int ncol, int4 r, float *out,
                                              unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int f = r.z & 7, bid = (r.z >> 8) & 0xff;
    const float sg = (f & 1) ? 1.f : -1.f;
    float c[V][kNB];
    col_coef<V>(s_u, ncol, r.x, c);
    float n[3] = {0.f, 0.f, 0.f};
    n[D] = sg;
    float S0[V], Ss[V], St[V];
#pragma unroll
    for (int v = 0; v < V; v++) S0[v] = Ss[v] = St[v] = 0.f;
#pragma unroll 1
    for (int g = 0; g < 6; g++) {
        const float ps = c_face_psf[g], pt = c_face_ptf[g];
        float U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + 0.5f * sg * c[v][1 + D] + ps * c[v][1 + s] + pt * c[v][1 + t];
        Prim<float, NC> pin, pout;
        cons_to_prim<float, NC>(U, pin);
        bnd_cond<float, NC>(bid, pin, pout, n);
        float q[V];
        num_flux<FLUX, float, NC, D>(pin, pout, n, q, err);
#pragma unroll
        for (int v = 0; v < V; v++) {
            S0[v] += q[v];
            Ss[v] += q[v] * ps;
            St[v] += q[v] * pt;
        }
    }
    const float w = level_ht<float>(m, r.w, s) * level_ht<float>(m, r.w, t) * (1.f / 6.f);
#pragma unroll
    for (int v = 0; v < V; v++) {
        out[v] = w * S0[v];
        out[V + v] = w * Ss[v];
        out[2 * V + v] = w * St[v];
    }
}

// Add the projections of element e's two faces along D to R (code: the
// element face's packed slot, position << 2 | kind).
template <int NC, int D>
__device__ __forceinline__ void tile_gather_axis(const float *s_f, const int code[6], float R[4 + NC][kNB],
                                                 float R0l[4 + NC])
{
    constexpr int V = 4 + NC;
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int kind = code[2 * D + side] & 3;
        const int slot = code[2 * D + side] >> 2;
        if (kind == 1) {   // boundary: outward normal sg * e_D
            const float sg = side ? 1.f : -1.f;
            const float *o = s_f + (int64_t) slot * 3 * V;
#pragma unroll
            for (int v = 0; v < V; v++) {
                acc0(R[v][0], R0l[v], o[v]);
                R[v][1 + D] += 0.5f * sg * o[v];
                R[v][1 + s] += o[V + v];
                R[v][1 + t] += o[2 * V + v];
            }
            continue;
        }
        const float sg = side ? 1.f : -1.f;   // upper face of e: e is the lower leaf (+)
        const int nsub = (kind == 2) ? 4 : 1;
        for (int k = 0; k < nsub; k++) {
            const float *o = s_f + (int64_t) (slot + k) * 3 * V;
            const float os = (k & 1) ? 0.25f : -0.25f, ot = (k & 2) ? 0.25f : -0.25f;
#pragma unroll
            for (int v = 0; v < V; v++) {
                const float a0 = o[v];
                float as = o[V + v], at = o[2 * V + v];
                if (kind == 2) { as = 0.5f * as + os * a0; at = 0.5f * at + ot * a0; }
                acc0(R[v][0], R0l[v], sg * a0);
                R[v][1 + D] += 0.5f * a0;
                R[v][1 + s] += sg * as;
                R[v][1 + t] += sg * at;
            }
        }
    }
}

// ---- bulk asynchronous copies into shared memory (completion on an mbarrier)

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// Wait for phase `parity` of the barrier to complete, at most `tries`
// polls; false when it did not.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned tries)
{
    for (unsigned i = 0; i < tries; i++) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

enum : unsigned { kErrWait = 8u };   // a bounded device wait ran out

template <int NC, int FLUX>
__global__ void __launch_bounds__(kTile, 4)
tile_stage_kernel(MeshDev m, TileDev tl, const float *__restrict__ uh, const float *__restrict__ ul, const float *u0h,
                  const float *u0l, float *oh, float *ol, float dth, float dtl, const double *__restrict__ dt_dev,
                  float ah, float al, float bh, float bl, int comb, unsigned *err)
{
    constexpr int V = 4 + NC;
    extern __shared__ __align__(128) float smem[];
    __shared__ uint64_t bar;
    const int ncol = tl.ncol;
    float *s_u = smem;                         // [V*4][ncol]: tile columns 0..kTile-1, then the halo
    float *s_f = smem + V * kNB * ncol;        // [faces][3V]
    const int64_t E = m.n_elem;
    const int64_t e_begin = (int64_t) blockIdx.x * kTile;
    const int nloc = (int) min((int64_t) kTile, E - e_begin);
    const bool bulk = tl.bulk && (nloc % 4) == 0;
    // ---- stage: tile planes (bulk copies), halo (all threads) ----
    if (bulk) {
        if (threadIdx.x == 0) mbar_init(&bar, 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_expect_tx(&bar, (unsigned) (V * kNB * nloc * sizeof(float)));
            for (int p = 0; p < V * kNB; p++)
                bulk_g2s(s_u + p * ncol, uh + (int64_t) p * E + e_begin, (unsigned) (nloc * sizeof(float)), &bar);
        }
    } else {
        for (int i = threadIdx.x; i < V * kNB * kTile; i += kTile) {
            const int plane = i / kTile, l = i % kTile;
            if (l < nloc) s_u[plane * ncol + l] = __ldg(uh + (int64_t) plane * E + e_begin + l);
        }
    }
    {
        const int h0 = tl.hptr[blockIdx.x], nh = tl.hptr[blockIdx.x + 1] - h0;
        for (int hl = threadIdx.x; hl < nh; hl += kTile) {
            const int64_t g = __ldg(tl.halo + h0 + hl);
            float v[V * kNB];
#pragma unroll
            for (int p = 0; p < V * kNB; p++) v[p] = __ldg(uh + (int64_t) p * E + g);
#pragma unroll
            for (int p = 0; p < V * kNB; p++) s_u[p * ncol + kTile + hl] = v[p];
        }
    }
    // the element's packed face slots, for the gather after the faces
    int code[6] = {0, 0, 0, 0, 0, 0};
    const int l = threadIdx.x;
    const int64_t e = e_begin + l;
    if (l < nloc) {
#pragma unroll
        for (int f = 0; f < 6; f++) code[f] = __ldg(tl.slot + (int64_t) f * E + e);
    }
    if (bulk && !mbar_wait(&bar, 0, 1u << 20)) {
        // the copies did not land: report, wait (bounded) once more so that
        // none is still writing this CTA's shared memory, and stop
        if (threadIdx.x == 0) set_error(err, kErrWait);
        mbar_wait(&bar, 0, 1u << 20);
        return;
    }
    __syncthreads();
    // ---- faces of the tile ----
    const int f0 = tl.fptr[blockIdx.x], f1 = tl.fptr[blockIdx.x + 1];
    for (int j = f0 + threadIdx.x; j < f1; j += kTile) {
        const int4 r = __ldg(tl.rec + j);
        float *out = s_f + (int64_t) (j - f0) * 3 * V;
        if (r.z & kRecBoundary) {
            switch ((r.z & 7) >> 1) {
            case 0: tile_boundary<NC, FLUX, 0>(m, s_u, ncol, r, out, err); break;
            case 1: tile_boundary<NC, FLUX, 1>(m, s_u, ncol, r, out, err); break;
            default: tile_boundary<NC, FLUX, 2>(m, s_u, ncol, r, out, err); break;
            }
        } else {
            tile_interior<NC, FLUX>(m, s_u, ncol, r, out, err);
        }
    }
    __syncthreads();
    if (l >= nloc) return;
    // ---- element: volume integral, gather, update ----
    const int lev = m.level[e];
    const float hx = level_ht<float>(m, lev, 0), hy = level_ht<float>(m, lev, 1), hz = level_ht<float>(m, lev, 2);
    const float vol = hx * hy * hz;
    float c[V][kNB];
    col_coef<V>(s_u, ncol, l, c);
    float R[V][kNB], R0l[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
        R0l[v] = 0.f;
#pragma unroll
        for (int k = 0; k < kNB; k++) R[v][k] = 0.f;
    }
    {
        float F[V], G[V], H[V];
#pragma unroll
        for (int v = 0; v < V; v++) F[v] = G[v] = H[v] = 0.f;
        const bool grav = c_cfg.has_grav != 0;
        float gr[3][kNB];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int k = 0; k < kNB; k++) gr[a][k] = 0.f;
#pragma unroll 1
        for (int g = 0; g < 8; g++) {
            const float px = (g & 1) ? (float) kGaussPhi : -(float) kGaussPhi;
            const float py = (g & 2) ? (float) kGaussPhi : -(float) kGaussPhi;
            const float pz = (g & 4) ? (float) kGaussPhi : -(float) kGaussPhi;
            float U[V];
#pragma unroll
            for (int v = 0; v < V; v++) U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
            Prim<float, NC> p;
            cons_to_prim<float, NC>(U, p);
            if (!(p.r > 0.f) || !(p.p > 0.f)) set_error(err, (isfinite(p.r) && isfinite(p.p)) ? kErrNegative : kErrNonFinite);
            const auto hp = U[3] + p.p;   // r e_tot + p: the energy fluxes are u hp, v hp, w hp
            F[0] += U[0] * p.u + p.p; F[1] += U[0] * p.v; F[2] += U[0] * p.w; F[3] += p.u * hp;
            G[0] += U[1] * p.u; G[1] += U[1] * p.v + p.p; G[2] += U[1] * p.w; G[3] += p.v * hp;
            H[0] += U[2] * p.u; H[1] += U[2] * p.v; H[2] += U[2] * p.w + p.p; H[3] += p.w * hp;
#pragma unroll
            for (int i = 0; i < NC; i++) {
                F[4 + i] += U[0] * p.c[i];
                G[4 + i] += U[1] * p.c[i];
                H[4 + i] += U[2] * p.c[i];
            }
            if (grav) {
                const float phi[4] = {1.f, px, py, pz};
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int k = 0; k < kNB; k++) gr[a][k] += p.r * c_cfg.grav_f[a] * phi[k];
            }
        }
        const float w8 = vol * 0.125f;
#pragma unroll
        for (int v = 0; v < V; v++) {
            R[v][1] -= F[v] * (w8 / hx);
            R[v][2] -= G[v] * (w8 / hy);
            R[v][3] -= H[v] * (w8 / hz);
        }
        if (grav) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                acc0(R[a][0], R0l[a], -gr[a][0] * w8);
#pragma unroll
                for (int k = 1; k < kNB; k++) R[a][k] -= gr[a][k] * w8;
            }
        }
    }
    tile_gather_axis<NC, 0>(s_f, code, R, R0l);
    tile_gather_axis<NC, 1>(s_f, code, R, R0l);
    tile_gather_axis<NC, 2>(s_f, code, R, R0l);
    if (dt_dev) {
        const double d = *dt_dev;
        dth = __double2float_rn(d);
        dtl = __double2float_rn(d - (double) dth);
    }
    const float minv0 = 1.f / vol, minv1 = 12.f / vol;
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            FF x = {c[v][k], ul[idx]};
            FF y;
            if (k == 0) {
                const float rh = __fmul_rn(R[v][0], minv0);
                const float rl = __fmaf_rn(R0l[v], minv0, __fmaf_rn(R[v][0], minv0, -rh));
                y = ff_sub_scaled(x, rh, dth, dtl);
                y = ff_sub_scaled(y, rl, dth, dtl);
            } else {
                y = ff_sub_scaled(x, R[v][k] * minv1, dth, dtl);
            }
            if (comb) {
                const FF w0 = {u0h[idx], u0l[idx]};
                y = ff_comb(y, w0, ah, al, bh, bl);
            }
            oh[idx] = y.h;
            ol[idx] = y.l;
        }
    }
}

// ---------------------------------------------------------------------------
// output
// ---------------------------------------------------------------------------

// cell-centre primitive fields (the Taylor basis is 1, 0, 0, ... at the
// centre: the conserved values are the coefficient-0 planes)
template <int NC>
__global__ void __launch_bounds__(256) cell_fields_kernel(const double *__restrict__ u, int64_t E, int nb,
                                                          double *__restrict__ out)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double U[V];
    for (int v = 0; v < V; v++) U[v] = u[(int64_t) (v * nb) * E + e];
    Prim<double, NC> p;
    cons_to_prim<double, NC>(U, p);
    const double f[8] = {p.r, p.p, p.e, p.e_tot, p.u, p.v, p.w, p.t};
    for (int k = 0; k < 8; k++) out[(int64_t) k * E + e] = f[k];
    for (int i = 0; i < NC; i++) out[(int64_t) (8 + i) * E + e] = p.c[i];
}


}  // namespace charm
