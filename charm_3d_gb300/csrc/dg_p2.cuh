// p2 path: the 10-function Taylor basis of charm_base_func
// (src/charm_base_func.c:8-125 with CHARM_BASE_FN_COUNT = 10) on boxes,
// with a 27-point (3x3x3 Gauss) cell rule and a 9-point (3x3 Gauss) face
// rule: the reference's 8/6-point rules under-integrate p2.  Uniform
// (conforming) meshes; convective, viscous and chemistry terms.
//
// State [V][10][E]; slots [V*10][S] with the p1 face-record layout.  The
// kernels mirror the p1 ones (face pass into per-side slots, element-owned
// gather, no atomics); basis values come from the rule tables and the
// closed-form basis below, the mass matrix is the reference element's (the
// same for every box up to its volume), inverted once on the host.
//
// Every kernel is instantiated for T = double (the FP64 form) and T = float
// (the mixed form: arithmetic in FP32 on the hi plane of the FP32 hi/lo
// state, the update u - dt*M^-1*R and the SSP combination in float-float,
// chemistry and diffusion coefficients in FP64 from hi + lo).
//
// Structure used by both forms:
// - On a face along axis D every basis function is (normal coordinate)^p
//   times one of the six tangential monomials {1, a, b, a^2, b^2, ab}
//   (kTJ, kPW below), and the normal coordinate is +-1/2.  The projection of
//   a face flux on the 10 functions of either side is therefore a power of
//   1/2 times one of six tangential moments of the flux: 6 accumulators per
//   field instead of 2 x 10, with the same rounding as the direct sums
//   (scaling by a power of 2 is exact).
// - The gradient of a basis function has one or two non-zero components
//   (d(x^2)/dx = 2x, d(xy)/dx = y, ...); volume terms apply only those.
// - FP32 kernels read an element's coefficients once (cells) or reduce each
//   side's 10 coefficients to the 6 of its trace on the face once per face,
//   instead of re-reading them at every point.  The FP64 kernels read them
//   per point: they are bound by the FP64 pipe, not by loads.
#pragma once

#include "dg_launch.h"

namespace charm {

static __constant__ P2TabT<double> c_p2;
static __constant__ P2TabT<float> c_p2f;   // the same tables rounded to FP32

template <typename T> __device__ __forceinline__ T p2_cx(int g, int a)
{
    if constexpr (sizeof(T) == sizeof(float)) return c_p2f.cxi[g][a]; else return c_p2.cxi[g][a];
}
template <typename T> __device__ __forceinline__ T p2_cw(int g)
{
    if constexpr (sizeof(T) == sizeof(float)) return c_p2f.cw[g]; else return c_p2.cw[g];
}
template <typename T> __device__ __forceinline__ T p2_fx(int g, int a)
{
    if constexpr (sizeof(T) == sizeof(float)) return c_p2f.fxi[g][a]; else return c_p2.fxi[g][a];
}
template <typename T> __device__ __forceinline__ T p2_fw(int g)
{
    if constexpr (sizeof(T) == sizeof(float)) return c_p2f.fw[g]; else return c_p2.fw[g];
}
template <typename T> __device__ __forceinline__ T p2_minv(int i, int j)
{
    if constexpr (sizeof(T) == sizeof(float)) return c_p2f.minv[i][j]; else return c_p2.minv[i][j];
}
template <typename T> __device__ __forceinline__ T p2_mean(int k)
{
    if constexpr (sizeof(T) == sizeof(float)) return c_p2f.mean[k]; else return c_p2.mean[k];
}

// basis values at reference coordinates (x, y, z) = (x - c) / h
template <typename T>
__device__ __forceinline__ void basis10(T x, T y, T z, T phi[kNB2])
{
    phi[0] = T(1); phi[1] = x; phi[2] = y; phi[3] = z;
    phi[4] = x * x; phi[5] = y * y; phi[6] = z * z;
    phi[7] = x * y; phi[8] = x * z; phi[9] = y * z;
}

// point on face D of a box: the normal coordinate xd, tangential (xs, xt)
template <int D, typename T>
__device__ __forceinline__ void face_basis10(T xd, T xs, T xt, T phi[kNB2])
{
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    T r[3];
    r[D] = xd; r[s] = xs; r[t] = xt;
    basis10<T>(r[0], r[1], r[2], phi);
}

// face along axis D: basis function k = xd^kPW[D][k] * tangential monomial
// kTJ[D][k] of {1, a, b, a^2, b^2, ab} (a, b: the lower and upper tangential
// reference coordinates)
__device__ constexpr int kTJ[3][kNB2] = {{0, 0, 1, 2, 0, 3, 4, 1, 2, 5},
                                         {0, 1, 0, 2, 3, 0, 4, 1, 5, 2},
                                         {0, 1, 2, 0, 3, 4, 0, 5, 1, 2}};
__device__ constexpr int kPW[3][kNB2] = {{0, 1, 0, 0, 2, 0, 0, 1, 1, 0},
                                         {0, 0, 1, 0, 0, 2, 0, 1, 0, 1},
                                         {0, 0, 0, 1, 0, 0, 2, 0, 1, 1}};

template <typename T>
__device__ __forceinline__ void mono6(T a, T b, T mn[6])
{
    mn[0] = T(1); mn[1] = a; mn[2] = b; mn[3] = a * a; mn[4] = b * b; mn[5] = a * b;
}

// xd^p for xd = sg/2, sg = +-1: 1, sg/2, 1/4
template <typename T>
__device__ __forceinline__ T half_pow(int p, T sg)
{
    return p == 0 ? T(1) : (p == 1 ? T(0.5) * sg : T(0.25));
}

template <typename T, int V>
__device__ __forceinline__ void eval10(const T *__restrict__ u, int64_t E, int64_t e, const T phi[kNB2], T U[V])
{
#pragma unroll
    for (int v = 0; v < V; v++) {
        T x = T(0);
#pragma unroll
        for (int k = 0; k < kNB2; k++) x += __ldg(u + (int64_t) (v * kNB2 + k) * E + e) * phi[k];
        U[v] = x;
    }
}

template <typename T, int V>
__device__ __forceinline__ void load10(const T *__restrict__ u, int64_t E, int64_t e, T c[V][kNB2])
{
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) c[v][k] = __ldg(u + (int64_t) (v * kNB2 + k) * E + e);
}

template <typename T, int V>
__device__ __forceinline__ void evalc10(const T c[V][kNB2], const T phi[kNB2], T U[V])
{
#pragma unroll
    for (int v = 0; v < V; v++) {
        T x = T(0);
#pragma unroll
        for (int k = 0; k < kNB2; k++) x += c[v][k] * phi[k];
        U[v] = x;
    }
}

// the 6 coefficients of the trace of fields [0, V) of element e on its face
// along D at normal coordinate sg/2
template <typename T, int V, int D>
__device__ __forceinline__ void trace6(const T *__restrict__ u, int64_t E, int64_t e, T sg, T c6[V][6])
{
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int j = 0; j < 6; j++) c6[v][j] = T(0);
#pragma unroll
        for (int k = 0; k < kNB2; k++)
            c6[v][kTJ[D][k]] += __ldg(u + (int64_t) (v * kNB2 + k) * E + e) * half_pow<T>(kPW[D][k], sg);
    }
}

template <typename T, int V>
__device__ __forceinline__ void eval6(const T c6[V][6], const T mn[6], T U[V])
{
#pragma unroll
    for (int v = 0; v < V; v++) {
        T x = c6[v][0];
#pragma unroll
        for (int j = 1; j < 6; j++) x += c6[v][j] * mn[j];
        U[v] = x;
    }
}

// r = M^-1 a for one field on the reference box: odd moments vanish, so the
// inverse mass matrix couples {1, x^2, y^2, z^2} (k = 0, 4, 5, 6) in a 4x4
// block and is diagonal on the other six functions (the host stores the
// vanishing entries as exact zeros; same sums as the dense product)
template <typename T>
__device__ __forceinline__ void minv10(const T a[kNB2], T r[kNB2])
{
    constexpr int blk[4] = {0, 4, 5, 6};
    constexpr int dia[6] = {1, 2, 3, 7, 8, 9};
#pragma unroll
    for (int i = 0; i < 6; i++) r[dia[i]] = p2_minv<T>(dia[i], dia[i]) * a[dia[i]];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        T x = T(0);
#pragma unroll
        for (int j = 0; j < 4; j++) x += p2_minv<T>(blk[i], blk[j]) * a[blk[j]];
        r[blk[i]] = x;
    }
}

// R[k] += a * d(phi_k)/dx (resp. b d/dy, c d/dz) at (x, y, z)
template <typename T> __device__ __forceinline__ void add_gx(T R[kNB2], T a, T x, T y, T z)
{
    R[1] += a; R[4] += T(2) * x * a; R[7] += y * a; R[8] += z * a;
}
template <typename T> __device__ __forceinline__ void add_gy(T R[kNB2], T b, T x, T y, T z)
{
    R[2] += b; R[5] += T(2) * y * b; R[7] += x * b; R[9] += z * b;
}
template <typename T> __device__ __forceinline__ void add_gz(T R[kNB2], T c, T x, T y, T z)
{
    R[3] += c; R[6] += T(2) * z * c; R[8] += x * c; R[9] += y * c;
}

template <typename T> __device__ __forceinline__ void add_pair(T *slots, int64_t idx, T a, T b);
template <> __device__ __forceinline__ void add_pair<double>(double *slots, int64_t idx, double a, double b)
{
    double2 *p = reinterpret_cast<double2 *>(slots + idx);
    p->x += a;
    p->y += b;
}
template <> __device__ __forceinline__ void add_pair<float>(float *slots, int64_t idx, float a, float b)
{
    float2 *p = reinterpret_cast<float2 *>(slots + idx);
    p->x += a;
    p->y += b;
}

// Projections of an interior face's moments M on both sides' basis: side 0
// (normal coordinate +1/2) gets s0 * sum flux phi0, side 1 (-1/2) gets
// s1 * sum flux phi1; stored, or added to the slots' values (ADD).
template <typename T, int NF, int D, bool ADD>
__device__ __forceinline__ void put_interior(T *__restrict__ slots, int64_t S, int64_t base, const T M[NF][6], T s0,
                                             T s1)
{
#pragma unroll
    for (int f = 0; f < NF; f++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) {
            const T a0 = half_pow<T>(kPW[D][k], T(1)) * M[f][kTJ[D][k]];
            const T a1 = half_pow<T>(kPW[D][k], T(-1)) * M[f][kTJ[D][k]];
            if constexpr (ADD) add_pair<T>(slots, (int64_t) (f * kNB2 + k) * S + base, s0 * a0, s1 * a1);
            else store_pair<T>(slots, (int64_t) (f * kNB2 + k) * S + base, s0 * a0, s1 * a1);
        }
}

// ---------------------------------------------------------------------------
// convective face pass
// ---------------------------------------------------------------------------

template <typename T, int NC, int FLUX, int D>
__device__ __forceinline__ void p2_interior(const MeshDev &m, const T *__restrict__ u, T *__restrict__ slots,
                                            int64_t i, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e0 = m.face_elem[i], e1 = m.face_elem[m.n_face + i];
    const int lev = m.level[e0];
    const T area = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t);
    T n[3] = {T(0), T(0), T(0)};
    n[D] = T(1);
    T ca[kF ? V : 1][6], cb[kF ? V : 1][6];
    if constexpr (kF) {
        trace6<T, V, D>(u, E, e0, T(1), ca);
        trace6<T, V, D>(u, E, e1, T(-1), cb);
    }
    T M[V][6];
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int j = 0; j < 6; j++) M[v][j] = T(0);
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        T mn[6], U0[V], U1[V];
        mono6<T>(p2_fx<T>(g, 0), p2_fx<T>(g, 1), mn);
        if constexpr (kF) {
            eval6<T, V>(ca, mn, U0);
            eval6<T, V>(cb, mn, U1);
        } else {
            T p0[kNB2], p1[kNB2];
            face_basis10<D, T>(T(0.5), mn[1], mn[2], p0);
            face_basis10<D, T>(T(-0.5), mn[1], mn[2], p1);
            eval10<T, V>(u, E, e0, p0, U0);
            eval10<T, V>(u, E, e1, p1, U1);
        }
        Prim<T, NC> pa, pb;
        cons_to_prim<T, NC>(U0, pa);
        cons_to_prim<T, NC>(U1, pb);
        T q[V];
        num_flux<FLUX, T, NC, D>(pa, pb, n, q, err);
        const T w = area * p2_fw<T>(g);
#pragma unroll
        for (int v = 0; v < V; v++) {
            const T qw = q[v] * w;
#pragma unroll
            for (int j = 0; j < 6; j++) M[v][j] += qw * mn[j];
        }
    }
    put_interior<T, V, D, false>(slots, S, 2 * i, M, T(1), T(-1));
}

template <typename T, int NC, int FLUX, int D>
__device__ __forceinline__ void p2_boundary(const MeshDev &m, const T *__restrict__ u, T *__restrict__ slots,
                                            int64_t j, unsigned *err)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
    const T sg = (f & 1) ? T(1) : T(-1);
    const int lev = m.level[e];
    const T area = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t);
    T n[3] = {T(0), T(0), T(0)};
    n[D] = sg;
    T ca[kF ? V : 1][6];
    if constexpr (kF) trace6<T, V, D>(u, E, e, sg, ca);
    T M[V][6];
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < 6; k++) M[v][k] = T(0);
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        T mn[6], U[V];
        mono6<T>(p2_fx<T>(g, 0), p2_fx<T>(g, 1), mn);
        if constexpr (kF) {
            eval6<T, V>(ca, mn, U);
        } else {
            T ph[kNB2];
            face_basis10<D, T>(T(0.5) * sg, mn[1], mn[2], ph);
            eval10<T, V>(u, E, e, ph, U);
        }
        Prim<T, NC> pin, pout;
        cons_to_prim<T, NC>(U, pin);
        bnd_cond<T, NC>(bid, pin, pout, n);
        T q[V];
        num_flux<FLUX, T, NC, D>(pin, pout, n, q, err);
        const T w = area * p2_fw<T>(g);
#pragma unroll
        for (int v = 0; v < V; v++) {
            const T qw = q[v] * w;
#pragma unroll
            for (int k = 0; k < 6; k++) M[v][k] += qw * mn[k];
        }
    }
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++)
            slots[(int64_t) (v * kNB2 + k) * S + slot] = half_pow<T>(kPW[D][k], sg) * M[v][kTJ[D][k]];
}

template <typename T, int NC, int FLUX>
__global__ void __launch_bounds__(128)
p2_face_kernel(MeshDev m, const T *__restrict__ u, T *__restrict__ slots, int64_t n_int_blocks, unsigned *err)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: p2_interior<T, NC, FLUX, 0>(m, u, slots, i, err); break;
        case 1: p2_interior<T, NC, FLUX, 1>(m, u, slots, i, err); break;
        default: p2_interior<T, NC, FLUX, 2>(m, u, slots, i, err); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        switch (m.bface_face[j] >> 1) {
        case 0: p2_boundary<T, NC, FLUX, 0>(m, u, slots, j, err); break;
        case 1: p2_boundary<T, NC, FLUX, 1>(m, u, slots, j, err); break;
        default: p2_boundary<T, NC, FLUX, 2>(m, u, slots, j, err); break;
        }
    }
}

// ---------------------------------------------------------------------------
// cell pass: volume integral (27 points), gather, M^-1, update
// ---------------------------------------------------------------------------


template <typename T, int NC>
__global__ void __launch_bounds__(128)
p2_cell_kernel(MeshDev m, const T *__restrict__ u, const T *__restrict__ slots, const T *u0, T *out, P2Upd up,
               unsigned *err, const T *__restrict__ radd)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const T hx = level_ht<T>(m, lev, 0), hy = level_ht<T>(m, lev, 1), hz = level_ht<T>(m, lev, 2);
    const T vol = hx * hy * hz;
    const T ihx = T(1) / hx, ihy = T(1) / hy, ihz = T(1) / hz;
    const bool grav = c_cfg.has_grav != 0;
    T c[kF ? V : 1][kNB2];
    if constexpr (kF) load10<T, V>(u, E, e, c);
    T R[V][kNB2];
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) R[v][k] = T(0);
#pragma unroll 1
    for (int g = 0; g < 27; g++) {
        const T x = p2_cx<T>(g, 0), y = p2_cx<T>(g, 1), z = p2_cx<T>(g, 2);
        T ph[kNB2], U[V];
        basis10<T>(x, y, z, ph);
        if constexpr (kF) evalc10<T, V>(c, ph, U);
        else eval10<T, V>(u, E, e, ph, U);
        Prim<T, NC> p;
        cons_to_prim<T, NC>(U, p);
        if (!(p.r > T(0)) || !(p.p > T(0))) set_error(err, isfinite(p.r) && isfinite(p.p) ? kErrNegative : kErrNonFinite);
        T F[V], G[V], H[V];
        const T hp = U[3] + p.p;   // r e_tot + p: the energy fluxes are u hp, v hp, w hp
        F[0] = U[0] * p.u + p.p; F[1] = U[0] * p.v; F[2] = U[0] * p.w; F[3] = p.u * hp;
        G[0] = U[1] * p.u; G[1] = U[1] * p.v + p.p; G[2] = U[1] * p.w; G[3] = p.v * hp;
        H[0] = U[2] * p.u; H[1] = U[2] * p.v; H[2] = U[2] * p.w + p.p; H[3] = p.w * hp;
#pragma unroll
        for (int k = 0; k < NC; k++) { F[4 + k] = U[0] * p.c[k]; G[4 + k] = U[1] * p.c[k]; H[4 + k] = U[2] * p.c[k]; }
        const T w = vol * p2_cw<T>(g);
        const T wx = w * ihx, wy = w * ihy, wz = w * ihz;
#pragma unroll
        for (int v = 0; v < V; v++) {
            add_gx<T>(R[v], -F[v] * wx, x, y, z);
            add_gy<T>(R[v], -G[v] * wy, x, y, z);
            add_gz<T>(R[v], -H[v] * wz, x, y, z);
        }
        if (grav) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const T ga = p.r * cfgv<T>(c_cfg.grav[a], c_cfg.grav_f[a]);
#pragma unroll
                for (int k = 0; k < kNB2; k++) R[a][k] -= ga * ph[k] * w;
            }
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
    if (up.mode == kCellResidual) {
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB2; k++) out[(int64_t) (v * kNB2 + k) * E + e] = R[v][k];
        return;
    }
    const T iv = T(1) / vol;
    if constexpr (kF) {
        const bool comb = (u0 != nullptr);
#pragma unroll
        for (int v = 0; v < V; v++) {
            T r[kNB2];
            minv10<T>(R[v], r);
#pragma unroll
            for (int i = 0; i < kNB2; i++) {
                const int64_t idx = (int64_t) (v * kNB2 + i) * E + e;
                FF x = ff_sub_scaled(FF{c[v][i], __ldg(up.u_lo + idx)}, r[i] * iv, up.dt_h, up.dt_l);
                if (comb) x = ff_comb(x, FF{u0[idx], up.u0_lo[idx]}, up.a_h, up.a_l, up.b_h, up.b_l);
                out[idx] = x.h;
                up.out_lo[idx] = x.l;
            }
        }
    } else {
        const double step = up.dt_dev ? *up.dt_dev : up.dt;
        const bool comb = (up.a_old != 0.0);
#pragma unroll
        for (int v = 0; v < V; v++) {
            T r[kNB2];
            minv10<T>(R[v], r);
#pragma unroll
            for (int i = 0; i < kNB2; i++) {
                const int64_t idx = (int64_t) (v * kNB2 + i) * E + e;
                double x = __ldg(u + idx) - step * (r[i] * iv);
                if (comb) x = up.a_new * x + up.a_old * u0[idx];
                out[idx] = x;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// chemistry on cell means (FP64 in both forms; the mixed form reads and
// writes the hi/lo planes)
// ---------------------------------------------------------------------------

template <typename S, int NC>
__global__ void __launch_bounds__(128)
p2_chem_kernel(MeshDev m, StIn<S> u, StOut<S> out, double *__restrict__ chem_rhs)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double U[V];
#pragma unroll
    for (int v = 0; v < V; v++) {   // charm_get_fields_avg
        double x = 0.0;
#pragma unroll
        for (int k = 0; k < kNB2; k++) x += u.at((int64_t) (v * kNB2 + k) * E + e) * c_p2.mean[k];
        U[v] = x;
    }
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
        for (int kk = 0; kk < kNB2; kk++) out.copy((int64_t) (v * kNB2 + kk) * E + e, u);
#pragma unroll
    for (int i = 0; i < NC; i++) {
        out.put((int64_t) ((4 + i) * kNB2) * E + e, ch[i] * c_cfg.comp_m[i]);
#pragma unroll
        for (int kk = 1; kk < kNB2; kk++) out.put((int64_t) ((4 + i) * kNB2 + kk) * E + e, 0.);
    }
}

// ---------------------------------------------------------------------------
// viscous terms (the p1 kernels' arithmetic on the p2 basis)
// ---------------------------------------------------------------------------

template <typename T, int NC, int D>
__device__ __forceinline__ void p2_vgrad_interior(const MeshDev &m, const T *__restrict__ u,
                                                  const T *__restrict__ dif, T *__restrict__ s9, int64_t i)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e0 = m.face_elem[i], e1 = m.face_elem[m.n_face + i];
    const int lev = m.level[e0];
    const T area = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t);
    T n[3] = {T(0), T(0), T(0)};
    n[D] = T(1);
    T dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = (dif[(int64_t) c * E + e0] + dif[(int64_t) c * E + e1]) * T(0.5);
    T ca[kF ? V : 1][6], cb[kF ? V : 1][6];
    if constexpr (kF) {
        trace6<T, V, D>(u, E, e0, T(1), ca);
        trace6<T, V, D>(u, E, e1, T(-1), cb);
    }
    T M[9][6];   // [field][moment], weight included, heat rows negated
#pragma unroll
    for (int f = 0; f < 9; f++)
#pragma unroll
        for (int j = 0; j < 6; j++) M[f][j] = T(0);
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        T mn[6], Ua[V], Ub[V];
        mono6<T>(p2_fx<T>(g, 0), p2_fx<T>(g, 1), mn);
        if constexpr (kF) {
            eval6<T, V>(ca, mn, Ua);
            eval6<T, V>(cb, mn, Ub);
        } else {
            T p0[kNB2], p1[kNB2];
            face_basis10<D, T>(T(0.5), mn[1], mn[2], p0);
            face_basis10<D, T>(T(-0.5), mn[1], mn[2], p1);
            eval10<T, V>(u, E, e0, p0, Ua);
            eval10<T, V>(u, E, e1, p1, Ub);
        }
        Prim<T, NC> pa, pb;
        cons_to_prim<T, NC>(Ua, pa);
        cons_to_prim<T, NC>(Ub, pb);
        T mua, kta, mub, ktb;
        transport<NC>(pa, mua, kta);
        transport<NC>(pb, mub, ktb);
        T fc[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) fc[c] = (pa.c[c] + pb.c[c]) * T(0.5);
        T q[9];
        vgrad_q<NC>(T(0.5) * (mua + mub), (kta + ktb) * T(0.5), (pa.r + pb.r) * T(0.5), (pa.t + pb.t) * T(0.5),
                    (pa.u + pb.u) * T(0.5), (pa.v + pb.v) * T(0.5), (pa.w + pb.w) * T(0.5), fc, dm, n, q);
        const T w = area * p2_fw<T>(g);
#pragma unroll
        for (int f = 0; f < 9; f++) {
            const T qw = (f < 6 ? w : -w) * q[f];
#pragma unroll
            for (int j = 0; j < 6; j++) M[f][j] += qw * mn[j];
        }
    }
    put_interior<T, 9, D, false>(s9, S, 2 * i, M, T(1), T(-1));
}

template <typename T, int NC, int D>
__device__ __forceinline__ void p2_vgrad_boundary(const MeshDev &m, const T *__restrict__ u,
                                                  const T *__restrict__ dif, T *__restrict__ s9, int64_t j)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
    const T sg = (f & 1) ? T(1) : T(-1);
    const int lev = m.level[e];
    const T area = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t);
    const bool noslip = c_cfg.bnd_type[bid] == CHARM_GPU_BND_WALL_NO_SLIP;
    T n[3] = {T(0), T(0), T(0)};
    n[D] = sg;
    T dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = dif[(int64_t) c * E + e];
    T ca[kF ? V : 1][6];
    if constexpr (kF) trace6<T, V, D>(u, E, e, sg, ca);
    T M[9][6];
#pragma unroll
    for (int r = 0; r < 9; r++)
#pragma unroll
        for (int k = 0; k < 6; k++) M[r][k] = T(0);
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        T mn[6], U[V];
        mono6<T>(p2_fx<T>(g, 0), p2_fx<T>(g, 1), mn);
        if constexpr (kF) {
            eval6<T, V>(ca, mn, U);
        } else {
            T ph[kNB2];
            face_basis10<D, T>(T(0.5) * sg, mn[1], mn[2], ph);
            eval10<T, V>(u, E, e, ph, U);
        }
        Prim<T, NC> pin, pout;
        cons_to_prim<T, NC>(U, pin);
        T mu, kt;
        transport<NC>(pin, mu, kt);
        bnd_cond<T, NC>(bid, pin, pout, n);
        T fu, fv, fw, ft;
        if (noslip) {
            fu = fv = fw = T(0);
            ft = cfgv<T>(c_cfg.bnd_par[bid][0], c_cfg.bnd_par_f[bid][0]);
        } else {
            fu = (pin.u + pout.u) * T(0.5); fv = (pin.v + pout.v) * T(0.5);
            fw = (pin.w + pout.w) * T(0.5); ft = (pin.t + pout.t) * T(0.5);
        }
        T fc[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) fc[c] = (pin.c[c] + pout.c[c]) * T(0.5);
        T q[9];
        vgrad_q<NC>(mu, kt, (pin.r + pout.r) * T(0.5), ft, fu, fv, fw, fc, dm, n, q);
        const T w = area * p2_fw<T>(g);
#pragma unroll
        for (int r = 0; r < 9; r++) {
            const T qw = (r < 6 ? w : -w) * q[r];
#pragma unroll
            for (int k = 0; k < 6; k++) M[r][k] += qw * mn[k];
        }
    }
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int r = 0; r < 9; r++)
#pragma unroll
        for (int k = 0; k < kNB2; k++)
            s9[(int64_t) (r * kNB2 + k) * S + slot] = half_pow<T>(kPW[D][k], sg) * M[r][kTJ[D][k]];
}

template <typename T, int NC>
__global__ void __launch_bounds__(128)
p2_vgrad_face_kernel(MeshDev m, const T *__restrict__ u, const T *__restrict__ dif, T *__restrict__ s9,
                     int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: p2_vgrad_interior<T, NC, 0>(m, u, dif, s9, i); break;
        case 1: p2_vgrad_interior<T, NC, 1>(m, u, dif, s9, i); break;
        default: p2_vgrad_interior<T, NC, 2>(m, u, dif, s9, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        switch (m.bface_face[j] >> 1) {
        case 0: p2_vgrad_boundary<T, NC, 0>(m, u, dif, s9, j); break;
        case 1: p2_vgrad_boundary<T, NC, 1>(m, u, dif, s9, j); break;
        default: p2_vgrad_boundary<T, NC, 2>(m, u, dif, s9, j); break;
        }
    }
}

// lifting volume term + gather + M^-1 -> vis [9][10][E]
template <typename T, int NC>
__global__ void __launch_bounds__(128)
p2_vgrad_cell_kernel(MeshDev m, const T *__restrict__ u, const T *__restrict__ dif, const T *__restrict__ s9,
                     T *__restrict__ vis)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const T hx = level_ht<T>(m, lev, 0), hy = level_ht<T>(m, lev, 1), hz = level_ht<T>(m, lev, 2);
    const T vol = hx * hy * hz;
    const T ihx = T(1) / hx, ihy = T(1) / hy, ihz = T(1) / hz;
    T dm[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) dm[c] = dif[(int64_t) c * E + e];
    T c[kF ? V : 1][kNB2];
    if constexpr (kF) load10<T, V>(u, E, e, c);
    T a[9][kNB2];
#pragma unroll
    for (int f = 0; f < 9; f++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) a[f][k] = T(0);
#pragma unroll 1
    for (int g = 0; g < 27; g++) {
        const T x = p2_cx<T>(g, 0), y = p2_cx<T>(g, 1), z = p2_cx<T>(g, 2);
        T ph[kNB2], U[V];
        basis10<T>(x, y, z, ph);
        if constexpr (kF) evalc10<T, V>(c, ph, U);
        else eval10<T, V>(u, E, e, ph, U);
        Prim<T, NC> p;
        cons_to_prim<T, NC>(U, p);
        T kt, mu;
        transport<NC>(p, mu, kt);
        const T lp = mu * T(4.0 / 3.0), lm = mu * T(-2.0 / 3.0);
        T hq = kt * p.t;
#pragma unroll
        for (int k = 0; k < NC; k++) hq += comp_h<T>(k, p.t) * p.r * dm[k] * p.c[k];
        const T w = vol * p2_cw<T>(g);
        const T wx = w * ihx, wy = w * ihy, wz = w * ihz;
        // a[f][k] -= X d(phi_k)/dx + Y d(phi_k)/dy + Z d(phi_k)/dz (physical derivatives)
        add_gx<T>(a[0], -lp * p.u * wx, x, y, z); add_gy<T>(a[0], -lm * p.v * wy, x, y, z); add_gz<T>(a[0], -lm * p.w * wz, x, y, z);
        add_gx<T>(a[1], -lm * p.u * wx, x, y, z); add_gy<T>(a[1], -lp * p.v * wy, x, y, z); add_gz<T>(a[1], -lm * p.w * wz, x, y, z);
        add_gx<T>(a[2], -lm * p.u * wx, x, y, z); add_gy<T>(a[2], -lm * p.v * wy, x, y, z); add_gz<T>(a[2], -lp * p.w * wz, x, y, z);
        add_gx<T>(a[3], -mu * p.v * wx, x, y, z); add_gy<T>(a[3], -mu * p.u * wy, x, y, z);
        add_gx<T>(a[4], -mu * p.w * wx, x, y, z); add_gz<T>(a[4], -mu * p.u * wz, x, y, z);
        add_gy<T>(a[5], -mu * p.w * wy, x, y, z); add_gz<T>(a[5], -mu * p.v * wz, x, y, z);
        add_gx<T>(a[6], hq * wx, x, y, z);
        add_gy<T>(a[7], hq * wy, x, y, z);
        add_gz<T>(a[8], hq * wz, x, y, z);
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
    const T iv = T(1) / vol;
#pragma unroll
    for (int f = 0; f < 9; f++) {
        T r[kNB2];
        minv10<T>(a[f], r);
#pragma unroll
        for (int i = 0; i < kNB2; i++) vis[(int64_t) (f * kNB2 + i) * E + e] = r[i] * iv;
    }
}

template <typename T>
__device__ __forceinline__ void vis_at10(const T *__restrict__ vis, int64_t E, int64_t e, const T phi[kNB2], T t[9])
{
#pragma unroll
    for (int f = 0; f < 9; f++) {
        T x = T(0);
#pragma unroll
        for (int k = 0; k < kNB2; k++) x += __ldg(vis + (int64_t) (f * kNB2 + k) * E + e) * phi[k];
        t[f] = x;
    }
}

template <typename T, int NC, int D>
__device__ __forceinline__ void p2_vflux_interior(const MeshDev &m, const T *__restrict__ u,
                                                  const T *__restrict__ vis, T *__restrict__ slots, int64_t i)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    constexpr int s = (D == 0) ? 1 : 0, t = (D == 2) ? 1 : 2;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e[2] = {m.face_elem[i], m.face_elem[m.n_face + i]};
    const int lev = m.level[e[0]];
    const T area = level_ht<T>(m, lev, s) * level_ht<T>(m, lev, t);
    constexpr int r0 = (D == 0) ? 0 : (D == 1) ? 3 : 4;
    constexpr int r1 = (D == 0) ? 3 : (D == 1) ? 1 : 5;
    constexpr int r2 = (D == 0) ? 4 : (D == 1) ? 5 : 2;
    // mixed form: traces of the state and of the lifted fields on both sides
    // (fields the flux does not use are eliminated by the compiler)
    T cu[kF ? 2 : 1][kF ? V : 1][6], cv[kF ? 2 : 1][kF ? 9 : 1][6];
    if constexpr (kF) {
#pragma unroll
        for (int sd = 0; sd < 2; sd++) {
            trace6<T, V, D>(u, E, e[sd], sd ? T(-1) : T(1), cu[sd]);
            trace6<T, 9, D>(vis, E, e[sd], sd ? T(-1) : T(1), cv[sd]);
        }
    }
    T M[4][6];
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int j = 0; j < 6; j++) M[v][j] = T(0);
#pragma unroll 1
    for (int g = 0; g < 9; g++) {
        T mn[6];
        mono6<T>(p2_fx<T>(g, 0), p2_fx<T>(g, 1), mn);
        T t6[6] = {T(0), T(0), T(0), T(0), T(0), T(0)}, fu = T(0), fv = T(0), fw = T(0), ft = T(0);
#pragma unroll
        for (int sd = 0; sd < 2; sd++) {
            T U[V], tq[9];
            if constexpr (kF) {
                eval6<T, V>(cu[sd], mn, U);
                eval6<T, 9>(cv[sd], mn, tq);
            } else {
                T ph[kNB2];
                face_basis10<D, T>(sd ? T(-0.5) : T(0.5), mn[1], mn[2], ph);
                eval10<T, V>(u, E, e[sd], ph, U);
                vis_at10<T>(vis, E, e[sd], ph, tq);
            }
            Prim<T, NC> p;
            cons_to_prim<T, NC>(U, p);
#pragma unroll
            for (int c = 0; c < 6; c++) t6[c] += tq[c];
            fu += p.u * tq[0] + p.v * tq[3] + p.w * tq[4];
            fv += p.u * tq[3] + p.v * tq[1] + p.w * tq[5];
            fw += p.u * tq[4] + p.v * tq[5] + p.w * tq[2];
            ft += tq[6 + D];
        }
        const T w = area * p2_fw<T>(g);
        T q[4];
        q[0] = T(0.5) * t6[r0] * w;
        q[1] = T(0.5) * t6[r1] * w;
        q[2] = T(0.5) * t6[r2] * w;
        q[3] = (T(0.5) * ((D == 0) ? fu : (D == 1) ? fv : fw) - T(0.5) * ft) * w;
#pragma unroll
        for (int v = 0; v < 4; v++)
#pragma unroll
            for (int j = 0; j < 6; j++) M[v][j] += q[v] * mn[j];
    }
    // the residual gets -flux phi0 on side 0 and +flux phi1 on side 1
    put_interior<T, 4, D, true>(slots, S, 2 * i, M, T(-1), T(1));
}

template <typename T, int NC>
__device__ __forceinline__ void p2_vflux_noslip(const MeshDev &m, const T *__restrict__ u,
                                                const T *__restrict__ vis, T *__restrict__ slots, int64_t j)
{
    constexpr int V = 4 + NC;
    const int64_t S = m.n_slot, E = m.n_elem;
    const int e = m.bface_elem[j], f = m.bface_face[j];
    const int d = f >> 1;
    const T sg = (f & 1) ? T(1) : T(-1);
    const int lev = m.level[e];
    const T hd = level_ht<T>(m, lev, d);
    const T area = level_ht<T>(m, lev, (d + 1) % 3) * level_ht<T>(m, lev, (d + 2) % 3);
    T r[3] = {T(0), T(0), T(0)};
    r[d] = T(0.5) * sg;
    T ph[kNB2], mean[kNB2], U[V], Um[V], tq[9];
    basis10<T>(r[0], r[1], r[2], ph);
#pragma unroll
    for (int k = 0; k < kNB2; k++) mean[k] = p2_mean<T>(k);
    eval10<T, V>(u, E, e, ph, U);
    eval10<T, V>(u, E, e, mean, Um);
    Prim<T, NC> px, pm;
    cons_to_prim<T, NC>(U, px);
    cons_to_prim<T, NC>(Um, pm);
    T mu, kt;
    transport<NC>(px, mu, kt);
    vis_at10<T>(vis, E, e, ph, tq);
    const T vv[3] = {pm.u, pm.v, pm.w};
    const T un = vv[d] * sg;
    T vt[3] = {vv[0], vv[1], vv[2]};
    vt[d] -= un * sg;
    const T ll = T(0.5) * hd;
    const T fl[4] = {-mu * vt[0] / ll, -mu * vt[1] / ll, -mu * vt[2] / ll, -tq[6 + d] * sg};
    const int64_t slot = 2 * m.n_face + j;
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) slots[(int64_t) (v * kNB2 + k) * S + slot] -= fl[v] * ph[k] * area;
}

template <typename T, int NC>
__global__ void __launch_bounds__(128)
p2_vflux_face_kernel(MeshDev m, const T *__restrict__ u, const T *__restrict__ vis, T *__restrict__ slots,
                     int64_t n_int_blocks)
{
    if ((int64_t) blockIdx.x < n_int_blocks) {
        const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= m.n_face) return;
        switch (m.face_info[i] & 3) {
        case 0: p2_vflux_interior<T, NC, 0>(m, u, vis, slots, i); break;
        case 1: p2_vflux_interior<T, NC, 1>(m, u, vis, slots, i); break;
        default: p2_vflux_interior<T, NC, 2>(m, u, vis, slots, i); break;
        }
    } else {
        const int64_t j = ((int64_t) blockIdx.x - n_int_blocks) * blockDim.x + threadIdx.x;
        if (j >= m.n_bface) return;
        if (c_cfg.bnd_type[m.bface_bnd[j]] == CHARM_GPU_BND_WALL_NO_SLIP) p2_vflux_noslip<T, NC>(m, u, vis, slots, j);
    }
}

// viscous volume terms (27 points) + chem_rhs -> radd [4][10][E]
template <typename T, int NC>
__global__ void __launch_bounds__(128)
p2_vvol_kernel(MeshDev m, const T *__restrict__ u, const T *__restrict__ vis, const double *__restrict__ chem_rhs,
               T *__restrict__ radd)
{
    constexpr int V = 4 + NC;
    constexpr bool kF = sizeof(T) == sizeof(float);
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    const int lev = m.level[e];
    const T hx = level_ht<T>(m, lev, 0), hy = level_ht<T>(m, lev, 1), hz = level_ht<T>(m, lev, 2);
    const T vol = hx * hy * hz;
    const T ihx = T(1) / hx, ihy = T(1) / hy, ihz = T(1) / hz;
    const T cr = chem_rhs ? T(chem_rhs[e]) : T(0);
    T c[kF ? V : 1][kNB2], cv[kF ? 9 : 1][kNB2];
    if constexpr (kF) {
        load10<T, V>(u, E, e, c);
        load10<T, 9>(vis, E, e, cv);
    }
    T R[4][kNB2];
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) R[v][k] = T(0);
#pragma unroll 1
    for (int g = 0; g < 27; g++) {
        const T x = p2_cx<T>(g, 0), y = p2_cx<T>(g, 1), z = p2_cx<T>(g, 2);
        T ph[kNB2], U[V], tq[9];
        basis10<T>(x, y, z, ph);
        if constexpr (kF) {
            evalc10<T, V>(c, ph, U);
            evalc10<T, 9>(cv, ph, tq);
        } else {
            eval10<T, V>(u, E, e, ph, U);
            vis_at10<T>(vis, E, e, ph, tq);
        }
        Prim<T, NC> p;
        cons_to_prim<T, NC>(U, p);
        const T w = vol * p2_cw<T>(g);
        const T wx = w * ihx, wy = w * ihy, wz = w * ihz;
        const T ex = tq[0] * p.u + tq[3] * p.v + tq[4] * p.w;
        const T ey = tq[3] * p.u + tq[1] * p.v + tq[5] * p.w;
        const T ez = tq[4] * p.u + tq[5] * p.v + tq[2] * p.w;
        add_gx<T>(R[0], tq[0] * wx, x, y, z); add_gy<T>(R[0], tq[3] * wy, x, y, z); add_gz<T>(R[0], tq[4] * wz, x, y, z);
        add_gx<T>(R[1], tq[3] * wx, x, y, z); add_gy<T>(R[1], tq[1] * wy, x, y, z); add_gz<T>(R[1], tq[5] * wz, x, y, z);
        add_gx<T>(R[2], tq[4] * wx, x, y, z); add_gy<T>(R[2], tq[5] * wy, x, y, z); add_gz<T>(R[2], tq[2] * wz, x, y, z);
        add_gx<T>(R[3], ex * wx, x, y, z); add_gy<T>(R[3], ey * wy, x, y, z); add_gz<T>(R[3], ez * wz, x, y, z);
        const T cw = cr * w;
#pragma unroll
        for (int k = 0; k < kNB2; k++) R[3][k] += cw * ph[k];
    }
#pragma unroll
    for (int v = 0; v < 4; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) radd[(int64_t) (v * kNB2 + k) * E + e] = R[v][k];
}

// ---------------------------------------------------------------------------
// Barth-Jespersen limiter on the p2 basis (src/limiters/charm_limiter_bj.c,
// whose loops run over CHARM_BASE_FN_COUNT) + SSP combination, FP64: the
// own and neighbour values are quadrature means (c_0 + (c_4 + c_5 + c_6)/12
// on a box), a hanging neighbour's is its centre value c_0, psi is the
// minimum over the 8 corners of the p2 field, and coefficients 1..9 are
// scaled by it.
// ---------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(128)
p2_limit_kernel(MeshDev m, const double *__restrict__ ua, const double *u0, double *out, double a_new, double a_old)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    auto mean = [&](int64_t x, double *U) {
#pragma unroll
        for (int v = 0; v < V; v++) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < kNB2; k++) s += __ldg(ua + (int64_t) (v * kNB2 + k) * E + x) * c_p2.mean[k];
            U[v] = s;
        }
    };
    double own[V], umin[V], umax[V];
    mean(e, own);
#pragma unroll
    for (int v = 0; v < V; v++) umin[v] = umax[v] = own[v];
#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        const int kind = m.lim_kind[(int64_t) f * E + e] & 3;
        const int idx = m.lim_idx[(int64_t) f * E + e];
        double nbv[V];
        if (kind == 0) {
            mean(idx, nbv);
        } else if (kind == 3) {
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = __ldg(ua + (int64_t) (v * kNB2) * E + idx);
        } else if (kind == 2) {
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
                for (int v = 0; v < V; v++) nbv[v] += __ldg(ua + (int64_t) (v * kNB2) * E + small) * vs;
            }
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] /= svol;
        } else {
            const int fb = m.bface_face[idx], bid = m.bface_bnd[idx];
            double n[3] = {0.0, 0.0, 0.0};
            n[fb >> 1] = (fb & 1) ? 1.0 : -1.0;
            Prim<double, NC> pin, pout;
            cons_to_prim<double, NC>(own, pin);
            bnd_cond<double, NC>(bid, pin, pout, n);
            prim_to_cons<double, NC>(pout, nbv);
        }
#pragma unroll
        for (int v = 0; v < V; v++) {
            if (umin[v] > nbv[v]) umin[v] = nbv[v];
            if (umax[v] < nbv[v]) umax[v] = nbv[v];
        }
    }
    // psi over the 8 corners: the largest and the most negative difference
    // per variable, then two quotients (bj_side_psi: the reference's
    // per-corner minimum)
    double psi[V], dmax[V], dmin[V];
#pragma unroll
    for (int v = 0; v < V; v++) dmax[v] = dmin[v] = 0.0;
#pragma unroll 1
    for (int vx = 0; vx < 8; vx++) {
        double ph[kNB2];
        basis10<double>((vx & 1) ? 0.5 : -0.5, (vx & 2) ? 0.5 : -0.5, (vx & 4) ? 0.5 : -0.5, ph);
#pragma unroll
        for (int v = 0; v < V; v++) {
            double f = 0.0;
#pragma unroll
            for (int k = 0; k < kNB2; k++) f += __ldg(ua + (int64_t) (v * kNB2 + k) * E + e) * ph[k];
            const double df = f - own[v];
            dmax[v] = fmax(dmax[v], df);
            dmin[v] = fmin(dmin[v], df);
        }
    }
#pragma unroll
    for (int v = 0; v < V; v++) psi[v] = bj_side_psi(dmax[v], dmin[v], umin[v] - own[v], umax[v] - own[v]);
    const bool comb = (a_old != 0.0);
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB2; k++) {
            const int64_t i = (int64_t) (v * kNB2 + k) * E + e;
            double y = __ldg(ua + i);
            if (k) y *= psi[v];
            if (comb) y = a_new * y + a_old * u0[i];
            out[i] = y;
        }
}

}  // namespace charm
