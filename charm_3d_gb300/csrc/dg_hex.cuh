// Kernels of the DG time step on general (trilinear) hexahedra: the leaves
// of a forest over an unstructured hexahedral mesh (gmsh), FP64, p1.
//
// The box kernels of dg_kernels.cuh evaluate the Taylor basis from
// constants; here every element and face carries its own geometry, computed
// once per mesh upload from the element corners by the reference's
// formulas (src/charm_geom.c):
//   element planes  double [kHexG][E]: centre, dh (the corner bounding
//                   box) and 1/dh, volume, the basis values phi_1..3 and the weights
//                   gw*gj at the 8 Gauss points of the trilinear map
//                   (_charm_quad_calc_gp, :40-172), the inverse of the full
//                   4x4 mass matrix (charm_geom_quad_calc, :496-530), the
//                   quadrature mean of phi_1..3, phi_1..3 at the 8 corners
//                   (the limiter's vertices) and the 6 outward face normals
//                   (_charm_face_calc_normal, :181-211, flipped away from
//                   the centre as the face callbacks do);
//   face planes     double [kHexF][F + Fb]: the normal from side 0's face
//                   (outward of side 0), the 6 triangle-rule points and
//                   their gw*gj (_charm_face_calc_gp_by_tri, :443-494) on
//                   the face that carries the points: side 0's, or the
//                   small side's of a mortar sub-face
//                   (src/models/ns/charm_model_ns_conv.c:174-331).
// The slot buffer, the element-owned gather and the limiter tables are
// those of the box path.
#pragma once

#include "dg_launch.h"

namespace charm {

// corners of each face, lower tangential axis first (p4est's face corners)
__device__ __forceinline__ int hex_face_corner(int f, int i)
{
    // {0,2,4,6} {1,3,5,7} {0,1,4,5} {2,3,6,7} {0,1,2,3} {4,5,6,7}
    const int d = f >> 1, up = f & 1;
    const int lo = (d == 0) ? 1 : 0, hi = (d == 2) ? 1 : 2;
    return (up << d) | ((i & 1) << lo) | (((i >> 1) & 1) << hi);
}

// Point of the trilinear map at reference coordinates r in [-1,1]^3 and
// the determinant of its Jacobian (the reference's weights (1 -+ r)/8 with
// x fastest, src/charm_geom.c:40-128).
__device__ __forceinline__ void hex_map(const double v[8][3], const double r[3], double x[3], double *det)
{
    double J[3][3];
#pragma unroll
    for (int d = 0; d < 3; d++) { x[d] = 0.0; J[d][0] = J[d][1] = J[d][2] = 0.0; }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const double sx = (k & 1) ? 1.0 : -1.0, sy = (k & 2) ? 1.0 : -1.0, sz = (k & 4) ? 1.0 : -1.0;
        const double wx = 1.0 + sx * r[0], wy = 1.0 + sy * r[1], wz = 1.0 + sz * r[2];
        const double w = wz * wy * wx * 0.125, dx = wz * wy * sx * 0.125, dy = wz * wx * sy * 0.125,
                     dz = wy * wx * sz * 0.125;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            x[d] += w * v[k][d];
            J[d][0] += dx * v[k][d];
            J[d][1] += dy * v[k][d];
            J[d][2] += dz * v[k][d];
        }
    }
    *det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

__device__ __forceinline__ void hex_load_vert(const HexDev &x, int64_t E, int64_t e, double v[8][3])
{
#pragma unroll
    for (int k = 0; k < 8; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) v[k][d] = __ldg(x.vert + (int64_t) (3 * k + d) * E + e);
}

// ---------------------------------------------------------------------------
// geometry of every element (once per upload); err bit kErrNegative for a
// non-positive Jacobian at a Gauss point
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) hex_geom_kernel(HexDev x, int64_t E, double *__restrict__ g, unsigned *err)
{
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double v[8][3];
    hex_load_vert(x, E, e, v);
    auto put = [&](int k, double val) { g[(int64_t) k * E + e] = val; };
    double c[3], dh[3];
    {
        const double r0[3] = {0.0, 0.0, 0.0};
        double dj;
        hex_map(v, r0, c, &dj);
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double lo = v[0][d], hi = v[0][d];
#pragma unroll
        for (int k = 1; k < 8; k++) { lo = fmin(lo, v[k][d]); hi = fmax(hi, v[k][d]); }
        dh[d] = hi - lo;
        put(kGc + d, c[d]);
        put(kGdh + d, dh[d]);
        put(kGidh + d, 1.0 / dh[d]);
    }
    const double s3 = 0.57735026918962576451;   // 1/sqrt(3)
    double phi[8][4], w[8], vol = 0.0;
#pragma unroll 1
    for (int q = 0; q < 8; q++) {
        const double r[3] = {(q & 1) ? s3 : -s3, (q & 2) ? s3 : -s3, (q & 4) ? s3 : -s3};
        double xq[3], dj;
        hex_map(v, r, xq, &dj);
        if (!(dj > 0.0)) set_error(err, kErrNegative);
        w[q] = dj;   // gw = 1
        vol += dj;
        phi[q][0] = 1.0;
#pragma unroll
        for (int d = 0; d < 3; d++) phi[q][1 + d] = (xq[d] - c[d]) / dh[d];
    }
    put(kGvol, vol);
    for (int q = 0; q < 8; q++) {
        put(kGw + q, w[q]);
        for (int d = 0; d < 3; d++) put(kGphi + 3 * q + d, phi[q][1 + d]);
    }
    // mass matrix and its inverse (Gauss-Jordan with partial pivoting)
    double a[4][4], ai[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0.0;
            for (int q = 0; q < 8; q++) s += w[q] * phi[q][i] * phi[q][j];
            a[i][j] = s;
            ai[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int i = 0; i < 4; i++) {
        int p = i;
        for (int r = i + 1; r < 4; r++)
            if (fabs(a[r][i]) > fabs(a[p][i])) p = r;
        if (p != i)
            for (int j = 0; j < 4; j++) {
                double t = a[i][j]; a[i][j] = a[p][j]; a[p][j] = t;
                t = ai[i][j]; ai[i][j] = ai[p][j]; ai[p][j] = t;
            }
        const double inv = 1.0 / a[i][i];
        for (int j = 0; j < 4; j++) { a[i][j] *= inv; ai[i][j] *= inv; }
        for (int r = 0; r < 4; r++) {
            if (r == i) continue;
            const double f = a[r][i];
            for (int j = 0; j < 4; j++) { a[r][j] -= f * a[i][j]; ai[r][j] -= f * ai[i][j]; }
        }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) put(kGminv + 4 * i + j, ai[i][j]);
    for (int d = 0; d < 3; d++) {
        double s = 0.0;
        for (int q = 0; q < 8; q++) s += phi[q][1 + d] * w[q];
        put(kGmean + d, s / vol);
    }
    for (int k = 0; k < 8; k++)
        for (int d = 0; d < 3; d++) put(kGvert + 3 * k + d, (v[k][d] - c[d]) / dh[d]);
    // face normals from the first three corners of each face, turned away
    // from the centre (the face centre is the mean of its corners)
    for (int f = 0; f < 6; f++) {
        const int k0 = hex_face_corner(f, 0), k1 = hex_face_corner(f, 1), k2 = hex_face_corner(f, 2),
                  k3 = hex_face_corner(f, 3);
        double a1[3], a2[3], n[3], l[3];
        for (int d = 0; d < 3; d++) {
            a1[d] = v[k1][d] - v[k0][d];
            a2[d] = v[k2][d] - v[k0][d];
            l[d] = 0.25 * (v[k0][d] + v[k1][d] + v[k2][d] + v[k3][d]) - c[d];
        }
        n[0] = a1[1] * a2[2] - a1[2] * a2[1];
        n[1] = a1[2] * a2[0] - a1[0] * a2[2];
        n[2] = a1[0] * a2[1] - a1[1] * a2[0];
        const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        double sg = 1.0 / nl;
        if (n[0] * l[0] + n[1] * l[1] + n[2] * l[2] < 0.0) sg = -sg;
        for (int d = 0; d < 3; d++) put(kGnrm + 3 * f + d, n[d] * sg);
    }
}

// ---------------------------------------------------------------------------
// geometry of every face record: interior records [0, F), boundary records
// [F, F + Fb)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) hex_face_geom_kernel(MeshDev m, HexDev x, double *__restrict__ fg)
{
    const int64_t r = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t F = m.n_face, NR = m.n_face + m.n_bface, E = m.n_elem;
    if (r >= NR) return;
    int64_t en, ep;   // element of the normal, element of the points
    int fn, fp;
    if (r < F) {
        const int kind = (m.face_info[r] >> 2) & 3;
        en = m.face_elem[r];
        fn = x.face_face[r];
        ep = (kind == 2) ? m.face_elem[F + r] : en;
        fp = (kind == 2) ? x.face_face[F + r] : fn;
    } else {
        en = ep = m.bface_elem[r - F];
        fn = fp = m.bface_face[r - F];
    }
    auto put = [&](int k, double val) { fg[(int64_t) k * NR + r] = val; };
    for (int d = 0; d < 3; d++) put(kFn + d, __ldg(x.g + (int64_t) (kGnrm + 3 * fn + d) * E + en));
    // the face's corners as the reference lists them, two triangles (v0, v1,
    // v2), (v1, v2, v3), 3 points each at (2/3, 1/6), (1/6, 2/3), (1/6, 1/6)
    double v[4][3];
    for (int i = 0; i < 4; i++) {
        const int k = hex_face_corner(fp, i);
        for (int d = 0; d < 3; d++) v[i][d] = __ldg(x.vert + (int64_t) (3 * k + d) * E + ep);
    }
    const double A = 2.0 / 3.0, B = 1.0 / 6.0;
    for (int t = 0; t < 2; t++) {
        double a1[3], a2[3], a3[3];
        for (int d = 0; d < 3; d++) {
            a1[d] = v[t][d] - v[t + 2][d];
            a2[d] = v[t + 1][d] - v[t + 2][d];
            a3[d] = v[t + 2][d];
        }
        const double EE = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
        const double FF = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
        const double GG = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
        const double gj = sqrt(EE * FF - GG * GG);
        for (int d = 0; d < 3; d++) {
            put(kFgp + 3 * (3 * t + 0) + d, A * a1[d] + B * a2[d] + a3[d]);
            put(kFgp + 3 * (3 * t + 1) + d, B * a1[d] + A * a2[d] + a3[d]);
            put(kFgp + 3 * (3 * t + 2) + d, B * a1[d] + B * a2[d] + a3[d]);
        }
        for (int j = 0; j < 3; j++) put(kFw + 3 * t + j, gj * (1.0 / 6.0));
    }
}

__device__ __forceinline__ double hex_g(const HexDev &x, int64_t E, int k, int64_t e)
{
    return __ldg(x.g + (int64_t) k * E + e);
}

// ---------------------------------------------------------------------------
// face kernel: flux at the 6 points of every record, projected on both
// sides' basis -> slots (side 1 with the opposite sign)
// ---------------------------------------------------------------------------
template <int NC, int FLUX>
__global__ void __launch_bounds__(128)
hex_face_kernel(MeshDev m, HexDev x, const double *__restrict__ u, double *__restrict__ slots, unsigned *err)
{
    constexpr int V = 4 + NC;
    const int64_t r = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t F = m.n_face, NR = m.n_face + m.n_bface, E = m.n_elem, S = m.n_slot;
    if (r >= NR) return;
    const bool inner = r < F;
    const int64_t e0 = inner ? m.face_elem[r] : m.bface_elem[r - F];
    const int64_t e1 = inner ? m.face_elem[F + r] : e0;
    const int ns = inner ? 2 : 1;
    double c0[3], c1[3], h0[3], h1[3];   // centres and 1/dh of both sides
    for (int d = 0; d < 3; d++) {
        c0[d] = hex_g(x, E, kGc + d, e0); h0[d] = hex_g(x, E, kGidh + d, e0);
        c1[d] = hex_g(x, E, kGc + d, e1); h1[d] = hex_g(x, E, kGidh + d, e1);
    }
    double a0[V][kNB], a1[V][kNB];
    load_coef<double, V>(u, E, e0, a0);
    if (inner) load_coef<double, V>(u, E, e1, a1);
    double n[3];
    for (int d = 0; d < 3; d++) n[d] = __ldg(x.fg + (int64_t) (kFn + d) * NR + r);
    // the flux frame of the face's normal, once for its 6 points
    double nt[3][3];
    normal_frame<double>(n, nt);
    const int bid = inner ? 0 : m.bface_bnd[r - F];
    double acc[2][V][kNB];
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) acc[s][v][k] = 0.0;
#pragma unroll 1
    for (int q = 0; q < 6; q++) {
        double gp[3];
        for (int d = 0; d < 3; d++) gp[d] = __ldg(x.fg + (int64_t) (kFgp + 3 * q + d) * NR + r);
        const double wq = __ldg(x.fg + (int64_t) (kFw + q) * NR + r);
        double p0[4], p1[4];
        p0[0] = p1[0] = 1.0;
        for (int d = 0; d < 3; d++) {
            p0[1 + d] = (gp[d] - c0[d]) * h0[d];
            p1[1 + d] = (gp[d] - c1[d]) * h1[d];
        }
        double U0[V], U1[V];
#pragma unroll
        for (int v = 0; v < V; v++) {
            U0[v] = a0[v][0] + p0[1] * a0[v][1] + p0[2] * a0[v][2] + p0[3] * a0[v][3];
            U1[v] = inner ? a1[v][0] + p1[1] * a1[v][1] + p1[2] * a1[v][2] + p1[3] * a1[v][3] : 0.0;
        }
        Prim<double, NC> q0, q1;
        cons_to_prim<double, NC>(U0, q0);
        if (inner) cons_to_prim<double, NC>(U1, q1);
        else bnd_cond<double, NC>(bid, q0, q1, n);
        double fl[V];
        num_flux<FLUX, double, NC, -1>(q0, q1, n, fl, err, nt);
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) {
                acc[0][v][k] += fl[v] * (p0[k] * wq);
                acc[1][v][k] += fl[v] * (p1[k] * wq);
            }
    }
    const int64_t slot = inner ? 2 * r : 2 * F + (r - F);
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t o = (int64_t) (v * kNB + k) * S + slot;
            if (ns == 2) store_pair<double>(slots, o, acc[0][v][k], -acc[1][v][k]);
            else slots[o] = acc[0][v][k];
        }
}

// ---------------------------------------------------------------------------
// cell kernel: volume integral, gather, full M^-1, update (+ SSP
// combination), or the residual (mode kCellResidual)
// ---------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(128)
hex_cell_kernel(MeshDev m, HexDev x, const double *__restrict__ u, const double *__restrict__ slots, const double *u0,
                double *out, double dt, const double *__restrict__ dt_dev, double a_new, double a_old, int mode,
                unsigned *err, unsigned long long *dt_next, double cfl)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double c[V][kNB];
    load_coef<double, V>(u, E, e, c);
    const double idh[3] = {hex_g(x, E, kGidh, e), hex_g(x, E, kGidh + 1, e), hex_g(x, E, kGidh + 2, e)};
    double R[V][kNB];
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int k = 0; k < kNB; k++) R[v][k] = 0.0;
    const bool grav = c_cfg.has_grav != 0;
    // volume integral (src/models/ns/charm_model_ns_conv.c:23-89): the
    // gradient of phi_k is e_k / dh_k
#pragma unroll 1
    for (int q = 0; q < 8; q++) {
        const double phi[4] = {1.0, hex_g(x, E, kGphi + 3 * q, e), hex_g(x, E, kGphi + 3 * q + 1, e),
                               hex_g(x, E, kGphi + 3 * q + 2, e)};
        const double w = hex_g(x, E, kGw + q, e);
        double U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + phi[1] * c[v][1] + phi[2] * c[v][2] + phi[3] * c[v][3];
        Prim<double, NC> p;
        cons_to_prim<double, NC>(U, p);
        if (!(p.r > 0.0) || !(p.p > 0.0)) set_error(err, isfinite(p.r) && isfinite(p.p) ? kErrNegative : kErrNonFinite);
        const double hp = U[3] + p.p;
        double F[V], G[V], H[V];
        F[0] = U[0] * p.u + p.p; F[1] = U[0] * p.v; F[2] = U[0] * p.w; F[3] = p.u * hp;
        G[0] = U[1] * p.u; G[1] = U[1] * p.v + p.p; G[2] = U[1] * p.w; G[3] = p.v * hp;
        H[0] = U[2] * p.u; H[1] = U[2] * p.v; H[2] = U[2] * p.w + p.p; H[3] = p.w * hp;
#pragma unroll
        for (int i = 0; i < NC; i++) { F[4 + i] = U[0] * p.c[i]; G[4 + i] = U[1] * p.c[i]; H[4 + i] = U[2] * p.c[i]; }
#pragma unroll
        for (int v = 0; v < V; v++) {
            R[v][1] -= F[v] * (idh[0] * w);
            R[v][2] -= G[v] * (idh[1] * w);
            R[v][3] -= H[v] * (idh[2] * w);
        }
        if (grav) {
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int k = 0; k < kNB; k++) R[a][k] -= p.r * c_cfg.grav[a] * (phi[k] * w);
        }
    }
    // element-owned gather of the face contributions
    const int32_t g0 = m.gather_ptr[e], g1 = m.gather_ptr[e + 1];
    const int64_t S = m.n_slot;
    for (int32_t j = g0; j < g1; j++) {
        const int64_t sl = m.gather_slot[j];
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) R[v][k] += slots[(int64_t) (v * kNB + k) * S + sl];
    }
    if (mode == kCellResidual) {
#pragma unroll
        for (int v = 0; v < V; v++)
#pragma unroll
            for (int k = 0; k < kNB; k++) out[(int64_t) (v * kNB + k) * E + e] = R[v][k];
        return;
    }
    // u -= dt * A^-1 int (src/models/ns/charm_model.c:68-99)
    double Ai[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) Ai[i][j] = hex_g(x, E, kGminv + 4 * i + j, e);
    const double step = dt_dev ? *dt_dev : dt;
    const bool comb = (a_old != 0.0);
    double cen[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const double rhs = Ai[k][0] * R[v][0] + Ai[k][1] * R[v][1] + Ai[k][2] * R[v][2] + Ai[k][3] * R[v][3];
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            double y = c[v][k] - step * rhs;
            if (comb) y = a_new * y + a_old * u0[idx];
            out[idx] = y;
            if (k == 0) cen[v] = y;
        }
    }
    if (dt_next) warp_min_to(cell_cfl_dt<NC>(cen, cfl, hex_g(x, E, kGvol, e)), dt_next);
}

// quadrature mean of the fields of element e (charm_get_fields_avg,
// src/charm_base_func.c:214-240): c_0 + sum_k c_k mean(phi_k)
template <int V>
__device__ __forceinline__ void hex_mean(const HexDev &x, int64_t E, int64_t e, const double *__restrict__ u, double *U)
{
    const double m1 = hex_g(x, E, kGmean, e), m2 = hex_g(x, E, kGmean + 1, e), m3 = hex_g(x, E, kGmean + 2, e);
#pragma unroll
    for (int v = 0; v < V; v++)
        U[v] = __ldg(u + (int64_t) (v * kNB) * E + e) + m1 * __ldg(u + (int64_t) (v * kNB + 1) * E + e) +
               m2 * __ldg(u + (int64_t) (v * kNB + 2) * E + e) + m3 * __ldg(u + (int64_t) (v * kNB + 3) * E + e);
}

// ---------------------------------------------------------------------------
// Barth-Jespersen limiter (src/limiters/charm_limiter_bj.c) + SSP
// combination on general hexahedra: bounds from the own quadrature mean and
// the six neighbour values (conforming: the neighbour's quadrature mean;
// boundary: BC ghost of the own mean; big side of a mortar: volume-weighted
// mean of the small leaves' centre values; small side: the big leaf's
// centre value), psi = min over the 8 corners
// ---------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(128)
hex_limit_kernel(MeshDev m, HexDev x, const double *__restrict__ ua, const double *u0, double *out, double a_new,
                 double a_old, unsigned long long *dt_next, double cfl)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double c[V][kNB];
    load_coef<double, V>(ua, E, e, c);
    double own[V], umin[V], umax[V];
    hex_mean<V>(x, E, e, ua, own);
#pragma unroll
    for (int v = 0; v < V; v++) umin[v] = umax[v] = own[v];
#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        const int kind = m.lim_kind[(int64_t) f * E + e] & 3;
        const int idx = m.lim_idx[(int64_t) f * E + e];
        double nbv[V];
        if (kind == 0) {
            hex_mean<V>(x, E, idx, ua, nbv);
        } else if (kind == 3) {
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = __ldg(ua + (int64_t) (v * kNB) * E + idx);
        } else if (kind == 2) {
            double svol = 0.0;
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] = 0.0;
            for (int k = 0; k < 4; k++) {
                const int64_t fi = idx + k;
                const unsigned info = m.face_info[fi];
                const int small = (((info >> 2) & 3) == 1) ? m.face_elem[fi] : m.face_elem[m.n_face + fi];
                const double vs = hex_g(x, E, kGvol, small);
                svol += vs;
#pragma unroll
                for (int v = 0; v < V; v++) nbv[v] += __ldg(ua + (int64_t) (v * kNB) * E + small) * vs;
            }
#pragma unroll
            for (int v = 0; v < V; v++) nbv[v] /= svol;
        } else {
            const int fb = m.bface_face[idx], bid = m.bface_bnd[idx];
            const double n[3] = {hex_g(x, E, kGnrm + 3 * fb, e), hex_g(x, E, kGnrm + 3 * fb + 1, e),
                                 hex_g(x, E, kGnrm + 3 * fb + 2, e)};
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
    for (int k = 0; k < 8; k++) {
        const double p1 = hex_g(x, E, kGvert + 3 * k, e), p2 = hex_g(x, E, kGvert + 3 * k + 1, e),
                     p3 = hex_g(x, E, kGvert + 3 * k + 2, e);
#pragma unroll
        for (int v = 0; v < V; v++) {
            const double f = c[v][0] + p1 * c[v][1] + p2 * c[v][2] + p3 * c[v][3];
            const double df = f - own[v];
            dmax[v] = fmax(dmax[v], df);
            dmin[v] = fmin(dmin[v], df);
        }
    }
#pragma unroll
    for (int v = 0; v < V; v++) psi[v] = bj_side_psi(dmax[v], dmin[v], umin[v] - own[v], umax[v] - own[v]);
    const bool comb = (a_old != 0.0);
    double cen[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
#pragma unroll
        for (int k = 0; k < kNB; k++) {
            const int64_t idx = (int64_t) (v * kNB + k) * E + e;
            double y = (k == 0) ? c[v][0] : c[v][k] * psi[v];
            if (comb) y = a_new * y + a_old * u0[idx];
            out[idx] = y;
            if (k == 0) cen[v] = y;
        }
    }
    if (dt_next) warp_min_to(cell_cfl_dt<NC>(cen, cfl, hex_g(x, E, kGvol, e)), dt_next);
}

// ---------------------------------------------------------------------------
// density-gradient estimate of charm_adapt on general hexahedra
// (src/charm_amr.c:350-573): grad_e = (1/vol_e) * the sum over e's face
// records of +-0.5 (r_L + r_R) n gw gj at the face points (side 0 adds,
// side 1 subtracts; a boundary's right state is its ghost).  Each element
// walks its own records through the gather table: deterministic, no atomics.
// ---------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(128)
hex_amr_grad_kernel(MeshDev m, HexDev x, const double *__restrict__ u, double *__restrict__ grad)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem, F = m.n_face, NR = m.n_face + m.n_bface;
    if (e >= E) return;
    double g[3] = {0.0, 0.0, 0.0};
    for (int32_t j = m.gather_ptr[e]; j < m.gather_ptr[e + 1]; j++) {
        const int64_t sl = m.gather_slot[j];
        const bool inner = sl < 2 * F;
        const int64_t r = inner ? (sl >> 1) : F + (sl - 2 * F);
        const double sg = (inner && (sl & 1)) ? -1.0 : 1.0;
        const int64_t e0 = inner ? m.face_elem[r] : e, e1 = inner ? m.face_elem[F + r] : e;
        double c0[3], c1[3], h0[3], h1[3], n[3];   // centres and 1/dh of both sides
        for (int d = 0; d < 3; d++) {
            c0[d] = hex_g(x, E, kGc + d, e0); h0[d] = hex_g(x, E, kGidh + d, e0);
            c1[d] = hex_g(x, E, kGc + d, e1); h1[d] = hex_g(x, E, kGidh + d, e1);
            n[d] = __ldg(x.fg + (int64_t) (kFn + d) * NR + r);
        }
        double a0[V][kNB], a1[V][kNB];
        load_coef<double, V>(u, E, e0, a0);
        load_coef<double, V>(u, E, e1, a1);
        const int bid = inner ? 0 : m.bface_bnd[r - F];
#pragma unroll 1
        for (int q = 0; q < 6; q++) {
            double p0[3], p1[3];
            for (int d = 0; d < 3; d++) {
                const double gp = __ldg(x.fg + (int64_t) (kFgp + 3 * q + d) * NR + r);
                p0[d] = (gp - c0[d]) * h0[d];
                p1[d] = (gp - c1[d]) * h1[d];
            }
            const double wq = __ldg(x.fg + (int64_t) (kFw + q) * NR + r);
            double U0[V], U1[V];
#pragma unroll
            for (int v = 0; v < V; v++) {
                U0[v] = a0[v][0] + p0[0] * a0[v][1] + p0[1] * a0[v][2] + p0[2] * a0[v][3];
                U1[v] = a1[v][0] + p1[0] * a1[v][1] + p1[1] * a1[v][2] + p1[2] * a1[v][3];
            }
            Prim<double, NC> q0, q1;
            cons_to_prim<double, NC>(U0, q0);
            if (inner) cons_to_prim<double, NC>(U1, q1);
            else bnd_cond<double, NC>(bid, q0, q1, n);
            const double qr = 0.5 * (q0.r + q1.r);
            for (int d = 0; d < 3; d++) g[d] += sg * (qr * wq * n[d]);
        }
    }
    const double vol = hex_g(x, E, kGvol, e);
    for (int d = 0; d < 3; d++) grad[(int64_t) d * E + e] = g[d] / vol;
}

// CFL step of the first step (the reference's get_dt, charm_model.c:21-36)
template <int NC>
__global__ void __launch_bounds__(128)
hex_cfl_kernel(MeshDev m, HexDev x, const double *__restrict__ u, unsigned long long *dt, double cfl)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem;
    if (e >= E) return;
    double U[V];
#pragma unroll
    for (int v = 0; v < V; v++) U[v] = __ldg(u + (int64_t) (v * kNB) * E + e);
    warp_min_to(cell_cfl_dt<NC>(U, cfl, hex_g(x, E, kGvol, e)), dt);
}

}  // namespace charm
