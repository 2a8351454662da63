// Reverse-mode (vector-Jacobian) derivatives of the pointwise arithmetic of
// the DG residual, FP64: conserved -> primitive variables for an ideal gas
// with constant cp, the Euler volume flux, the LF / CD / HLLC numerical
// fluxes and the INLET / OUTLET / WALL_SLIP / WALL_NO_SLIP boundary states.
//
// Each *_vjp routine recomputes the forward quantities it needs from its
// inputs (the same operations, in the same order, as the forward path:
// charm_param_cons_to_prim src/charm_globals.c:183-208 with
// charm_mat_eos_ideal src/charm_eos.c:98-118; charm_calc_flux_lf
// src/charm_fluxes.c:255-315; charm_calc_flux_cd :513-559;
// charm_calc_flux_hllc :439-510 with _charm_calc_flux_hllc_x_1 :324-437;
// charm_bnd_cond src/charm_bnd_cond.c:21-146) and then accumulates the
// adjoint.  Branches (upwind side, star region, clamps, max) are taken as the
// forward evaluation takes them: the derivative is that of the active piece.
//
// Header-only and free of device intrinsics so that the same code is
// compiled into the GPU kernels (__host__ __device__) and, for unit tests of
// the derivatives, into a host library.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define ADJ_HD __host__ __device__ __forceinline__
#else
#define ADJ_HD inline
#endif

namespace charm {
namespace adj {

// 1 / sqrt(x) for x > 0: the device's reciprocal square root (one rounding
// step from the correctly rounded value), the plain quotient on the host.
// Where a routine needs both sqrt(x) and its reciprocal it takes
// x * rsqrt(x) and rsqrt(x), which saves a division per use.
ADJ_HD double rsq(double x)
{
#ifdef __CUDA_ARCH__
    return rsqrt(x);
#else
    return 1.0 / sqrt(x);
#endif
}

// 1 / x: on the device the hardware's approximate reciprocal refined by two
// Newton-Raphson steps y <- y + y (1 - x y) (within 1 ulp of IEEE 1/x for
// normal x; the forward flux path's reciprocal), the plain quotient on the
// host.
ADJ_HD double rcp(double x)
{
#ifdef __CUDA_ARCH__
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
#else
    return 1.0 / x;
#endif
}

// 1 / x with one Newton-Raphson step from the hardware seed: the relative
// error squares once (about 1e-13 and below), which the derivatives of the
// reverse sweep carry without loss at their 1e-6 bar; the plain quotient on
// the host.
ADJ_HD double rcp1(double x)
{
#ifdef __CUDA_ARCH__
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return fma(y, fma(-x, y, 1.0), y);
#else
    return 1.0 / x;
#endif
}

// 1 / sqrt(x), x > 0, with one Newton-Raphson step y <- y + y (1 - x y^2) / 2
// from the hardware seed (about 1e-6): within about 1.3e-12 relative, which
// the reverse sweep's derivatives carry without loss at their 1e-6 bar; the
// plain quotient on the host.
ADJ_HD double rsq1(double x)
{
#ifdef __CUDA_ARCH__
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-(x * y), y, 1.0);
    return fma(0.5 * y, e, y);
#else
    return 1.0 / sqrt(x);
#endif
}

// Ideal gas with constant cp (the only EOS the adjoint supports).
struct Gas {
    double gam;      // cp / cv
    double inv_cv;   // 1 / cv
    double m;        // molar mass
    double R;        // universal gas constant
    double eps;      // clamp of the reference's EOS switch (1e-12)
};

template <int NC>
struct Pr {                 // primitive state as the fluxes use it
    double r, u, v, w, e, e_tot, p, t, cz;
    double ir;              // 1 / r
    double icz;             // 1 / cz (set by prim; 0 where cz = 0)
    double c[NC];
    unsigned clamp;         // bit i: species fraction i was clamped to [0, 1]
};

template <int NC>
struct PrBar {              // adjoint of Pr
    double r, u, v, w, e, e_tot, p, t, cz;
    double c[NC];
};

template <int NC>
ADJ_HD void zero(PrBar<NC> &b)
{
    b.r = b.u = b.v = b.w = b.e = b.e_tot = b.p = b.t = b.cz = 0.0;
    for (int i = 0; i < NC; i++) b.c[i] = 0.0;
}

// Parts of the primitive state a caller uses besides r, velocities,
// energies, p and the fractions: the sound speed (fluxes) and the
// temperature (boundary states).  Leaving one out skips its arithmetic in
// prim and its (zero) adjoint in prim_vjp.
// kPrFast: 1 / r by rcp1 and 1 / cz by rsq1 (inside the flux and volume
// derivatives; the objective and the boundary states keep the full ones).
enum { kPrCz = 1, kPrT = 2, kPrAll = 3, kPrFast = 4 };

// U = (ru, rv, rw, re, rc_0 ..) -> primitive state (eos flag 4 of an ideal
// gas with constant cp).
template <int NC, int PARTS = kPrAll>
ADJ_HD void prim(const double *U, const Gas &g, Pr<NC> &p)
{
    double r = 0.0;
    for (int i = 0; i < NC; i++) r += U[4 + i];
    p.r = r;
    const double ir = (PARTS & kPrFast) ? rcp1(r) : rcp(r);
    p.ir = ir;
    p.u = U[0] * ir;
    p.v = U[1] * ir;
    p.w = U[2] * ir;
    p.e_tot = U[3] * ir;
    p.e = p.e_tot - 0.5 * (p.u * p.u + p.v * p.v + p.w * p.w);
    p.clamp = 0;
    for (int i = 0; i < NC; i++) {
#ifdef __CUDA_ARCH__
        // the forward path's clamp to [0, 1] on the bit pattern (integer
        // pipe; -0 counts as below 0 there too)
        long long b = __double_as_longlong(U[4 + i] * ir);
        const bool below = b < 0, above = b > 0x3FF0000000000000LL;
        if (below) b = 0;
        if (above) b = 0x3FF0000000000000LL;
        if (below || above) p.clamp |= 1u << i;
        p.c[i] = __longlong_as_double(b);
#else
        double c = U[4 + i] * ir;
        if (c < 0.0) { c = 0.0; p.clamp |= 1u << i; }
        if (c > 1.0) { c = 1.0; p.clamp |= 1u << i; }
        p.c[i] = c;
#endif
    }
    p.p = r * p.e * (g.gam - 1.0);
    p.icz = p.cz = p.t = 0.0;
    if (PARTS & kPrCz) {
        const double x = g.gam * p.p * ir;
        p.icz = (x > 0.0) ? ((PARTS & kPrFast) ? rsq1(x) : rsq(x)) : 0.0;
        // sqrt(x) from the reciprocal square root; x <= 0 (a state the
        // forward path reports) gives 0 or NaN like sqrt, without a second
        // square root
        p.cz = (x > 0.0) ? x * p.icz : ((x == 0.0) ? 0.0 : NAN);
    }
    if (PARTS & kPrT) p.t = p.e * g.inv_cv;
}

// Ub += (d prim / d U)^T b (b.cz, b.t taken as zero for the parts not in
// PARTS); ASSIGN: Ub = (d prim / d U)^T b, which saves the additions to a
// zeroed Ub (x + 0 is not x in IEEE arithmetic when x = -0, so they stay).
template <int NC, int PARTS = kPrAll, bool ASSIGN = false>
ADJ_HD void prim_vjp(const double *U, const Pr<NC> &p, const Gas &g, PrBar<NC> b, double *Ub)
{
    const double ir = p.ir;
    double b_ir = 0.0;
    if (PARTS & kPrT) b.e += b.t * g.inv_cv;                 // t = e / cv
    if ((PARTS & kPrCz) && p.cz > 0.0) {                     // cz = sqrt(gam p ir)
        const double d = 0.5 * g.gam * p.icz;
        b.p += b.cz * d * ir;
        b_ir += b.cz * d * p.p;
    }
    b.r += b.p * p.e * (g.gam - 1.0);                        // p = r e (gam - 1)
    b.e += b.p * p.r * (g.gam - 1.0);
    b.e_tot += b.e;                                          // e = e_tot - |v|^2/2
    b.u -= b.e * p.u;
    b.v -= b.e * p.v;
    b.w -= b.e * p.w;
    double bc[NC];                                           // c_i = rc_i / r
    for (int i = 0; i < NC; i++) {
        const bool free_c = !((p.clamp >> i) & 1u);
        bc[i] = free_c ? b.c[i] : 0.0;
        if (free_c) b_ir += b.c[i] * U[4 + i];
    }
    if (ASSIGN) {
        Ub[0] = b.u * ir;
        Ub[1] = b.v * ir;
        Ub[2] = b.w * ir;
        Ub[3] = b.e_tot * ir;
    } else {
        Ub[0] += b.u * ir;
        Ub[1] += b.v * ir;
        Ub[2] += b.w * ir;
        Ub[3] += b.e_tot * ir;
    }
    b_ir += b.u * U[0] + b.v * U[1] + b.w * U[2] + b.e_tot * U[3];
    b.r -= b_ir * ir * ir;                                   // ir = 1 / r
    for (int i = 0; i < NC; i++) {                           // r = sum rc_i
        if (ASSIGN) Ub[4 + i] = bc[i] * ir + b.r;
        else Ub[4 + i] += bc[i] * ir + b.r;
    }
}

// Euler volume fluxes F_d(U) (src/models/ns/charm_model_ns_conv.c:45-65):
// F_d[j] = U[d] vel_j + p delta_dj, F_d[3] = U[d] e_tot + p vel_d,
// F_d[4+i] = U[d] c_i.  Given a[d][.] = the adjoint of F_d, accumulate the
// adjoint of the primitive state into b and of U[0..2] into Ub.
template <int NC>
ADJ_HD void vflux_vjp(const double *U, const Pr<NC> &p, const double a[3][4 + NC], PrBar<NC> &b, double *Ub)
{
    const double vel[3] = {p.u, p.v, p.w};
    double vb[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 3; d++) {
        double m = 0.0;
        for (int j = 0; j < 3; j++) {
            m += a[d][j] * vel[j];
            vb[j] += a[d][j] * U[d];
        }
        m += a[d][3] * p.e_tot;
        for (int i = 0; i < NC; i++) {
            m += a[d][4 + i] * p.c[i];
            b.c[i] += a[d][4 + i] * U[d];
        }
        Ub[d] += m;
        b.p += a[d][d] + a[d][3] * vel[d];
        vb[d] += a[d][3] * p.p;
        b.e_tot += a[d][3] * U[d];
    }
    b.u += vb[0];
    b.v += vb[1];
    b.w += vb[2];
}

// Tangent frame of charm_calc_flux_hllc (src/charm_fluxes.c:458-488).
ADJ_HD void frame(const double n[3], double nt[3][3])
{
    nt[0][0] = n[0]; nt[0][1] = n[1]; nt[0][2] = n[2];
    double ri = sqrt(n[0] * n[0] + n[1] * n[1]);
    if (ri > 1.e-12) {
        nt[1][0] = -n[1] / ri; nt[1][1] = n[0] / ri; nt[1][2] = 0.0;
    } else {
        ri = sqrt(n[1] * n[1] + n[2] * n[2]);
        if (ri > 1.e-12) {
            nt[1][0] = 0.0; nt[1][1] = -n[2] / ri; nt[1][2] = n[1] / ri;
        } else {
            ri = sqrt(n[0] * n[0] + n[2] * n[2]);
            nt[1][0] = -n[2] / ri; nt[1][1] = 0.0; nt[1][2] = n[0] / ri;
        }
    }
    nt[2][0] = nt[0][1] * nt[1][2] - nt[0][2] * nt[1][1];
    nt[2][1] = -nt[0][0] * nt[1][2] + nt[0][2] * nt[1][0];
    nt[2][2] = nt[0][0] * nt[1][1] - nt[0][1] * nt[1][0];
}

// Frame of an axis-aligned normal n = s e_AX (AX >= 0): a signed
// permutation, applied without the products with its zero entries; AX < 0
// uses the general frame nt.  frame_in gives the components along the rows
// of the frame, frame_out sums rows weighted by (fu, fv, fw); each is the
// transpose of the other.
template <int AX>
ADJ_HD void frame_in(const double nt[3][3], double s, double x, double y, double z, double &un, double &u1,
                     double &u2)
{
    if (AX == 0) { un = s * x; u1 = s * y; u2 = z; }
    else if (AX == 1) { un = s * y; u1 = -s * x; u2 = z; }
    else if (AX == 2) { un = s * z; u1 = -s * y; u2 = x; }
    else {
        un = x * nt[0][0] + y * nt[0][1] + z * nt[0][2];
        u1 = x * nt[1][0] + y * nt[1][1] + z * nt[1][2];
        u2 = x * nt[2][0] + y * nt[2][1] + z * nt[2][2];
    }
}

template <int AX>
ADJ_HD void frame_out(const double nt[3][3], double s, double fu, double fv, double fw, double *q)
{
    if (AX == 0) { q[0] = s * fu; q[1] = s * fv; q[2] = fw; }
    else if (AX == 1) { q[1] = s * fu; q[0] = -s * fv; q[2] = fw; }
    else if (AX == 2) { q[2] = s * fu; q[1] = -s * fv; q[0] = fw; }
    else {
        q[0] = fu * nt[0][0] + fv * nt[1][0] + fw * nt[2][0];
        q[1] = fu * nt[0][1] + fv * nt[1][1] + fw * nt[2][1];
        q[2] = fu * nt[0][2] + fv * nt[1][2] + fw * nt[2][2];
    }
}

// v.n, without the zero products for an axis-aligned n
template <int AX>
ADJ_HD double vdotn(const double v[3], const double n[3])
{
    if (AX >= 0) return v[AX] * n[AX];
    return v[0] * n[0] + v[1] * n[1] + v[2] * n[2];
}

// LF (central = false) or CD (central = true) flux adjoint.  q (optional)
// receives the flux value.
template <int NC, int AX = -1>
ADJ_HD void flux_lf_vjp(const Pr<NC> &a, const Pr<NC> &b, const double n[3], bool central, const double *qb,
                        PrBar<NC> &ab, PrBar<NC> &bb, double *q)
{
    constexpr int V = 4 + NC;
    const double h = 0.5;
    const double va[3] = {a.u, a.v, a.w}, vbv[3] = {b.u, b.v, b.w};
    const double vna = vdotn<AX>(va, n);
    const double vnb = vdotn<AX>(vbv, n);
    // n_j, zero off the axis
    auto nj = [&](int j) { return (AX < 0 || j == AX) ? n[j] : 0.0; };
    const double A = fabs(vna) + a.cz, B = fabs(vnb) + b.cz;
    const double alpha = central ? 0.0 : fmax(A, B);
    if (q) {
        for (int j = 0; j < 3; j++)
            q[j] = h * ((b.r * vnb * vbv[j] + b.p * nj(j)) + (a.r * vna * va[j] + a.p * nj(j)) -
                        alpha * (b.r * vbv[j] - a.r * va[j]));
        q[3] = h * (((b.r * b.e_tot + b.p) * vnb) + ((a.r * a.e_tot + a.p) * vna) - alpha * (b.r * b.e_tot - a.r * a.e_tot));
        for (int i = 0; i < NC; i++)
            q[4 + i] = h * ((b.r * vnb * b.c[i]) + (a.r * vna * a.c[i]) - alpha * (b.r * b.c[i] - a.r * a.c[i]));
    }
    double alb = 0.0, vnab = 0.0, vnbb = 0.0;
    double vab[3] = {0.0, 0.0, 0.0}, vbb[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < 3; j++) {
        const double x = h * qb[j];
        alb -= x * (b.r * vbv[j] - a.r * va[j]);
        bb.r += x * (vnb * vbv[j] - alpha * vbv[j]);
        vnbb += x * b.r * vbv[j];
        vbb[j] += x * (b.r * vnb - alpha * b.r);
        if (AX < 0 || j == AX) { bb.p += x * n[j]; ab.p += x * n[j]; }
        ab.r += x * (vna * va[j] + alpha * va[j]);
        vnab += x * a.r * va[j];
        vab[j] += x * (a.r * vna + alpha * a.r);
    }
    {
        const double x = h * qb[3];
        alb -= x * (b.r * b.e_tot - a.r * a.e_tot);
        bb.r += x * (b.e_tot * vnb - alpha * b.e_tot);
        bb.e_tot += x * (b.r * vnb - alpha * b.r);
        bb.p += x * vnb;
        vnbb += x * (b.r * b.e_tot + b.p);
        ab.r += x * (a.e_tot * vna + alpha * a.e_tot);
        ab.e_tot += x * (a.r * vna + alpha * a.r);
        ab.p += x * vna;
        vnab += x * (a.r * a.e_tot + a.p);
    }
    for (int i = 0; i < NC; i++) {
        const double x = h * qb[4 + i];
        alb -= x * (b.r * b.c[i] - a.r * a.c[i]);
        bb.r += x * (vnb * b.c[i] - alpha * b.c[i]);
        vnbb += x * b.r * b.c[i];
        bb.c[i] += x * (b.r * vnb - alpha * b.r);
        ab.r += x * (vna * a.c[i] + alpha * a.c[i]);
        vnab += x * a.r * a.c[i];
        ab.c[i] += x * (a.r * vna + alpha * a.r);
    }
    if (!central) {                                  // alpha = max(A, B)
        if (A >= B) {
            vnab += alb * ((vna > 0.0) ? 1.0 : ((vna < 0.0) ? -1.0 : 0.0));
            ab.cz += alb;
        } else {
            vnbb += alb * ((vnb > 0.0) ? 1.0 : ((vnb < 0.0) ? -1.0 : 0.0));
            bb.cz += alb;
        }
    }
    if (AX >= 0) {
        vab[AX] += vnab * n[AX];
        vbb[AX] += vnbb * n[AX];
    } else {
        for (int j = 0; j < 3; j++) { vab[j] += vnab * n[j]; vbb[j] += vnbb * n[j]; }
    }
    ab.u += vab[0]; ab.v += vab[1]; ab.w += vab[2];
    bb.u += vbb[0]; bb.v += vbb[1]; bb.w += vbb[2];
    (void) V;
}

// HLLC flux adjoint (the PVRS wave speeds of src/charm_fluxes.c:340-372, the
// four upwind / star cases of :374-435, rotation back :505-509).
template <int NC, int AX = -1>
ADJ_HD void flux_hllc_vjp(const Pr<NC> &a, const Pr<NC> &b, const double n[3], const Gas &g, const double *qb,
                          PrBar<NC> &ab, PrBar<NC> &bb, double *q)
{
    double nt[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    double sn = 1.0;
    if (AX < 0) frame(n, nt);
    else sn = n[AX < 0 ? 0 : AX];
    double ua, va, wa, ub, vb, wb;
    frame_in<AX>(nt, sn, a.u, a.v, a.w, ua, va, wa);
    frame_in<AX>(nt, sn, b.u, b.v, b.w, ub, vb, wb);
    const double gam = g.gam;

    const double p_pvrs = 0.5 * (a.p + b.p) - 0.5 * (ub - ua) * 0.25 * (a.r + b.r) * (a.cz + b.cz);
    const double p_star = (p_pvrs > 0.0) ? p_pvrs : 0.0;
    const double kq = (gam + 1.0) / (2.0 * gam);   // loop-invariant: hoisted by the compiler
    const bool shock_a = !(p_star <= a.p), shock_b = !(p_star <= b.p);
    // c q of each side, q = sqrt(1 + kq (p*/p - 1)) on a shock side: as
    // sqrt(Q), Q = gam / r (p + kq (p* - p)) (one square root, no 1/p, as the
    // forward flux evaluates it); c where q = 1
    const double gia = gam * a.ir, gib = gam * b.ir;
    const double Qa = gia * (a.p + kq * (p_star - a.p)), Qb = gib * (b.p + kq * (p_star - b.p));
    const double iqa = shock_a ? rsq1(Qa) : 0.0, iqb = shock_b ? rsq1(Qb) : 0.0;
    const double cqa = shock_a ? Qa * iqa : a.cz, cqb = shock_b ? Qb * iqb : b.cz;
    const double sl0 = ua - cqa, sr0 = ub + cqb;
    const bool swap = sl0 > sr0;
    const double sl = swap ? sr0 : sl0, sr = swap ? sl0 : sr0;
    double num = b.p - a.p;
    num += a.r * ua * (sl - ua);
    num -= b.r * ub * (sr - ub);
    const double den = a.r * (sl - ua) - b.r * (sr - ub);
    const double iden = rcp1(den);
    double ss = num * iden;
    int clamp = 0;
    if (ss < sl) { ss = sl; clamp = 1; }
    if (ss > sr) { ss = sr; clamp = 2; }

    // the state k of the active case
    const bool sup_a = (sl >= 0.0), sup_b = !sup_a && (sr <= 0.0);
    const bool star = !sup_a && !sup_b;
    const bool ka = sup_a || (star && ss >= 0.0);
    const double rk = ka ? a.r : b.r, uk = ka ? ua : ub, vk = ka ? va : vb, wk = ka ? wa : wb;
    const double pk = ka ? a.p : b.p, ek = ka ? a.e_tot : b.e_tot, sk = ka ? sl : sr;
    const double *ck = ka ? a.c : b.c;

    if (q) {
        double fu, fv, fw;
        if (!star) {
            fu = rk * uk * uk + pk; fv = rk * vk * uk; fw = rk * wk * uk;
            q[3] = (rk * ek + pk) * uk;
            for (int i = 0; i < NC; i++) q[4 + i] = rk * uk * ck[i];
        } else {   // the factored star flux of the reverse below
            const double X = sk - uk, Y = ss - uk, G = rcp(sk - ss);
            const double rX = rk * X, mf = ss * (rX * G), P = pk + rX * Y;
            fu = mf * ss + P;
            fv = mf * vk;
            fw = mf * wk;
            q[3] = mf * (ek + Y * ss) + ss * (G * Y) * pk + P * ss;
            for (int i = 0; i < NC; i++) q[4 + i] = mf * ck[i];
        }
        frame_out<AX>(nt, sn, fu, fv, fw, q);
    }

    // ---- reverse ----
    double fub, fvb, fwb;
    frame_in<AX>(nt, sn, qb[0], qb[1], qb[2], fub, fvb, fwb);
    const double qeb = qb[3];
    double rkb = 0.0, ukb = 0.0, vkb = 0.0, wkb = 0.0, pkb = 0.0, ekb = 0.0, skb = 0.0, ssb = 0.0;
    double ckb[NC];
    for (int i = 0; i < NC; i++) ckb[i] = 0.0;
    if (!star) {
        rkb = fub * uk * uk + fvb * vk * uk + fwb * wk * uk + qeb * ek * uk;
        ukb = fub * 2.0 * rk * uk + fvb * rk * vk + fwb * rk * wk + qeb * (rk * ek + pk);
        vkb = fvb * rk * uk;
        wkb = fwb * rk * uk;
        pkb = fub + qeb * uk;
        ekb = qeb * rk * uk;
        for (int i = 0; i < NC; i++) {
            const double x = qb[4 + i];
            rkb += x * uk * ck[i];
            ukb += x * rk * ck[i];
            ckb[i] += x * rk * uk;
        }
    } else {
        // The star flux of :374-435, S_k (S_k U_k - F_k) / (S_k - S*) + S_k p*
        // D* / (S_k - S*), equals S* U*_k + p* D* for any S* (the clamped one
        // included), with U*_k = m (1, S*, v_k, w_k, c_k, E*), m = r_k X G:
        //   X = s_k - u_k, Y = s* - u_k, G = 1 / (s_k - s*), mf = s* m,
        //   P = p_k + r_k X Y,  fu = mf s* + P,  fv = mf v_k,  fw = mf w_k,
        //   fc_i = mf c_i,  qe = mf T + Z p_k + P s*,  T = e_k + Y s*,  Z = s* G Y
        // (e_k the specific total energy); the reverse of that form.
        const double X = sk - uk, Y = ss - uk, G = rcp1(sk - ss);
        const double rX = rk * X, m = rX * G, mf = ss * m, P = pk + rX * Y;
        const double T = ek + Y * ss, GY = G * Y, Z = ss * GY;
        double mfb = fub * ss + fvb * vk + fwb * wk + qeb * T;
        for (int i = 0; i < NC; i++) {
            mfb += qb[4 + i] * ck[i];
            ckb[i] += qb[4 + i] * mf;
        }
        vkb += fvb * mf;
        wkb += fwb * mf;
        const double Pb = fub + qeb * ss, Tb = qeb * mf, Zb = qeb * pk;
        pkb += Pb + qeb * Z;
        ekb += Tb;
        const double mb = mfb * ss;
        const double Yb = Tb * ss + Zb * ss * G + Pb * rX;
        const double Gb = Zb * ss * Y + mb * rX;
        const double W = Pb * Y + mb * G;            // X^ / r_k and r_k^ / X of P and m
        ssb += fub * mf + qeb * P + Tb * Y + Zb * GY + mfb * m + Gb * G * G + Yb;
        rkb += X * W;
        const double Xb = rk * W;
        skb += Xb - Gb * G * G;
        ukb -= Xb + Yb;
    }
    // wave speeds
    double slb = 0.0, srb = 0.0;
    if (ka) slb += skb; else srb += skb;
    double uab = 0.0, ubb = 0.0;
    if (clamp == 1) slb += ssb;
    else if (clamp == 2) srb += ssb;
    else {
        const double numb = ssb * iden, denb = -numb * ss;
        bb.p += numb; ab.p -= numb;
        ab.r += numb * ua * (sl - ua); uab += numb * a.r * (sl - 2.0 * ua); slb += numb * a.r * ua;
        bb.r -= numb * ub * (sr - ub); ubb -= numb * b.r * (sr - 2.0 * ub); srb -= numb * b.r * ub;
        ab.r += denb * (sl - ua); slb += denb * a.r; uab -= denb * a.r;
        bb.r -= denb * (sr - ub); srb -= denb * b.r; ubb += denb * b.r;
    }
    const double sl0b = swap ? srb : slb, sr0b = swap ? slb : srb;
    uab += sl0b;
    ubb += sr0b;
    double pstarb = 0.0;
    if (shock_a) {   // c q = sqrt(Q): Q^ = (c q)^ / (2 c q); Q = gam ir (p (1 - kq) + kq p*)
        const double Qab = -0.5 * sl0b * iqa;
        pstarb += Qab * gia * kq;
        ab.p += Qab * gia * (1.0 - kq);
        ab.r -= Qab * Qa * a.ir;                     // ir = 1 / r
    } else {
        ab.cz -= sl0b;
    }
    if (shock_b) {
        const double Qbb = 0.5 * sr0b * iqb;
        pstarb += Qbb * gib * kq;
        bb.p += Qbb * gib * (1.0 - kq);
        bb.r -= Qbb * Qb * b.ir;
    } else {
        bb.cz += sr0b;
    }
    if (p_pvrs > 0.0) {
        const double D = ub - ua, Rs = 0.25 * (a.r + b.r), Cs = a.cz + b.cz;
        ab.p += 0.5 * pstarb; bb.p += 0.5 * pstarb;
        const double Db = -0.5 * pstarb * Rs * Cs;
        ubb += Db; uab -= Db;
        const double Rsb = -0.5 * pstarb * D * Cs;
        ab.r += 0.25 * Rsb; bb.r += 0.25 * Rsb;
        const double Csb = -0.5 * pstarb * D * Rs;
        ab.cz += Csb; bb.cz += Csb;
    }
    // the active state's adjoint
    if (ka) {
        ab.r += rkb; uab += ukb; ab.p += pkb; ab.e_tot += ekb;
        for (int i = 0; i < NC; i++) ab.c[i] += ckb[i];
    } else {
        bb.r += rkb; ubb += ukb; bb.p += pkb; bb.e_tot += ekb;
        for (int i = 0; i < NC; i++) bb.c[i] += ckb[i];
    }
    const double vab = ka ? vkb : 0.0, wab = ka ? wkb : 0.0;
    const double vbbv = ka ? 0.0 : vkb, wbb = ka ? 0.0 : wkb;
    // rotated velocities
    double da[3], db[3];
    frame_out<AX>(nt, sn, uab, vab, wab, da);
    frame_out<AX>(nt, sn, ubb, vbbv, wbb, db);
    ab.u += da[0]; ab.v += da[1]; ab.w += da[2];
    bb.u += db[0]; bb.v += db[1]; bb.w += db[2];
}

// Boundary types (values of CHARM_GPU_BND_*).
enum { kBndInlet = 0, kBndOutlet = 1, kBndWallSlip = 2, kBndWallNoSlip = 3, kBndMassFlow = 4 };

// Ghost state of a boundary face (charm_bnd_cond, src/charm_bnd_cond.c:21-146)
// followed by eos flag 3 ((T, p) -> r, cz, e) and e_tot.  `pressure_clamped`
// records the p >= eps clamp of the EOS switch.
template <int NC>
ADJ_HD void bnd(int type, const double *par, const Pr<NC> &in, const double n[3], const Gas &g, Pr<NC> &out,
                bool &pressure_clamped)
{
    out = in;
    if (type == kBndInlet) {
        out.u = par[0]; out.v = par[1]; out.w = par[2];
        out.t = par[3]; out.p = par[4];
    } else if (type == kBndWallSlip) {
        const double svn = in.u * n[0] + in.v * n[1] + in.w * n[2];
        const double vv0 = n[0] * svn, vv1 = n[1] * svn, vv2 = n[2] * svn;
        out.u = (in.u - vv0) - vv0;
        out.v = (in.v - vv1) - vv1;
        out.w = (in.w - vv2) - vv2;
    } else if (type == kBndWallNoSlip) {
        const double svn = in.u * n[0] + in.v * n[1] + in.w * n[2];
        out.u = in.u - n[0] * svn;
        out.v = in.v - n[1] * svn;
        out.w = in.w - n[2] * svn;
        out.t = par[0];
    }
    pressure_clamped = out.p < g.eps;
    if (pressure_clamped) out.p = g.eps;
    out.r = out.p * g.m / (out.t * g.R);
    out.ir = 1.0 / out.r;   // the HLLC wave speeds use 1 / r of each side
    out.cz = sqrt(g.gam * out.p / out.r);
    out.e = out.p / (out.r * (g.gam - 1.0));
    out.e_tot = out.e + 0.5 * (out.u * out.u + out.v * out.v + out.w * out.w);
}

// inb += (d out / d in)^T outb for the ghost state of bnd().
template <int NC>
ADJ_HD void bnd_vjp(int type, const Pr<NC> &out, bool pressure_clamped, const double n[3], const Gas &g,
                    PrBar<NC> ob, PrBar<NC> &inb)
{
    // e_tot = e + |v|^2 / 2
    ob.e += ob.e_tot;
    ob.u += ob.e_tot * out.u; ob.v += ob.e_tot * out.v; ob.w += ob.e_tot * out.w;
    // e = p / (r (gam - 1))
    ob.p += ob.e / (out.r * (g.gam - 1.0));
    ob.r -= ob.e * out.e / out.r;
    // cz = sqrt(gam p / r)
    if (out.cz > 0.0) {
        ob.p += ob.cz * out.cz / (2.0 * out.p);
        ob.r -= ob.cz * out.cz / (2.0 * out.r);
    }
    // r = p m / (t R)
    ob.p += ob.r * out.r / out.p;
    ob.t -= ob.r * out.r / out.t;
    if (pressure_clamped) ob.p = 0.0;
    for (int i = 0; i < NC; i++) inb.c[i] += ob.c[i];
    if (type == kBndInlet) return;
    inb.p += ob.p;
    if (type != kBndWallNoSlip) inb.t += ob.t;
    if (type == kBndWallSlip) {
        const double s = ob.u * n[0] + ob.v * n[1] + ob.w * n[2];
        inb.u += ob.u - 2.0 * n[0] * s; inb.v += ob.v - 2.0 * n[1] * s; inb.w += ob.w - 2.0 * n[2] * s;
    } else if (type == kBndWallNoSlip) {
        const double s = ob.u * n[0] + ob.v * n[1] + ob.w * n[2];
        inb.u += ob.u - n[0] * s; inb.v += ob.v - n[1] * s; inb.w += ob.w - n[2] * s;
    } else {
        inb.u += ob.u; inb.v += ob.v; inb.w += ob.w;
    }
}

// Flux selector values (CHARM_GPU_FLUX_*).
enum { kFluxLF = 0, kFluxGodunov = 1, kFluxHLLC = 2, kFluxCD = 3 };

// AX >= 0: n = s e_AX (axis-aligned faces), the frame products with zeros
// left out; AX < 0: any unit normal.
template <int NC, int AX = -1>
ADJ_HD void num_flux_vjp(int flux, const Pr<NC> &a, const Pr<NC> &b, const double n[3], const Gas &g,
                         const double *qb, PrBar<NC> &ab, PrBar<NC> &bb, double *q)
{
    if (flux == kFluxHLLC) flux_hllc_vjp<NC, AX>(a, b, n, g, qb, ab, bb, q);
    else flux_lf_vjp<NC, AX>(a, b, n, flux == kFluxCD, qb, ab, bb, q);
}

// Interior point: (Ua, Ub) -> q; Uab/Ubb = (dq/dU)^T qb.
template <int NC, int AX = -1>
ADJ_HD void point_vjp(int flux, const double *Ua, const double *Ub, const double n[3], const Gas &g,
                      const double *qb, double *Uab, double *Ubb, double *q)
{
    Pr<NC> a, b;
    prim<NC, kPrCz | kPrFast>(Ua, g, a);
    prim<NC, kPrCz | kPrFast>(Ub, g, b);
    PrBar<NC> ab, bb;
    zero<NC>(ab);
    zero<NC>(bb);
    num_flux_vjp<NC, AX>(flux, a, b, n, g, qb, ab, bb, q);
    prim_vjp<NC, kPrCz, true>(Ua, a, g, ab, Uab);
    prim_vjp<NC, kPrCz, true>(Ub, b, g, bb, Ubb);
}

// Boundary point: U -> q(U, ghost(U)); Uab = (dq/dU)^T qb.
template <int NC, int AX = -1>
ADJ_HD void bpoint_vjp(int flux, int type, const double *par, const double *U, const double n[3], const Gas &g,
                       const double *qb, double *Uab, double *q)
{
    Pr<NC> a, o;
    prim<NC>(U, g, a);
    bool pc;
    bnd<NC>(type, par, a, n, g, o, pc);
    PrBar<NC> ab, ob;
    zero<NC>(ab);
    zero<NC>(ob);
    num_flux_vjp<NC, AX>(flux, a, o, n, g, qb, ab, ob, q);
    bnd_vjp<NC>(type, o, pc, n, g, ob, ab);
    prim_vjp<NC, kPrAll, true>(U, a, g, ab, Uab);
}

// Volume point: U -> F_d(U), d = 0..2; Uab += sum_d (dF_d/dU)^T a[d].
template <int NC>
ADJ_HD void vpoint_vjp(const double *U, const Gas &g, const double a[3][4 + NC], double *Uab)
{
    Pr<NC> p;
    prim<NC, kPrFast>(U, g, p);
    PrBar<NC> b;
    zero<NC>(b);
    vflux_vjp<NC>(U, p, a, b, Uab);
    prim_vjp<NC, 0>(U, p, g, b, Uab);
}

}  // namespace adj
}  // namespace charm
