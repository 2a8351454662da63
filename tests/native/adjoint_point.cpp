// Test-only host build of charm_3d_gb300/csrc/adjoint_math.h: exposes the
// pointwise vector-Jacobian products so that the derivative tests can
// compare them with central differences of the oracle's fluxes on the CPU.
#include "adjoint_math.h"

using namespace charm::adj;

namespace {
Gas gas_of(const double *g) { return Gas{g[0], g[1], g[2], g[3], g[4]}; }

// the axis-aligned specialisations when n = +-e_d exactly, else the general frame
int axis_of(const double *n)
{
    for (int d = 0; d < 3; d++)
        if ((n[d] == 1.0 || n[d] == -1.0) && n[(d + 1) % 3] == 0.0 && n[(d + 2) % 3] == 0.0) return d;
    return -1;
}

template <int NC>
void point(int flux, const double *g, const double *Ua, const double *Ub, const double *n, const double *qb,
           double *Uab, double *Ubb, double *q)
{
    switch (axis_of(n)) {
    case 0: point_vjp<NC, 0>(flux, Ua, Ub, n, gas_of(g), qb, Uab, Ubb, q); break;
    case 1: point_vjp<NC, 1>(flux, Ua, Ub, n, gas_of(g), qb, Uab, Ubb, q); break;
    case 2: point_vjp<NC, 2>(flux, Ua, Ub, n, gas_of(g), qb, Uab, Ubb, q); break;
    default: point_vjp<NC>(flux, Ua, Ub, n, gas_of(g), qb, Uab, Ubb, q); break;
    }
}
template <int NC>
void bpoint(int flux, int type, const double *par, const double *g, const double *U, const double *n,
            const double *qb, double *Uab, double *q)
{
    switch (axis_of(n)) {
    case 0: bpoint_vjp<NC, 0>(flux, type, par, U, n, gas_of(g), qb, Uab, q); break;
    case 1: bpoint_vjp<NC, 1>(flux, type, par, U, n, gas_of(g), qb, Uab, q); break;
    case 2: bpoint_vjp<NC, 2>(flux, type, par, U, n, gas_of(g), qb, Uab, q); break;
    default: bpoint_vjp<NC>(flux, type, par, U, n, gas_of(g), qb, Uab, q); break;
    }
}
template <int NC>
void vpoint(const double *g, const double *U, const double *a, double *Uab)
{
    double aa[3][4 + NC];
    for (int d = 0; d < 3; d++)
        for (int v = 0; v < 4 + NC; v++) aa[d][v] = a[d * (4 + NC) + v];
    vpoint_vjp<NC>(U, gas_of(g), aa, Uab);
}
}  // namespace

extern "C" {
// gas = {gam, 1/cv, m, R, eps}
int adj_point(int flux, int nc, const double *gas, const double *Ua, const double *Ub, const double *n,
              const double *qb, double *Uab, double *Ubb, double *q)
{
    if (nc == 1) point<1>(flux, gas, Ua, Ub, n, qb, Uab, Ubb, q);
    else if (nc == 2) point<2>(flux, gas, Ua, Ub, n, qb, Uab, Ubb, q);
    else return 1;
    return 0;
}
int adj_bpoint(int flux, int type, int nc, const double *par, const double *gas, const double *U, const double *n,
               const double *qb, double *Uab, double *q)
{
    if (nc == 1) bpoint<1>(flux, type, par, gas, U, n, qb, Uab, q);
    else if (nc == 2) bpoint<2>(flux, type, par, gas, U, n, qb, Uab, q);
    else return 1;
    return 0;
}
int adj_vpoint(int nc, const double *gas, const double *U, const double *a, double *Uab)
{
    if (nc == 1) vpoint<1>(gas, U, a, Uab);
    else if (nc == 2) vpoint<2>(gas, U, a, Uab);
    else return 1;
    return 0;
}
}
