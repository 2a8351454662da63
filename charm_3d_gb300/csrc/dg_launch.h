// Launchers of the kernel families compiled in their own translation units
// (several units compile in parallel; the host code in charm_gpu.cu calls
// these).  Each unit holds its own constant-memory configuration, uploaded
// by its *_upload_cfg.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "dg_kernels.cuh"
#include "dg_visc.cuh"

namespace charm {

// ---- p2 basis (charm_p2.cu) ------------------------------------------------

constexpr int kNB2 = 10;

// Rule tables and the inverse mass matrix of the reference box.
template <typename T>
struct P2TabT {
    T cxi[27][3];        // cell points in reference coordinates, [-1/2, 1/2]^3, x fastest
    T cw[27];            // cell weights, sum 1
    T fxi[9][2];         // face points (lower, upper tangential axis), [-1/2, 1/2]^2
    T fw[9];             // face weights, sum 1
    T minv[kNB2][kNB2];  // inverse mass matrix of the reference box (volume 1)
    T mean[kNB2];        // cell mean of each basis function
};

// Update arguments of the p2 cell kernel.  FP64 form: out = a_new*(u -
// dt*M^-1*(R + radd)) + a_old*u0 with the doubles.  Mixed form: the state
// pointers are the hi planes, the lo planes and the float-float splits of
// dt, a_new and a_old come here, and u0 == nullptr means no combination.
struct P2Upd {
    double dt, a_new, a_old;
    const double *dt_dev;
    int mode;   // kCellUpdate, or kCellResidual: out = R + radd
    const float *u_lo, *u0_lo;
    float *out_lo;
    float dt_h, dt_l, a_h, a_l, b_h, b_l;
};

cudaError_t p2_upload_cfg(const DevCfg *cfg, cudaStream_t st);
cudaError_t p2_upload_tables(const P2TabT<double> &t, const P2TabT<float> &tf);

// T = double (FP64 form) or float (mixed form; u is the hi plane).  nbi:
// blocks of 128 over the interior faces, nb: all blocks (interior, boundary).
template <typename T, int NC>
void p2_launch_face(int flux, const MeshDev &m, const T *u, T *slots, int64_t nbi, unsigned nb, unsigned *err,
                    cudaStream_t st);
template <typename T, int NC>
void p2_launch_cell(const MeshDev &m, const T *u, const T *slots, const T *u0, T *out, const P2Upd &up,
                    unsigned *err, const T *radd, cudaStream_t st);
template <typename S, int NC>
void p2_launch_chem(const MeshDev &m, StIn<S> in, StOut<S> out, double *chem_rhs, cudaStream_t st);
// Barth-Jespersen limiter on the p2 basis + SSP combination (FP64)
template <int NC>
void p2_launch_limit(const MeshDev &m, const double *ua, const double *u0, double *out, double a_new, double a_old,
                     cudaStream_t st);
// diffusion coefficients (FP64 from the state; u_lo: the lo plane of the
// mixed form), lifting and the viscous volume terms
template <typename T, int NC>
void p2_launch_visc(const MeshDev &m, bool diff, const T *u, const float *u_lo, T *dif, T *s9, T *vis,
                    const double *chem_rhs, T *radd, int64_t nbi, unsigned nbf, cudaStream_t st);
template <typename T, int NC>
void p2_launch_vflux(const MeshDev &m, const T *u, const T *vis, T *slots, int64_t nbi, unsigned nb,
                     cudaStream_t st);

// ---- double-word form (charm_dw.cu) ------------------------------------------

cudaError_t dw_upload_cfg(const DevCfg *cfg, cudaStream_t st);
// face_kernel<dw> (flux LF, CD or HLLC) and cell_kernel<dw>, arguments as theirs
template <int NC>
void dw_launch_face(int flux, const MeshDev &m, const double *u, dw *slots, int64_t nbi, unsigned nb, unsigned *err,
                    cudaStream_t st);
template <int NC>
void dw_launch_cell(const MeshDev &m, const double *u, const dw *slots, const double *u0, double *out, double dt,
                    const double *dt_dev, double a_new, double a_old, int mode, unsigned *err, const double *radd,
                    unsigned long long *dt_next, double cfl, cudaStream_t st);

// ---- general hexahedra (charm_hex.cu) -----------------------------------------

// element geometry planes [kHexG][E] and face geometry planes [kHexF][F + Fb]
// (dg_hex.cuh describes them)
enum {
    kGc = 0,        // centre x, y, z
    kGdh = 3,       // dh x, y, z
    kGvol = 6,      // volume (sum of gw*gj)
    kGphi = 7,      // phi_1..3 at cell point q: kGphi + 3 q + (k - 1)
    kGw = 31,       // gw*gj at cell point q
    kGminv = 39,    // inverse mass matrix, row-major 4x4
    kGmean = 55,    // quadrature mean of phi_1..3 (over the volume)
    kGvert = 58,    // phi_1..3 at corner k: kGvert + 3 k + (k' - 1)
    kGnrm = 82,     // outward unit normal of face f: kGnrm + 3 f + d
    kGidh = 100,    // 1 / dh x, y, z
    kHexG = 103
};
enum { kFn = 0, kFgp = 3, kFw = 21, kHexF = 27 };

struct HexDev {
    const double *g;          // [kHexG][E]
    const double *fg;         // [kHexF][F + Fb]
    const int8_t *face_face;  // [2][F]
    const double *vert;       // [24][E]: corner k coordinate d at (3 k + d)
};

cudaError_t hex_upload_cfg(const DevCfg *cfg, cudaStream_t st);
// element and face geometry tables of dg_hex.cuh from the corners (x.vert)
// and face numbers (x.face_face); err: kErrNegative for a non-positive Jacobian
cudaError_t hex_launch_geom(const MeshDev &m, const HexDev &x, double *g, double *fg, unsigned *err, cudaStream_t st);
template <int NC>
void hex_launch_face(int flux, const MeshDev &m, const HexDev &x, const double *u, double *slots, unsigned *err,
                     cudaStream_t st);
template <int NC>
void hex_launch_cell(const MeshDev &m, const HexDev &x, const double *u, const double *slots, const double *u0,
                     double *out, double dt, const double *dt_dev, double a_new, double a_old, int mode, unsigned *err,
                     unsigned long long *dt_next, double cfl, cudaStream_t st);
template <int NC>
void hex_launch_limit(const MeshDev &m, const HexDev &x, const double *ua, const double *u0, double *out, double a_new,
                      double a_old, unsigned long long *dt_next, double cfl, cudaStream_t st);
template <int NC>
void hex_launch_cfl(const MeshDev &m, const HexDev &x, const double *u, unsigned long long *dt, double cfl,
                    cudaStream_t st);
// density-gradient estimate of the refine criterion, grad [3][E]
template <int NC>
void hex_launch_amr_grad(const MeshDev &m, const HexDev &x, const double *u, double *grad, cudaStream_t st);

// ---- point fluxes (charm_point.cu) ------------------------------------------

// Upload cfg to the unit's constants, then q[i] = flux between the state
// pair U2[i] along nrm[i] (n pairs; T = double, float for `mixed`, dw for
// `dword`).
cudaError_t point_launch_flux(const DevCfg *cfg, int flux, int n_comp, bool mixed, bool dword, int64_t n,
                              const double *U2, const double *nrm, double *q, unsigned *err, cudaStream_t st);

// out[i] = rcp_nr(b[i]) (which 0) or qdiv(a[i], b[i]) (which 1), device arrays.
cudaError_t point_launch_math(int which, int64_t n, const double *a, const double *b, double *out, cudaStream_t st);

}  // namespace charm
