// Translation unit of the general-hexahedron kernels (dg_hex.cuh): FP64, p1,
// the convective terms of the Euler and NS models.  Holds its own copy of the
// configuration constants, uploaded by hex_upload_cfg whenever charm_gpu.cu
// uploads its own.
#include <cuda_runtime.h>

#include "charm_gpu.h"
#include "dg_hex.cuh"
#include "dg_launch.h"

namespace charm {

cudaError_t hex_upload_cfg(const DevCfg *cfg, cudaStream_t st)
{
    return cudaMemcpyToSymbolAsync(c_cfg, cfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, st);
}

static unsigned blocks(int64_t n) { return (unsigned) ((n + 127) / 128); }

cudaError_t hex_launch_geom(const MeshDev &m, const HexDev &x, double *g, double *fg, unsigned *err, cudaStream_t st)
{
    hex_geom_kernel<<<blocks(m.n_elem), 128, 0, st>>>(x, m.n_elem, g, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    HexDev xg = x;
    xg.g = g;
    if (m.n_face + m.n_bface > 0) hex_face_geom_kernel<<<blocks(m.n_face + m.n_bface), 128, 0, st>>>(m, xg, fg);
    return cudaGetLastError();
}

template <int NC>
void hex_launch_face(int flux, const MeshDev &m, const HexDev &x, const double *u, double *slots, unsigned *err,
                     cudaStream_t st)
{
    const int64_t n = m.n_face + m.n_bface;
    if (n == 0) return;
    switch (flux) {
    case CHARM_GPU_FLUX_LF: hex_face_kernel<NC, CHARM_GPU_FLUX_LF><<<blocks(n), 128, 0, st>>>(m, x, u, slots, err); break;
    case CHARM_GPU_FLUX_HLLC: hex_face_kernel<NC, CHARM_GPU_FLUX_HLLC><<<blocks(n), 128, 0, st>>>(m, x, u, slots, err); break;
    case CHARM_GPU_FLUX_CD: hex_face_kernel<NC, CHARM_GPU_FLUX_CD><<<blocks(n), 128, 0, st>>>(m, x, u, slots, err); break;
    default: hex_face_kernel<NC, CHARM_GPU_FLUX_GODUNOV><<<blocks(n), 128, 0, st>>>(m, x, u, slots, err); break;
    }
}

template <int NC>
void hex_launch_cell(const MeshDev &m, const HexDev &x, const double *u, const double *slots, const double *u0,
                     double *out, double dt, const double *dt_dev, double a_new, double a_old, int mode, unsigned *err,
                     unsigned long long *dt_next, double cfl, cudaStream_t st)
{
    hex_cell_kernel<NC><<<blocks(m.n_elem), 128, 0, st>>>(m, x, u, slots, u0, out, dt, dt_dev, a_new, a_old, mode, err,
                                                         dt_next, cfl);
}

template <int NC>
void hex_launch_limit(const MeshDev &m, const HexDev &x, const double *ua, const double *u0, double *out, double a_new,
                      double a_old, unsigned long long *dt_next, double cfl, cudaStream_t st)
{
    hex_limit_kernel<NC><<<blocks(m.n_elem), 128, 0, st>>>(m, x, ua, u0, out, a_new, a_old, dt_next, cfl);
}

template <int NC>
void hex_launch_cfl(const MeshDev &m, const HexDev &x, const double *u, unsigned long long *dt, double cfl,
                    cudaStream_t st)
{
    hex_cfl_kernel<NC><<<blocks(m.n_elem), 128, 0, st>>>(m, x, u, dt, cfl);
}

template <int NC>
void hex_launch_amr_grad(const MeshDev &m, const HexDev &x, const double *u, double *grad, cudaStream_t st)
{
    hex_amr_grad_kernel<NC><<<blocks(m.n_elem), 128, 0, st>>>(m, x, u, grad);
}

#define CHARM_HEX_INST(NC)                                                                                              \
    template void hex_launch_face<NC>(int, const MeshDev &, const HexDev &, const double *, double *, unsigned *,       \
                                      cudaStream_t);                                                                    \
    template void hex_launch_cell<NC>(const MeshDev &, const HexDev &, const double *, const double *, const double *, \
                                      double *, double, const double *, double, double, int, unsigned *,                \
                                      unsigned long long *, double, cudaStream_t);                                      \
    template void hex_launch_limit<NC>(const MeshDev &, const HexDev &, const double *, const double *, double *,      \
                                       double, double, unsigned long long *, double, cudaStream_t);                     \
    template void hex_launch_cfl<NC>(const MeshDev &, const HexDev &, const double *, unsigned long long *, double,    \
                                     cudaStream_t);                                                                     \
    template void hex_launch_amr_grad<NC>(const MeshDev &, const HexDev &, const double *, double *, cudaStream_t);
CHARM_HEX_INST(1)
CHARM_HEX_INST(2)

}  // namespace charm
