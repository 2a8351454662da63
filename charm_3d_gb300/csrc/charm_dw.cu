// Translation unit of the double-word form's kernels (CHARM_GPU_PREC_DW):
// face_kernel and cell_kernel of dg_kernels.cuh instantiated for the dw
// type (dw.cuh), so that their compilation runs beside the other units'.
// Holds its own copy of the configuration constants, uploaded by
// dw_upload_cfg whenever charm_gpu.cu uploads its own.
#include <cuda_runtime.h>

#include "charm_gpu.h"
#include "dg_launch.h"

namespace charm {

cudaError_t dw_upload_cfg(const DevCfg *cfg, cudaStream_t st)
{
    return cudaMemcpyToSymbolAsync(c_cfg, cfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, st);
}

template <int NC>
void dw_launch_face(int flux, const MeshDev &m, const double *u, dw *slots, int64_t nbi, unsigned nb, unsigned *err,
                    cudaStream_t st)
{
    switch (flux) {
    case CHARM_GPU_FLUX_LF: face_kernel<dw, NC, CHARM_GPU_FLUX_LF><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    case CHARM_GPU_FLUX_CD: face_kernel<dw, NC, CHARM_GPU_FLUX_CD><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    default: face_kernel<dw, NC, CHARM_GPU_FLUX_HLLC><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    }
}

template <int NC>
void dw_launch_cell(const MeshDev &m, const double *u, const dw *slots, const double *u0, double *out, double dt,
                    const double *dt_dev, double a_new, double a_old, int mode, unsigned *err, const double *radd,
                    unsigned long long *dt_next, double cfl, cudaStream_t st)
{
    const unsigned nb = (unsigned) ((m.n_elem + 127) / 128);
    cell_kernel<dw, NC><<<nb, 128, 0, st>>>(m, u, slots, u0, out, dt, dt_dev, a_new, a_old, mode, err, radd, dt_next,
                                            cfl);
}

template void dw_launch_face<1>(int, const MeshDev &, const double *, dw *, int64_t, unsigned, unsigned *, cudaStream_t);
template void dw_launch_face<2>(int, const MeshDev &, const double *, dw *, int64_t, unsigned, unsigned *, cudaStream_t);
template void dw_launch_cell<1>(const MeshDev &, const double *, const dw *, const double *, double *, double,
                                const double *, double, double, int, unsigned *, const double *, unsigned long long *,
                                double, cudaStream_t);
template void dw_launch_cell<2>(const MeshDev &, const double *, const dw *, const double *, double *, double,
                                const double *, double, double, int, unsigned *, const double *, unsigned long long *,
                                double, cudaStream_t);

}  // namespace charm
