// Translation unit of the p2 kernels (dg_p2.cuh): launchers called by the
// host code in charm_gpu.cu, instantiated for the FP64 form (double) and the
// mixed form (float on the hi plane), 1 and 2 species.
#include <cuda_runtime.h>

#include "charm_gpu.h"
#include "dg_p2.cuh"

namespace charm {

cudaError_t p2_upload_cfg(const DevCfg *cfg, cudaStream_t st)
{
    return cudaMemcpyToSymbolAsync(c_cfg, cfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, st);
}

cudaError_t p2_upload_tables(const P2TabT<double> &t, const P2TabT<float> &tf)
{
    cudaError_t e = cudaMemcpyToSymbol(c_p2, &t, sizeof(t));
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_p2f, &tf, sizeof(tf));
}

template <typename T, int NC>
void p2_launch_face(int flux, const MeshDev &m, const T *u, T *slots, int64_t nbi, unsigned nb, unsigned *err,
                    cudaStream_t st)
{
    switch (flux) {
    case CHARM_GPU_FLUX_LF: p2_face_kernel<T, NC, CHARM_GPU_FLUX_LF><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    case CHARM_GPU_FLUX_HLLC: p2_face_kernel<T, NC, CHARM_GPU_FLUX_HLLC><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    case CHARM_GPU_FLUX_CD: p2_face_kernel<T, NC, CHARM_GPU_FLUX_CD><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    default: p2_face_kernel<T, NC, CHARM_GPU_FLUX_GODUNOV><<<nb, 128, 0, st>>>(m, u, slots, nbi, err); break;
    }
}

template <typename T, int NC>
void p2_launch_cell(const MeshDev &m, const T *u, const T *slots, const T *u0, T *out, const P2Upd &up,
                    unsigned *err, const T *radd, cudaStream_t st)
{
    const unsigned nb = (unsigned) ((m.n_elem + 127) / 128);
    p2_cell_kernel<T, NC><<<nb, 128, 0, st>>>(m, u, slots, u0, out, up, err, radd);
}

template <int NC>
void p2_launch_limit(const MeshDev &m, const double *ua, const double *u0, double *out, double a_new, double a_old,
                     cudaStream_t st)
{
    const unsigned nb = (unsigned) ((m.n_elem + 127) / 128);
    p2_limit_kernel<NC><<<nb, 128, 0, st>>>(m, ua, u0, out, a_new, a_old);
}
template void p2_launch_limit<1>(const MeshDev &, const double *, const double *, double *, double, double,
                                 cudaStream_t);
template void p2_launch_limit<2>(const MeshDev &, const double *, const double *, double *, double, double,
                                 cudaStream_t);

template <typename S, int NC>
void p2_launch_chem(const MeshDev &m, StIn<S> in, StOut<S> out, double *chem_rhs, cudaStream_t st)
{
    const unsigned nb = (unsigned) ((m.n_elem + 127) / 128);
    p2_chem_kernel<S, NC><<<nb, 128, 0, st>>>(m, in, out, chem_rhs);
}

template <typename T, int NC>
void p2_launch_visc(const MeshDev &m, bool diff, const T *u, const float *u_lo, T *dif, T *s9, T *vis,
                    const double *chem_rhs, T *radd, int64_t nbi, unsigned nbf, cudaStream_t st)
{
    const unsigned nbe = (unsigned) ((m.n_elem + 127) / 128);
    if (diff && NC >= 2) {
        if constexpr (sizeof(T) == sizeof(float))
            diffcoef_kernel<NC, kNB2, float, float><<<nbe, 128, 0, st>>>(m, StIn<float>{u, u_lo}, dif);
        else
            diffcoef_kernel<NC, kNB2, double, double><<<nbe, 128, 0, st>>>(m, StIn<double>{u}, dif);
    }
    if (nbf) p2_vgrad_face_kernel<T, NC><<<nbf, 128, 0, st>>>(m, u, dif, s9, nbi);
    p2_vgrad_cell_kernel<T, NC><<<nbe, 128, 0, st>>>(m, u, dif, s9, vis);
    p2_vvol_kernel<T, NC><<<nbe, 128, 0, st>>>(m, u, vis, chem_rhs, radd);
}

template <typename T, int NC>
void p2_launch_vflux(const MeshDev &m, const T *u, const T *vis, T *slots, int64_t nbi, unsigned nb, cudaStream_t st)
{
    p2_vflux_face_kernel<T, NC><<<nb, 128, 0, st>>>(m, u, vis, slots, nbi);
}

#define CHARM_P2_INST(T, NC)                                                                                   \
    template void p2_launch_face<T, NC>(int, const MeshDev &, const T *, T *, int64_t, unsigned, unsigned *,     \
                                        cudaStream_t);                                                        \
    template void p2_launch_cell<T, NC>(const MeshDev &, const T *, const T *, const T *, T *, const P2Upd &,    \
                                        unsigned *, const T *, cudaStream_t);                                 \
    template void p2_launch_chem<T, NC>(const MeshDev &, StIn<T>, StOut<T>, double *, cudaStream_t);           \
    template void p2_launch_visc<T, NC>(const MeshDev &, bool, const T *, const float *, T *, T *, T *,         \
                                        const double *, T *, int64_t, unsigned, cudaStream_t);                \
    template void p2_launch_vflux<T, NC>(const MeshDev &, const T *, const T *, T *, int64_t, unsigned,         \
                                         cudaStream_t);

CHARM_P2_INST(double, 1)
CHARM_P2_INST(double, 2)
CHARM_P2_INST(float, 1)
CHARM_P2_INST(float, 2)

}  // namespace charm
