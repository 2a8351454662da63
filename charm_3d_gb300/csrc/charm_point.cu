// Translation unit of the point-flux kernels (charm_gpu_point_flux): the
// face kernels' cons_to_prim and numerical fluxes evaluated on given state
// pairs, for the verification of the flux functions against the reference's
// own (src/charm_fluxes.c).  It holds its own copy of the configuration
// constants (c_cfg), uploaded by point_launch_flux before each launch.
#include <cuda_runtime.h>

#include "charm_gpu.h"
#include "dg_launch.h"

namespace charm {

// One thread per state pair: the face kernels' cons_to_prim and num_flux.
template <typename T, int NC, int FLUX>
__global__ void __launch_bounds__(128)
point_flux_kernel(int64_t n, const double *__restrict__ U2, const double *__restrict__ nrm, double *__restrict__ q,
                  unsigned *err)
{
    constexpr int V = 4 + NC;
    const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T Ua[V], Ub[V], out[V];
#pragma unroll
    for (int v = 0; v < V; v++) {
        Ua[v] = T(U2[(2 * i) * V + v]);
        Ub[v] = T(U2[(2 * i + 1) * V + v]);
    }
    Prim<T, NC> pa, pb;
    cons_to_prim<T, NC>(Ua, pa);
    cons_to_prim<T, NC>(Ub, pb);
    const T nv[3] = {T(nrm[3 * i]), T(nrm[3 * i + 1]), T(nrm[3 * i + 2])};
    int ax = -1;
    for (int d = 0; d < 3; d++)
        if ((nv[d] == T(1) || nv[d] == T(-1)) && nv[(d + 1) % 3] == T(0) && nv[(d + 2) % 3] == T(0)) ax = d;
    switch (ax) {
    case 0: num_flux<FLUX, T, NC, 0>(pa, pb, nv, out, err); break;
    case 1: num_flux<FLUX, T, NC, 1>(pa, pb, nv, out, err); break;
    case 2: num_flux<FLUX, T, NC, 2>(pa, pb, nv, out, err); break;
    default: num_flux<FLUX, T, NC, -1>(pa, pb, nv, out, err); break;
    }
#pragma unroll
    for (int v = 0; v < V; v++) q[i * V + v] = (double) out[v];
}

template <typename T, int NC>
void launch_point_flux(int flux, int64_t n, const double *U2, const double *nrm, double *q, unsigned *err,
                       cudaStream_t st)
{
    const int bs = 128;
    const unsigned g = (unsigned) ((n + bs - 1) / bs);
    switch (flux) {
    case CHARM_GPU_FLUX_LF: point_flux_kernel<T, NC, CHARM_GPU_FLUX_LF><<<g, bs, 0, st>>>(n, U2, nrm, q, err); break;
    case CHARM_GPU_FLUX_HLLC: point_flux_kernel<T, NC, CHARM_GPU_FLUX_HLLC><<<g, bs, 0, st>>>(n, U2, nrm, q, err); break;
    case CHARM_GPU_FLUX_CD: point_flux_kernel<T, NC, CHARM_GPU_FLUX_CD><<<g, bs, 0, st>>>(n, U2, nrm, q, err); break;
    default: point_flux_kernel<T, NC, CHARM_GPU_FLUX_GODUNOV><<<g, bs, 0, st>>>(n, U2, nrm, q, err); break;
    }
}

cudaError_t point_launch_flux(const DevCfg *cfg, int flux, int n_comp, bool mixed, bool dword, int64_t n,
                              const double *U2, const double *nrm, double *q, unsigned *err, cudaStream_t st)
{
    cudaError_t e = cudaMemcpyToSymbolAsync(c_cfg, cfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    if (dword) {   // LF, HLLC, CD (the form's fluxes)
        const unsigned g = (unsigned) ((n + 127) / 128);
        if (n_comp == 1) {
            if (flux == CHARM_GPU_FLUX_LF) point_flux_kernel<dw, 1, CHARM_GPU_FLUX_LF><<<g, 128, 0, st>>>(n, U2, nrm, q, err);
            else if (flux == CHARM_GPU_FLUX_CD) point_flux_kernel<dw, 1, CHARM_GPU_FLUX_CD><<<g, 128, 0, st>>>(n, U2, nrm, q, err);
            else point_flux_kernel<dw, 1, CHARM_GPU_FLUX_HLLC><<<g, 128, 0, st>>>(n, U2, nrm, q, err);
        } else {
            if (flux == CHARM_GPU_FLUX_LF) point_flux_kernel<dw, 2, CHARM_GPU_FLUX_LF><<<g, 128, 0, st>>>(n, U2, nrm, q, err);
            else if (flux == CHARM_GPU_FLUX_CD) point_flux_kernel<dw, 2, CHARM_GPU_FLUX_CD><<<g, 128, 0, st>>>(n, U2, nrm, q, err);
            else point_flux_kernel<dw, 2, CHARM_GPU_FLUX_HLLC><<<g, 128, 0, st>>>(n, U2, nrm, q, err);
        }
        return cudaGetLastError();
    }
    switch (n_comp * 2 + (mixed ? 1 : 0)) {
    case 2: launch_point_flux<double, 1>(flux, n, U2, nrm, q, err, st); break;
    case 3: launch_point_flux<float, 1>(flux, n, U2, nrm, q, err, st); break;
    case 4: launch_point_flux<double, 2>(flux, n, U2, nrm, q, err, st); break;
    default: launch_point_flux<float, 2>(flux, n, U2, nrm, q, err, st); break;
    }
    return cudaGetLastError();
}

// The FP64 division helpers of the flux path on given operands (which = 0:
// rcp_nr(b); 1: qdiv(a, b)), for the check of their error against IEEE
// division.
__global__ void math_check_kernel(int which, int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                                  double *__restrict__ out)
{
    const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (which == 0) ? rcp_nr(b[i]) : qdiv<double>(a[i], b[i]);
}

cudaError_t point_launch_math(int which, int64_t n, const double *a, const double *b, double *out, cudaStream_t st)
{
    math_check_kernel<<<(unsigned) ((n + 127) / 128), 128, 0, st>>>(which, n, a, b, out);
    return cudaGetLastError();
}

}  // namespace charm
