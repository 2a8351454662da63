// C ABI of the GB300 DG time step (include/charm_gpu.h).
//
// Host orchestration of one time step, mirroring
// charm_model_ns_timestep_single (reference src/models/ns/charm_model.c:187-273):
//   rk_0 (save u^n), then 3 x [residual, u <- u - dt*M^-1*R, limiter] with
//   the 1/4-3/4 and 2/3-1/3 combinations after the 2nd and 3rd stage
//   (rk_1 / rk_2, :136-184), or one forward-Euler stage for the EULER model
//   (src/models/euler/charm_model.c:519-535).  Buffers:
//   u   state u^n, overwritten by u^{n+1} at the end of the step
//   ua  updated stage value before the limiter
//   ub  stage state (stage 1 and 2 results)
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "charm_gpu.h"
#include "dg_kernels.cuh"

using namespace charm;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(e_ == cudaErrorMemoryAllocation ? CHARM_GPU_ENOMEM : CHARM_GPU_ECUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    } while (0)

struct TimedLaunch {
    int cls;
    cudaEvent_t a, b;
};

}  // namespace

struct charm_gpu_handle_s {
    charm_gpu_config_t cfg;
    DevCfg dcfg;
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // mesh
    int64_t E = 0, F = 0, Fb = 0, S = 0;
    double tree_len[3] = {1, 1, 1};
    double *d_center = nullptr;
    int8_t *d_level = nullptr;
    int32_t *d_face_elem = nullptr;
    uint8_t *d_face_info = nullptr;
    int32_t *d_bface_elem = nullptr;
    int8_t *d_bface_face = nullptr, *d_bface_bnd = nullptr;
    int32_t *d_gather_ptr = nullptr, *d_gather_slot = nullptr;
    int32_t *d_lim_idx = nullptr;
    int8_t *d_lim_kind = nullptr;
    // state and work buffers
    double *d_u = nullptr, *d_ua = nullptr, *d_ub = nullptr;
    void *d_slots = nullptr;           // double or float [V*B][S]
    double *d_dt = nullptr;            // CFL step (bits as unsigned long long)
    unsigned *d_err = nullptr;
    bool mesh_ready = false;
    // accounting
    int64_t launches[4] = {0, 0, 0, 0};
    double ms[4] = {0, 0, 0, 0};
    bool timing = false;
    std::vector<TimedLaunch> pending;
    std::vector<cudaEvent_t> event_pool;
};

namespace {

const charm_gpu_handle_s *g_cfg_owner = nullptr;

int n_var(const charm_gpu_handle_s *h) { return 4 + h->cfg.n_comp; }

void free_mesh(charm_gpu_handle_s *h)
{
    void *ptrs[] = {h->d_center, h->d_level, h->d_face_elem, h->d_face_info, h->d_bface_elem, h->d_bface_face,
                    h->d_bface_bnd, h->d_gather_ptr, h->d_gather_slot, h->d_lim_idx, h->d_lim_kind, h->d_u,
                    h->d_ua, h->d_ub, h->d_slots};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    h->d_center = nullptr; h->d_level = nullptr; h->d_face_elem = nullptr; h->d_face_info = nullptr;
    h->d_bface_elem = nullptr; h->d_bface_face = nullptr; h->d_bface_bnd = nullptr;
    h->d_gather_ptr = nullptr; h->d_gather_slot = nullptr; h->d_lim_idx = nullptr; h->d_lim_kind = nullptr;
    h->d_u = h->d_ua = h->d_ub = nullptr;
    h->d_slots = nullptr;
    h->mesh_ready = false;
    h->E = h->F = h->Fb = h->S = 0;
}

int validate_config(const charm_gpu_config_t *c)
{
    if (c->model != CHARM_GPU_MODEL_EULER && c->model != CHARM_GPU_MODEL_NS)
        return fail(CHARM_GPU_EINVAL, "unknown model");
    if (c->flux < 0 || c->flux > 3) return fail(CHARM_GPU_EINVAL, "unknown flux type");
    if (c->limiter != CHARM_GPU_LIM_NONE && c->limiter != CHARM_GPU_LIM_BJ)
        return fail(CHARM_GPU_EINVAL, "unknown limiter type");
    if (c->eos != CHARM_GPU_EOS_IDEAL && c->eos != CHARM_GPU_EOS_MIX) return fail(CHARM_GPU_EINVAL, "unknown EOS");
    if (c->precision != CHARM_GPU_PREC_FP64 && c->precision != CHARM_GPU_PREC_MIXED)
        return fail(CHARM_GPU_EINVAL, "unknown precision");
    if (c->n_comp < 1 || c->n_comp > CHARM_GPU_MAX_COMP) return fail(CHARM_GPU_EINVAL, "n_comp out of range");
    if (c->n_comp > 2) return fail(CHARM_GPU_ENOTSUP, "more than 2 species not instantiated");
    if (c->n_bnd < 0 || c->n_bnd > CHARM_GPU_MAX_BND) return fail(CHARM_GPU_EINVAL, "n_bnd out of range");
    for (int i = 0; i < c->n_comp; i++) {
        if (!(c->comp[i].m > 0)) return fail(CHARM_GPU_EINVAL, "component molar mass must be > 0");
        if (c->comp[i].n_cp < 1 || c->comp[i].n_cp > CHARM_GPU_MAX_CP)
            return fail(CHARM_GPU_EINVAL, "component needs 1..8 cp coefficients");
    }
    for (int b = 0; b < c->n_bnd; b++)
        if (c->bnd[b].type < 0 || c->bnd[b].type > CHARM_GPU_BND_MASS_FLOW)
            return fail(CHARM_GPU_EINVAL, "unknown boundary type");
    if (c->use_visc) return fail(CHARM_GPU_ENOTSUP, "viscous terms are not implemented on the GPU path");
    if (c->dt_mode != CHARM_GPU_DT_TAU && c->dt_mode != CHARM_GPU_DT_CFL)
        return fail(CHARM_GPU_EINVAL, "unknown dt mode");
    return CHARM_GPU_OK;
}

void build_devcfg(const charm_gpu_config_t *c, DevCfg *d)
{
    memset(d, 0, sizeof(*d));
    d->n_comp = c->n_comp;
    d->eos = c->eos;
    for (int i = 0; i < c->n_comp; i++) {
        d->comp_m[i] = c->comp[i].m;
        d->comp_ncp[i] = c->comp[i].n_cp;
        d->comp_cp_type[i] = c->comp[i].cp_type;
        d->comp_ml_type[i] = c->comp[i].ml_type;
        for (int k = 0; k < c->comp[i].n_cp; k++) d->comp_cp[i][k] = c->comp[i].cp[k];
    }
    d->newton_t = (c->comp[0].cp_type == CHARM_GPU_CP_POLYNOM);
    // IDEAL with constant cp: the per-point values are the same every call
    // (src/charm_eos.c:113-116), computed once here in FP64.
    const bool cp_const0 = (c->comp[0].cp_type == CHARM_GPU_CP_CONST) ||
                           (c->comp[0].ml_type != CHARM_GPU_CP_POLYNOM && !d->newton_t);
    d->ideal_fast = (c->eos == CHARM_GPU_EOS_IDEAL) && cp_const0;
    if (d->ideal_fast) {
        d->ideal_cp = c->comp[0].cp[0];
        d->ideal_m = c->comp[0].m;
        d->ideal_cv = d->ideal_cp - kGasR / d->ideal_m;
        d->ideal_gam = d->ideal_cp / d->ideal_cv;
    }
    d->n_bnd = c->n_bnd;
    for (int b = 0; b < c->n_bnd; b++) {
        d->bnd_type[b] = c->bnd[b].type;
        for (int k = 0; k < 7 + CHARM_GPU_MAX_COMP; k++) d->bnd_par[b][k] = c->bnd[b].params[k];
    }
    for (int a = 0; a < 3; a++) d->grav[a] = c->grav[a];
    d->has_grav = (c->grav[0] != 0.0 || c->grav[1] != 0.0 || c->grav[2] != 0.0);
}

int ensure_cfg(charm_gpu_handle_s *h)
{
    if (g_cfg_owner == h) return CHARM_GPU_OK;
    CUDA_TRY(cudaMemcpyToSymbolAsync(c_cfg, &h->dcfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, h->stream));
    g_cfg_owner = h;
    return CHARM_GPU_OK;
}

MeshDev mesh_view(const charm_gpu_handle_s *h)
{
    MeshDev m;
    m.n_elem = h->E; m.n_face = h->F; m.n_bface = h->Fb; m.n_slot = h->S;
    m.center = h->d_center; m.level = h->d_level;
    m.face_elem = h->d_face_elem; m.face_info = h->d_face_info;
    m.bface_elem = h->d_bface_elem; m.bface_face = h->d_bface_face; m.bface_bnd = h->d_bface_bnd;
    m.gather_ptr = h->d_gather_ptr; m.gather_slot = h->d_gather_slot;
    m.lim_idx = h->d_lim_idx; m.lim_kind = h->d_lim_kind;
    for (int d = 0; d < 3; d++) m.tree_len[d] = h->tree_len[d];
    return m;
}

// ---- launch accounting ----------------------------------------------------

cudaEvent_t take_event(charm_gpu_handle_s *h)
{
    if (!h->event_pool.empty()) {
        cudaEvent_t e = h->event_pool.back();
        h->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void begin_launch(charm_gpu_handle_s *h, int cls, TimedLaunch *t)
{
    h->launches[cls]++;
    t->cls = cls;
    t->a = t->b = nullptr;
    if (h->timing) {
        t->a = take_event(h);
        t->b = take_event(h);
        cudaEventRecord(t->a, h->stream);
    }
}

void end_launch(charm_gpu_handle_s *h, TimedLaunch *t)
{
    if (h->timing && t->a) {
        cudaEventRecord(t->b, h->stream);
        h->pending.push_back(*t);
    }
}

void collect_timing(charm_gpu_handle_s *h)
{
    if (h->pending.empty()) return;
    cudaStreamSynchronize(h->stream);
    for (auto &t : h->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) h->ms[t.cls] += ms;
        h->event_pool.push_back(t.a);
        h->event_pool.push_back(t.b);
    }
    h->pending.clear();
}

// ---- typed launches -----------------------------------------------------------

template <typename T, int NC>
int launch_face(charm_gpu_handle_s *h, const double *u)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    if (nbi + nbb == 0) return CHARM_GPU_OK;
    T *slots = static_cast<T *>(h->d_slots);
    TimedLaunch t;
    begin_launch(h, 0, &t);
    switch (h->cfg.flux) {
    case CHARM_GPU_FLUX_LF:
        face_kernel<T, NC, CHARM_GPU_FLUX_LF><<<(unsigned) (nbi + nbb), bs, 0, h->stream>>>(m, u, slots, nbi, h->d_err);
        break;
    case CHARM_GPU_FLUX_HLLC:
        face_kernel<T, NC, CHARM_GPU_FLUX_HLLC><<<(unsigned) (nbi + nbb), bs, 0, h->stream>>>(m, u, slots, nbi, h->d_err);
        break;
    case CHARM_GPU_FLUX_CD:
        face_kernel<T, NC, CHARM_GPU_FLUX_CD><<<(unsigned) (nbi + nbb), bs, 0, h->stream>>>(m, u, slots, nbi, h->d_err);
        break;
    default:
        face_kernel<T, NC, CHARM_GPU_FLUX_GODUNOV><<<(unsigned) (nbi + nbb), bs, 0, h->stream>>>(m, u, slots, nbi, h->d_err);
        break;
    }
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <typename T, int NC>
int launch_cell(charm_gpu_handle_s *h, const double *u, const double *u0, double *out, double dt,
                const double *dt_dev, double a_new, double a_old, int mode)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 1, &t);
    cell_kernel<T, NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, u, static_cast<const T *>(h->d_slots), u0, out, dt,
                                                            dt_dev, a_new, a_old, mode, h->d_err);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_limit(charm_gpu_handle_s *h, const double *ua, const double *u0, double *out, double a_new, double a_old)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 2, &t);
    limit_kernel<NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, ua, u0, out, a_new, a_old);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_cfl(charm_gpu_handle_s *h, const double *u)
{
    MeshDev m = mesh_view(h);
    const double big = 1.0e300;
    CUDA_TRY(cudaMemcpyAsync(h->d_dt, &big, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const int bs = 256;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    cfl_dt_kernel<NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, u, h->cfg.cfl, reinterpret_cast<unsigned long long *>(h->d_dt));
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// One stage: out = a_new*L(u - dt*M^-1*R(u)) + a_old*u0 (L = limiter or identity).
template <typename T, int NC>
int stage(charm_gpu_handle_s *h, const double *u, const double *u0, double *out, double dt, const double *dt_dev,
          double a_new, double a_old)
{
    int rc = launch_face<T, NC>(h, u);
    if (rc) return rc;
    if (h->cfg.limiter == CHARM_GPU_LIM_BJ) {
        rc = launch_cell<T, NC>(h, u, nullptr, h->d_ua, dt, dt_dev, 1.0, 0.0, kCellUpdate);
        if (rc) return rc;
        return launch_limit<NC>(h, h->d_ua, u0, out, a_new, a_old);
    }
    return launch_cell<T, NC>(h, u, u0, out, dt, dt_dev, a_new, a_old, kCellUpdate);
}

template <typename T, int NC>
int step_impl(charm_gpu_handle_s *h, double dt, const double *dt_dev)
{
    int rc;
    const bool lim = h->cfg.limiter == CHARM_GPU_LIM_BJ;
    if (h->cfg.model == CHARM_GPU_MODEL_EULER) {
        if (lim) return stage<T, NC>(h, h->d_u, nullptr, h->d_u, dt, dt_dev, 1.0, 0.0);   // cell -> ua, limiter -> u
        if ((rc = stage<T, NC>(h, h->d_u, nullptr, h->d_ub, dt, dt_dev, 1.0, 0.0))) return rc;
        std::swap(h->d_u, h->d_ub);
        return CHARM_GPU_OK;
    }
    // SSP-RK3 in the reference's order (charm_model.c:259-266).  A stage
    // never writes the buffer it reads its residual from.
    if (lim) {
        if ((rc = stage<T, NC>(h, h->d_u, nullptr, h->d_ub, dt, dt_dev, 1.0, 0.0))) return rc;
        if ((rc = stage<T, NC>(h, h->d_ub, h->d_u, h->d_ub, dt, dt_dev, 0.25, 0.75))) return rc;
        return stage<T, NC>(h, h->d_ub, h->d_u, h->d_u, dt, dt_dev, 2.0 / 3.0, 1.0 / 3.0);
    }
    if ((rc = stage<T, NC>(h, h->d_u, nullptr, h->d_ub, dt, dt_dev, 1.0, 0.0))) return rc;
    if ((rc = stage<T, NC>(h, h->d_ub, h->d_u, h->d_ua, dt, dt_dev, 0.25, 0.75))) return rc;
    return stage<T, NC>(h, h->d_ua, h->d_u, h->d_u, dt, dt_dev, 2.0 / 3.0, 1.0 / 3.0);
}

template <typename T>
int step_dispatch_t(charm_gpu_handle_s *h, double dt, const double *dt_dev)
{
    switch (h->cfg.n_comp) {
    case 1: return step_impl<T, 1>(h, dt, dt_dev);
    case 2: return step_impl<T, 2>(h, dt, dt_dev);
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
}

int step_dispatch(charm_gpu_handle_s *h, double dt, const double *dt_dev)
{
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED) return step_dispatch_t<float>(h, dt, dt_dev);
    return step_dispatch_t<double>(h, dt, dt_dev);
}

int cfl_dispatch(charm_gpu_handle_s *h)
{
    switch (h->cfg.n_comp) {
    case 1: return launch_cfl<1>(h, h->d_u);
    case 2: return launch_cfl<2>(h, h->d_u);
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
}

int check_ready(charm_gpu_handle_s *h)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    if (!h->mesh_ready) return fail(CHARM_GPU_ESTATE, "no mesh uploaded");
    CUDA_TRY(cudaSetDevice(h->device));
    return ensure_cfg(h);
}

// Resolve the step for this call: explicit dt_in, fixed TAU, or CFL on device.
int resolve_dt(charm_gpu_handle_s *h, double dt_in, double *dt, const double **dt_dev)
{
    *dt_dev = nullptr;
    if (dt_in > 0) { *dt = dt_in; return CHARM_GPU_OK; }
    if (h->cfg.dt_mode == CHARM_GPU_DT_TAU) { *dt = h->cfg.tau; return CHARM_GPU_OK; }
    int rc = cfl_dispatch(h);
    if (rc) return rc;
    *dt = 0.0;
    *dt_dev = h->d_dt;
    return CHARM_GPU_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================

extern "C" {

const char *charm_gpu_version(void) { return "charm_gpu 0.1 (sm_103a)"; }
const char *charm_gpu_last_error(void) { return g_last_error.c_str(); }

int charm_gpu_create(charm_gpu_handle_t *out, const charm_gpu_config_t *cfg, int device)
{
    if (!out || !cfg) return fail(CHARM_GPU_EINVAL, "null argument");
    int rc = validate_config(cfg);
    if (rc) return rc;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(CHARM_GPU_EINVAL, "device index out of range");
    CUDA_TRY(cudaSetDevice(device));
    auto *h = new charm_gpu_handle_s();
    h->cfg = *cfg;
    h->device = device;
    build_devcfg(cfg, &h->dcfg);
    if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(CHARM_GPU_ECUDA, "cudaStreamCreate failed");
    }
    h->stream = h->own_stream;
    if (cudaMalloc(&h->d_err, sizeof(unsigned)) != cudaSuccess || cudaMalloc(&h->d_dt, sizeof(double)) != cudaSuccess) {
        if (h->d_err) cudaFree(h->d_err);
        cudaStreamDestroy(h->own_stream);
        delete h;
        return fail(CHARM_GPU_ENOMEM, "cudaMalloc failed");
    }
    cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), h->stream);
    *out = h;
    return CHARM_GPU_OK;
}

int charm_gpu_destroy(charm_gpu_handle_t h)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    collect_timing(h);
    free_mesh(h);
    if (h->d_err) cudaFree(h->d_err);
    if (h->d_dt) cudaFree(h->d_dt);
    for (auto e : h->event_pool) cudaEventDestroy(e);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (g_cfg_owner == h) g_cfg_owner = nullptr;
    delete h;
    return CHARM_GPU_OK;
}

int charm_gpu_upload_mesh(charm_gpu_handle_t h, const charm_gpu_mesh_t *mesh)
{
    if (!h || !mesh) return fail(CHARM_GPU_EINVAL, "null argument");
    const int64_t E = mesh->n_elem, F = mesh->n_face, Fb = mesh->n_bface;
    if (E <= 0 || F < 0 || Fb < 0) return fail(CHARM_GPU_EINVAL, "bad mesh sizes");
    if (E >= (int64_t) INT32_MAX) return fail(CHARM_GPU_EINVAL, "too many elements for int32 indices");
    if (!mesh->center || !mesh->level || (F && (!mesh->face_elem || !mesh->face_info)) ||
        (Fb && (!mesh->bface_elem || !mesh->bface_face || !mesh->bface_bnd)))
        return fail(CHARM_GPU_EINVAL, "null mesh array");
    // ---- validate indices and build the element tables on the host ----
    std::vector<int32_t> cnt(E + 1, 0);
    std::vector<int32_t> lim_idx(6 * E, -1);
    std::vector<int8_t> lim_kind(6 * E, -1);
    for (int64_t i = 0; i < F; i++) {
        const int32_t a = mesh->face_elem[i], b = mesh->face_elem[F + i];
        const unsigned info = mesh->face_info[i];
        const int d = info & 3, kind = (info >> 2) & 3;
        if (a < 0 || a >= E || b < 0 || b >= E || d > 2 || kind > 2)
            return fail(CHARM_GPU_EINVAL, "face record out of range");
        cnt[a]++; cnt[b]++;
        const int fa = 2 * d + 1, fb = 2 * d;   // face ids on side 0 / side 1
        if (kind == 0) {
            lim_kind[fa * E + a] = 0; lim_idx[fa * E + a] = b;
            lim_kind[fb * E + b] = 0; lim_idx[fb * E + b] = a;
        } else {
            const int sub = (info >> 4) & 3;
            const int32_t small = (kind == 1) ? a : b, big = (kind == 1) ? b : a;
            const int fs = (kind == 1) ? fa : fb, fbig = (kind == 1) ? fb : fa;
            lim_kind[fs * E + small] = 3; lim_idx[fs * E + small] = big;
            if (sub == 0) {
                // the 4 sub-faces of one big face must be consecutive records
                if (i + 3 >= F) return fail(CHARM_GPU_EINVAL, "incomplete mortar");
                for (int k = 1; k < 4; k++) {
                    const unsigned ik = mesh->face_info[i + k];
                    const int32_t bigk = (((ik >> 2) & 3) == 1) ? mesh->face_elem[F + i + k] : mesh->face_elem[i + k];
                    if (((ik >> 4) & 3) != (unsigned) k || bigk != big || (ik & 3) != (unsigned) d)
                        return fail(CHARM_GPU_EINVAL, "mortar sub-faces not consecutive");
                }
                lim_kind[fbig * E + big] = 2; lim_idx[fbig * E + big] = (int32_t) i;
            }
        }
    }
    for (int64_t j = 0; j < Fb; j++) {
        const int32_t e = mesh->bface_elem[j];
        const int f = mesh->bface_face[j], bnd = mesh->bface_bnd[j];
        if (e < 0 || e >= E || f < 0 || f > 5 || bnd < 0 || bnd >= h->cfg.n_bnd)
            return fail(CHARM_GPU_EINVAL, "boundary face record out of range");
        cnt[e]++;
        lim_kind[f * E + e] = 1; lim_idx[f * E + e] = (int32_t) j;
    }
    for (int64_t k = 0; k < 6 * E; k++)
        if (lim_kind[k] < 0) return fail(CHARM_GPU_EINVAL, "element face without a face record");
    std::vector<int32_t> ptr(E + 1, 0);
    for (int64_t e = 0; e < E; e++) ptr[e + 1] = ptr[e] + cnt[e];
    std::vector<int32_t> slot(ptr[E]);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t i = 0; i < F; i++) {
        slot[fill[mesh->face_elem[i]]++] = (int32_t) (2 * i);
        slot[fill[mesh->face_elem[F + i]]++] = (int32_t) (2 * i + 1);
    }
    for (int64_t j = 0; j < Fb; j++) slot[fill[mesh->bface_elem[j]]++] = (int32_t) (2 * F + j);
    int64_t S = 2 * F + Fb;
    S += (S & 1);

    CUDA_TRY(cudaSetDevice(h->device));
    cudaStreamSynchronize(h->stream);
    free_mesh(h);
    const int V = n_var(h);
    const size_t st = (size_t) V * CHARM_GPU_BASIS * E * sizeof(double);
    const size_t sl = (size_t) V * CHARM_GPU_BASIS * (S > 0 ? S : 2) *
                      (h->cfg.precision == CHARM_GPU_PREC_MIXED ? sizeof(float) : sizeof(double));
    CUDA_TRY(cudaMalloc(&h->d_center, 3 * E * sizeof(double)));
    CUDA_TRY(cudaMalloc(&h->d_level, E));
    CUDA_TRY(cudaMalloc(&h->d_face_elem, 2 * (F ? F : 1) * sizeof(int32_t)));
    CUDA_TRY(cudaMalloc(&h->d_face_info, F ? F : 1));
    CUDA_TRY(cudaMalloc(&h->d_bface_elem, (Fb ? Fb : 1) * sizeof(int32_t)));
    CUDA_TRY(cudaMalloc(&h->d_bface_face, Fb ? Fb : 1));
    CUDA_TRY(cudaMalloc(&h->d_bface_bnd, Fb ? Fb : 1));
    CUDA_TRY(cudaMalloc(&h->d_gather_ptr, (E + 1) * sizeof(int32_t)));
    CUDA_TRY(cudaMalloc(&h->d_gather_slot, (ptr[E] ? ptr[E] : 1) * sizeof(int32_t)));
    CUDA_TRY(cudaMalloc(&h->d_lim_idx, 6 * E * sizeof(int32_t)));
    CUDA_TRY(cudaMalloc(&h->d_lim_kind, 6 * E));
    CUDA_TRY(cudaMalloc(&h->d_u, st));
    CUDA_TRY(cudaMalloc(&h->d_ua, st));
    CUDA_TRY(cudaMalloc(&h->d_ub, st));
    CUDA_TRY(cudaMalloc(&h->d_slots, sl));
    CUDA_TRY(cudaMemcpy(h->d_center, mesh->center, 3 * E * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_level, mesh->level, E, cudaMemcpyHostToDevice));
    if (F) {
        CUDA_TRY(cudaMemcpy(h->d_face_elem, mesh->face_elem, 2 * F * sizeof(int32_t), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_face_info, mesh->face_info, F, cudaMemcpyHostToDevice));
    }
    if (Fb) {
        CUDA_TRY(cudaMemcpy(h->d_bface_elem, mesh->bface_elem, Fb * sizeof(int32_t), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_bface_face, mesh->bface_face, Fb, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_bface_bnd, mesh->bface_bnd, Fb, cudaMemcpyHostToDevice));
    }
    CUDA_TRY(cudaMemcpy(h->d_gather_ptr, ptr.data(), (E + 1) * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (ptr[E]) CUDA_TRY(cudaMemcpy(h->d_gather_slot, slot.data(), ptr[E] * sizeof(int32_t), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_lim_idx, lim_idx.data(), 6 * E * sizeof(int32_t), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_lim_kind, lim_kind.data(), 6 * E, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(h->d_u, 0, st));
    CUDA_TRY(cudaMemset(h->d_ua, 0, st));
    CUDA_TRY(cudaMemset(h->d_ub, 0, st));
    CUDA_TRY(cudaMemset(h->d_slots, 0, sl));
    h->E = E; h->F = F; h->Fb = Fb; h->S = S;
    for (int d = 0; d < 3; d++) h->tree_len[d] = mesh->tree_len[d];
    h->mesh_ready = true;
    return CHARM_GPU_OK;
}

int charm_gpu_set_state(charm_gpu_handle_t h, const double *u, int on_device)
{
    if (!h || !u) return fail(CHARM_GPU_EINVAL, "null argument");
    if (!h->mesh_ready) return fail(CHARM_GPU_ESTATE, "no mesh uploaded");
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(h->d_u, u, st, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    if (!on_device) CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_get_state(charm_gpu_handle_t h, double *u, int on_device)
{
    if (!h || !u) return fail(CHARM_GPU_EINVAL, "null argument");
    if (!h->mesh_ready) return fail(CHARM_GPU_ESTATE, "no mesh uploaded");
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(u, h->d_u, st, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    if (!on_device) CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_step(charm_gpu_handle_t h, double dt_in, double *dt_out)
{
    int rc = check_ready(h);
    if (rc) return rc;
    double dt;
    const double *dt_dev;
    if ((rc = resolve_dt(h, dt_in, &dt, &dt_dev))) return rc;
    if ((rc = step_dispatch(h, dt, dt_dev))) return rc;
    if (dt_out) {
        if (dt_dev) {
            CUDA_TRY(cudaMemcpyAsync(dt_out, h->d_dt, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            CUDA_TRY(cudaStreamSynchronize(h->stream));
        } else {
            *dt_out = dt;
        }
    }
    return CHARM_GPU_OK;
}

int charm_gpu_run(charm_gpu_handle_t h, int nsteps, double dt_in)
{
    int rc = check_ready(h);
    if (rc) return rc;
    for (int s = 0; s < nsteps; s++) {
        double dt;
        const double *dt_dev;
        if ((rc = resolve_dt(h, dt_in, &dt, &dt_dev))) return rc;
        if ((rc = step_dispatch(h, dt, dt_dev))) return rc;
        if (h->cfg.check_every > 0 && (s + 1) % h->cfg.check_every == 0) {
            if ((rc = charm_gpu_sync(h, 600.0))) return rc;
        }
    }
    return CHARM_GPU_OK;
}

int charm_gpu_get_dt(charm_gpu_handle_t h, double *dt)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (!dt) return fail(CHARM_GPU_EINVAL, "null argument");
    if (h->cfg.dt_mode == CHARM_GPU_DT_TAU) { *dt = h->cfg.tau; return CHARM_GPU_OK; }
    if ((rc = cfl_dispatch(h))) return rc;
    CUDA_TRY(cudaMemcpyAsync(dt, h->d_dt, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_residual(charm_gpu_handle_t h, double *res, int on_device)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (!res) return fail(CHARM_GPU_EINVAL, "null argument");
    const bool mixed = h->cfg.precision == CHARM_GPU_PREC_MIXED;
    switch (h->cfg.n_comp * 2 + (mixed ? 1 : 0)) {
    case 2: rc = launch_face<double, 1>(h, h->d_u); if (!rc) rc = launch_cell<double, 1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    case 3: rc = launch_face<float, 1>(h, h->d_u); if (!rc) rc = launch_cell<float, 1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    case 4: rc = launch_face<double, 2>(h, h->d_u); if (!rc) rc = launch_cell<double, 2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    case 5: rc = launch_face<float, 2>(h, h->d_u); if (!rc) rc = launch_cell<float, 2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
    if (rc) return rc;
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(res, h->d_ua, st, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_limit(charm_gpu_handle_t h)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->cfg.limiter != CHARM_GPU_LIM_BJ) return CHARM_GPU_OK;
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(h->d_ua, h->d_u, st, cudaMemcpyDeviceToDevice, h->stream));
    switch (h->cfg.n_comp) {
    case 1: return launch_limit<1>(h, h->d_ua, nullptr, h->d_u, 1.0, 0.0);
    case 2: return launch_limit<2>(h, h->d_ua, nullptr, h->d_u, 1.0, 0.0);
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
}

int charm_gpu_refine_flags(charm_gpu_handle_t h, double max_err, int8_t *flags, double *grad_out)
{
    (void) h; (void) max_err; (void) flags; (void) grad_out;
    return fail(CHARM_GPU_ENOTSUP, "refine indicator not built yet");
}

int charm_gpu_set_stream(charm_gpu_handle_t h, void *stream)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    g_cfg_owner = nullptr;   // re-upload constants on the new stream
    return CHARM_GPU_OK;
}

int charm_gpu_sync(charm_gpu_handle_t h, double timeout_s)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    CUDA_TRY(cudaSetDevice(h->device));
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t q = cudaStreamQuery(h->stream);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) return fail(CHARM_GPU_ECUDA, std::string("stream: ") + cudaGetErrorString(q));
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > timeout_s) return fail(CHARM_GPU_ETIMEDOUT, "charm_gpu_sync: timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    unsigned err = 0;
    CUDA_TRY(cudaMemcpy(&err, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (err) {
        CUDA_TRY(cudaMemset(h->d_err, 0, sizeof(unsigned)));
        if (err & kErrNonFinite) return fail(CHARM_GPU_ENONFINITE, "non-finite state");
        if (err & kErrNegative) return fail(CHARM_GPU_ENEGATIVE, "non-positive density or pressure");
        return fail(CHARM_GPU_EHLLC, "HLLC: SL <= S* <= SR violated");
    }
    return CHARM_GPU_OK;
}

int charm_gpu_set_timing(charm_gpu_handle_t h, int enable)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    h->timing = enable != 0;
    return CHARM_GPU_OK;
}

int charm_gpu_kernel_stats(charm_gpu_handle_t h, int64_t launches[4], double ms[4])
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    collect_timing(h);
    for (int k = 0; k < 4; k++) {
        if (launches) launches[k] = h->launches[k];
        if (ms) ms[k] = h->ms[k];
    }
    return CHARM_GPU_OK;
}

int charm_gpu_reset_stats(charm_gpu_handle_t h)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    collect_timing(h);
    for (int k = 0; k < 4; k++) { h->launches[k] = 0; h->ms[k] = 0.0; }
    return CHARM_GPU_OK;
}

int charm_gpu_time_run(charm_gpu_handle_t h, int nsteps, double dt_in, double *ms)
{
    int rc = check_ready(h);
    if (rc) return rc;
    if (!ms) return fail(CHARM_GPU_EINVAL, "null argument");
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    CUDA_TRY(cudaEventRecord(a, h->stream));
    rc = charm_gpu_run(h, nsteps, dt_in);
    if (rc) { cudaEventDestroy(a); cudaEventDestroy(b); return rc; }
    CUDA_TRY(cudaEventRecord(b, h->stream));
    rc = charm_gpu_sync(h, 3600.0);
    float f = 0.f;
    if (!rc) {
        cudaError_t e = cudaEventElapsedTime(&f, a, b);
        if (e != cudaSuccess) rc = fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = f;
    return rc;
}

int charm_gpu_probe_peak(int device, int which, double *tflops)
{
    if (!tflops || (which != 0 && which != 1)) return fail(CHARM_GPU_EINVAL, "bad argument");
    CUDA_TRY(cudaSetDevice(device));
    int nsm = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    const int threads = 256, blocks = nsm * 8, iters = (which == 0) ? 4096 : 65536;
    void *buf = nullptr;
    CUDA_TRY(cudaMalloc(&buf, (size_t) blocks * threads * sizeof(double)));
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        CUDA_TRY(cudaEventRecord(a, 0));
        if (which == 0) fma_peak_kernel<double><<<blocks, threads>>>(static_cast<double *>(buf), iters);
        else fma_peak_kernel<float><<<blocks, threads>>>(static_cast<float *>(buf), iters);
        CUDA_TRY(cudaEventRecord(b, 0));
        CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0 && ms < best) best = ms;   // first launch is a warm-up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    const double flops = 2.0 * kPeakChains * (double) iters * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return CHARM_GPU_OK;
}

int charm_gpu_abi_sizes(int64_t out[4])
{
    if (!out) return fail(CHARM_GPU_EINVAL, "null argument");
    out[0] = sizeof(charm_gpu_config_t);
    out[1] = sizeof(charm_gpu_mesh_t);
    out[2] = sizeof(charm_gpu_comp_t);
    out[3] = sizeof(charm_gpu_bnd_t);
    return CHARM_GPU_OK;
}

int charm_gpu_dims(charm_gpu_handle_t h, int64_t *n_elem, int *nv, int *nb)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    if (n_elem) *n_elem = h->E;
    if (nv) *nv = n_var(h);
    if (nb) *nb = CHARM_GPU_BASIS;
    return CHARM_GPU_OK;
}

}  // extern "C"
