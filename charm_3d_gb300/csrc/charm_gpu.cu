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
#include <cmath>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <algorithm>
#include <unordered_map>
#include <vector>

#include "charm_gpu.h"
#include "dg_kernels.cuh"
#include "dg_adjoint.cuh"
#include "dg_visc.cuh"
#include "dg_launch.h"
#include "charm_forest.h"

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
    int nb = CHARM_GPU_BASIS;          // basis functions: 4 (p1) or 10 (p2)
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
    // mixed form: FP32 hi/lo planes of u, ua, ub ([V][B][E] each)
    float *d_fh[3] = {nullptr, nullptr, nullptr}, *d_fl[3] = {nullptr, nullptr, nullptr};
    // mixed form, block-local stage: per-tile face records, halo lists and element-face slots
    int32_t *d_tile_fptr = nullptr, *d_tile_slot = nullptr, *d_tile_hptr = nullptr, *d_tile_halo = nullptr;
    int4 *d_tile_rec = nullptr;
    int tile_ncol = 0;
    int64_t n_tiles = 0;
    size_t tile_smem = 0;      // dynamic shared memory of tile_stage_kernel (0: use ff_stage_kernel)
    // discrete adjoint (allocated by the first adjoint call, sized by the mesh)
    double *d_adj_lam = nullptr, *d_adj_s = nullptr, *d_adj_acc = nullptr;   // [V][B][E] each
    double *d_adj_u1 = nullptr, *d_adj_u2 = nullptr, *d_adj_fin = nullptr;   // stage states, final state
    double *d_adj_psi = nullptr;                                              // [3][V][E] limiter scalings
    double *d_adj_psi_all = nullptr;                                          // [steps][3][V][E]
    size_t n_psi_all = 0;
    double *d_obj_part = nullptr;                                             // objective partial sums
    std::vector<double *> d_snap;                                             // checkpoints
    bool adj_valid = false;           // d_adj_lam holds dJ/du0 of the last adjoint run
    // viscous terms and chemistry (NS model, FP64)
    double *d_s9 = nullptr;            // lifting face terms [9*B][S]
    double *d_vis = nullptr;           // lifted tau and q [9][B][E]
    double *d_radd = nullptr;          // viscous volume terms [4][B][E]
    double *d_dif = nullptr;           // species diffusion coefficients [n_comp][E]
    double *d_uc = nullptr;            // stage state after chemistry [V][B][E]
    double *d_chem_rhs = nullptr;      // heat release of the stage [E]
    double *d_dt = nullptr;            // CFL step (bits as unsigned long long)
    double *d_dt_next = nullptr;       // the next step's CFL step, reduced by the last stage of a step
    bool dt_next_valid = false;        // d_dt_next holds the CFL step of the current state
    double *d_proj[2] = {nullptr, nullptr};   // adapt projection ping-pong states
    int32_t *d_pmap = nullptr;         // one pass of an adapt plan
    unsigned *d_err = nullptr;
    bool mesh_ready = false;
    // general hexahedra (charm_gpu_upload_mesh_hex): corners, face numbers
    // and the geometry tables of dg_hex.cuh
    bool hex = false;
    double *d_hex_vert = nullptr, *d_hex_g = nullptr, *d_hex_fg = nullptr;
    int8_t *d_hex_ff = nullptr;
    // back-to-back steps replayed as a CUDA graph (charm_gpu_run): the
    // executable graph of two steps, the step and state buffers it was
    // captured with, and the launches per kernel class it contains
    cudaGraphExec_t run_graph = nullptr;
    double run_graph_dt = 0.0;
    cudaStream_t run_graph_stream = nullptr;
    std::vector<void *> run_graph_bufs;
    int64_t run_graph_launches[4] = {0, 0, 0, 0};
    // accounting
    int64_t launches[4] = {0, 0, 0, 0};
    double ms[4] = {0, 0, 0, 0};
    bool timing = false;
    std::vector<TimedLaunch> pending;
    std::vector<cudaEvent_t> event_pool;
    // capacity in bytes of the mesh-sized device buffers, by the address of
    // the handle member that holds each one: an upload after an adapt keeps
    // every buffer that is still large enough
    std::unordered_map<const void *, size_t> dcap;
};

namespace {

// The kernels read the solver configuration from one __constant__ symbol
// (c_cfg, one copy per device).  Handles on the same device take turns: each
// API call that launches kernels holds the device's CfgLease for its whole
// launch sequence, and when another handle (or another stream) takes the
// symbol over, its stream first waits on an event recorded after the last
// work that read the previous contents.  So handles with different
// configurations can be driven from several host threads and streams.
constexpr int kMaxCfgDevices = 64;
struct CfgSlot {
    std::recursive_mutex mu;
    const void *owner = nullptr;     // handle whose DevCfg c_cfg holds (nullptr: none)
    cudaStream_t stream = nullptr;   // stream of the last launches that read c_cfg
    bool live = false;               // `stream` may still have such work queued
    bool fence_pending = false;      // `fence` marks such work on a stream given up since
    cudaEvent_t fence = nullptr;
};
CfgSlot g_cfg_slot[kMaxCfgDevices];

CfgSlot &cfg_slot(int device) { return g_cfg_slot[(device >= 0 && device < kMaxCfgDevices) ? device : 0]; }

class CfgLease {
  public:
    explicit CfgLease(int device) : mu_(&cfg_slot(device).mu) { mu_->lock(); }
    explicit CfgLease(const charm_gpu_handle_s *h);
    ~CfgLease() { if (mu_) mu_->unlock(); }
    CfgLease(const CfgLease &) = delete;
    CfgLease &operator=(const CfgLease &) = delete;
  private:
    std::recursive_mutex *mu_ = nullptr;
};

// Order `next` after every queued launch that reads the current contents of
// c_cfg (the caller holds the lease).  Returns a CUDA error or cudaSuccess.
cudaError_t cfg_takeover(CfgSlot &s, cudaStream_t next)
{
    cudaError_t e = cudaSuccess;
    if ((s.live && s.stream != next) || s.fence_pending) {
        if (!s.fence && (e = cudaEventCreateWithFlags(&s.fence, cudaEventDisableTiming)) != cudaSuccess) return e;
        if (s.live && s.stream != next && (e = cudaEventRecord(s.fence, s.stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(next, s.fence, 0)) != cudaSuccess) return e;
    }
    s.fence_pending = false;
    return e;
}

int n_var(const charm_gpu_handle_s *h) { return 4 + h->cfg.n_comp; }

// Device buffer *p of at least `bytes` bytes: kept when the current one is
// large enough, else replaced (contents are not preserved).
template <typename P>
int ensure_buf(charm_gpu_handle_s *h, P **p, size_t bytes)
{
    size_t &cap = h->dcap[static_cast<const void *>(p)];
    if (*p && cap >= bytes) return CHARM_GPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = 0;
    if (cudaMalloc(reinterpret_cast<void **>(p), bytes) != cudaSuccess) {
        *p = nullptr;
        return fail(CHARM_GPU_ENOMEM, "cudaMalloc of a mesh buffer failed");
    }
    cap = bytes;
    return CHARM_GPU_OK;
}

// Drop what belongs to the previous mesh but is not a reusable buffer: the
// adjoint's buffers and checkpoints (sized by the run), the flags.
void drop_run_graph(charm_gpu_handle_s *h)
{
    if (h->run_graph) cudaGraphExecDestroy(h->run_graph);   // freed when its launches complete
    h->run_graph = nullptr;
    h->run_graph_bufs.clear();
}

void reset_mesh(charm_gpu_handle_s *h)
{
    drop_run_graph(h);
    double **adj[] = {&h->d_adj_lam, &h->d_adj_s, &h->d_adj_acc, &h->d_adj_u1, &h->d_adj_u2, &h->d_adj_fin,
                      &h->d_adj_psi, &h->d_obj_part, &h->d_adj_psi_all};
    for (double **q : adj) {
        if (*q) cudaFree(*q);
        *q = nullptr;
    }
    h->n_psi_all = 0;
    for (double *q : h->d_snap) cudaFree(q);
    h->d_snap.clear();
    h->adj_valid = false;
    h->dt_next_valid = false;
    h->n_tiles = 0;
    h->tile_smem = 0;
    h->mesh_ready = false;
    h->hex = false;
    h->E = h->F = h->Fb = h->S = 0;
}

void free_mesh(charm_gpu_handle_s *h)
{
    drop_run_graph(h);
    void *ptrs[] = {h->d_center, h->d_level, h->d_face_elem, h->d_face_info, h->d_bface_elem, h->d_bface_face,
                    h->d_bface_bnd, h->d_gather_ptr, h->d_gather_slot, h->d_lim_idx, h->d_lim_kind, h->d_u,
                    h->d_ua, h->d_ub, h->d_slots, h->d_hex_vert, h->d_hex_g, h->d_hex_fg, h->d_hex_ff};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int k = 0; k < 3; k++) {
        if (h->d_fh[k]) cudaFree(h->d_fh[k]);
        if (h->d_fl[k]) cudaFree(h->d_fl[k]);
        h->d_fh[k] = h->d_fl[k] = nullptr;
    }
    if (h->d_tile_fptr) cudaFree(h->d_tile_fptr);
    if (h->d_tile_rec) cudaFree(h->d_tile_rec);
    if (h->d_tile_slot) cudaFree(h->d_tile_slot);
    if (h->d_tile_hptr) cudaFree(h->d_tile_hptr);
    if (h->d_tile_halo) cudaFree(h->d_tile_halo);
    h->d_tile_fptr = h->d_tile_slot = h->d_tile_hptr = h->d_tile_halo = nullptr;
    h->d_tile_rec = nullptr;
    double **adj[] = {&h->d_adj_lam, &h->d_adj_s, &h->d_adj_acc, &h->d_adj_u1, &h->d_adj_u2, &h->d_adj_fin,
                      &h->d_adj_psi, &h->d_obj_part, &h->d_adj_psi_all};
    h->n_psi_all = 0;
    for (double **q : adj) {
        if (*q) cudaFree(*q);
        *q = nullptr;
    }
    for (double *q : h->d_snap) cudaFree(q);
    h->d_snap.clear();
    double **visc[] = {&h->d_s9, &h->d_vis, &h->d_radd, &h->d_dif, &h->d_uc, &h->d_chem_rhs, &h->d_proj[0],
                       &h->d_proj[1]};
    if (h->d_pmap) cudaFree(h->d_pmap);
    h->d_pmap = nullptr;
    for (double **q : visc) {
        if (*q) cudaFree(*q);
        *q = nullptr;
    }
    h->adj_valid = false;
    h->dcap.clear();
    h->n_tiles = 0;
    h->tile_smem = 0;
    h->d_center = nullptr; h->d_level = nullptr; h->d_face_elem = nullptr; h->d_face_info = nullptr;
    h->d_bface_elem = nullptr; h->d_bface_face = nullptr; h->d_bface_bnd = nullptr;
    h->d_gather_ptr = nullptr; h->d_gather_slot = nullptr; h->d_lim_idx = nullptr; h->d_lim_kind = nullptr;
    h->d_u = h->d_ua = h->d_ub = nullptr;
    h->d_slots = nullptr;
    h->d_hex_vert = h->d_hex_g = h->d_hex_fg = nullptr;
    h->d_hex_ff = nullptr;
    h->mesh_ready = false;
    h->hex = false;
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
    if (c->precision != CHARM_GPU_PREC_FP64 && c->precision != CHARM_GPU_PREC_MIXED && c->precision != CHARM_GPU_PREC_DW)
        return fail(CHARM_GPU_EINVAL, "unknown precision");
    if (c->precision == CHARM_GPU_PREC_DW && (c->p_order == 2 || c->use_visc || c->n_react))
        return fail(CHARM_GPU_ENOTSUP, "double-word form: p1 convective terms only");
    if (c->precision == CHARM_GPU_PREC_DW && c->flux == CHARM_GPU_FLUX_GODUNOV)
        return fail(CHARM_GPU_ENOTSUP, "double-word form: LF, HLLC or CD flux");
    if (c->precision == CHARM_GPU_PREC_DW &&
        (c->eos != CHARM_GPU_EOS_IDEAL || c->comp[0].cp_type == CHARM_GPU_CP_POLYNOM))
        return fail(CHARM_GPU_ENOTSUP, "double-word form: ideal gas with constant cp");
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
    if (c->p_order < 0 || c->p_order > 2) return fail(CHARM_GPU_EINVAL, "p_order must be 1 or 2");
    if (c->p_order == 2) {
        if (c->limiter != CHARM_GPU_LIM_NONE && c->precision != CHARM_GPU_PREC_FP64)
            return fail(CHARM_GPU_ENOTSUP, "p2: the limiter runs in the FP64 form only");
        if (c->dt_mode != CHARM_GPU_DT_TAU) return fail(CHARM_GPU_ENOTSUP, "p2: fixed time step (TAU) only");
    }
    if (c->n_react < 0 || c->n_react > CHARM_GPU_MAX_REACT) return fail(CHARM_GPU_EINVAL, "bad reaction count");
    for (int r = 0; r < c->n_react; r++)
        for (int k = 0; k < 3; k++)
            if (c->react[r].left[k] < -1 || c->react[r].left[k] >= c->n_comp || c->react[r].right[k] < -1 ||
                c->react[r].right[k] >= c->n_comp)
                return fail(CHARM_GPU_EINVAL, "reaction component index out of range");
    if ((c->use_visc || c->n_react) && c->precision != CHARM_GPU_PREC_FP64 && c->p_order != 2)
        return fail(CHARM_GPU_ENOTSUP, "viscous terms and reactions in the mixed form: p2 basis only");
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
        d->ideal_inv_cv = 1.0 / d->ideal_cv;
        d->ideal_qg = (d->ideal_gam + 1.0) / (2.0 * d->ideal_gam);
        d->ideal_gm1 = d->ideal_gam - 1.0;
    }
    d->n_bnd = c->n_bnd;
    for (int b = 0; b < c->n_bnd; b++) {
        d->bnd_type[b] = c->bnd[b].type;
        for (int k = 0; k < 7 + CHARM_GPU_MAX_COMP; k++) d->bnd_par[b][k] = c->bnd[b].params[k];
    }
    for (int a = 0; a < 3; a++) d->grav[a] = c->grav[a];
    d->has_grav = (c->grav[0] != 0.0 || c->grav[1] != 0.0 || c->grav[2] != 0.0);
    // float mirrors for the FP32 instantiations
    d->ideal_cp_f = (float) d->ideal_cp; d->ideal_m_f = (float) d->ideal_m; d->ideal_cv_f = (float) d->ideal_cv;
    d->ideal_gam_f = (float) d->ideal_gam; d->ideal_inv_cv_f = (float) d->ideal_inv_cv;
    d->ideal_qg_f = (float) d->ideal_qg;
    d->ideal_gm1_f = (float) d->ideal_gam - 1.f;   // as the float path computed it before
    for (int i = 0; i < CHARM_GPU_MAX_COMP; i++) {
        d->comp_m_f[i] = (float) d->comp_m[i];
        d->comp_inv_m[i] = d->comp_m[i] != 0.0 ? 1.0 / d->comp_m[i] : 0.0;
        d->comp_inv_m_f[i] = (float) d->comp_inv_m[i];
        for (int k = 0; k < CHARM_GPU_MAX_CP; k++) d->comp_cp_f[i][k] = (float) d->comp_cp[i][k];
    }
    for (int b = 0; b < CHARM_GPU_MAX_BND; b++)
        for (int k = 0; k < 7 + CHARM_GPU_MAX_COMP; k++) d->bnd_par_f[b][k] = (float) d->bnd_par[b][k];
    for (int a = 0; a < 3; a++) d->grav_f[a] = (float) d->grav[a];
    d->use_visc = c->use_visc;
    d->use_diff = c->use_diff;
    d->n_react = c->n_react;
    d->t_ref = c->t_ref;
    d->tau = c->tau;
    for (int i = 0; i < c->n_comp; i++) {
        d->comp_ml0[i] = c->comp[i].ml0; d->comp_kp0[i] = c->comp[i].kp0;
        d->comp_t0[i] = c->comp[i].t0; d->comp_ts[i] = c->comp[i].ts;
        d->comp_sig[i] = c->comp[i].sig; d->comp_ek[i] = c->comp[i].ek; d->comp_h0[i] = c->comp[i].h0;
        d->comp_kp_type[i] = c->comp[i].kp_type;
        d->comp_href[i] = 0.0;
        for (int k = 0; k < c->comp[i].n_cp; k++) {
            d->comp_hc[i][k] = c->comp[i].cp[k] / (k + 1);
            d->comp_href[i] += c->comp[i].cp[k] * pow(c->t_ref, k + 1) / (k + 1);
        }
        d->comp_ml0_f[i] = (float) d->comp_ml0[i]; d->comp_kp0_f[i] = (float) d->comp_kp0[i];
        d->comp_t0_f[i] = (float) d->comp_t0[i]; d->comp_ts_f[i] = (float) d->comp_ts[i];
        for (int k = 0; k < CHARM_GPU_MAX_CP; k++) d->comp_hc_f[i][k] = (float) d->comp_hc[i][k];
        d->comp_hoff_f[i] = (float) (d->comp_h0[i] - d->comp_href[i]);
    }
    for (int r = 0; r < c->n_react; r++) {
        for (int k = 0; k < 3; k++) { d->react_l[r][k] = c->react[r].left[k]; d->react_r[r][k] = c->react[r].right[k]; }
        d->react_a[r] = c->react[r].a; d->react_e[r] = c->react[r].e; d->react_n[r] = c->react[r].n;
    }
}

CfgLease::CfgLease(const charm_gpu_handle_s *h)
{
    if (h) {
        mu_ = &cfg_slot(h->device).mu;
        mu_->lock();
    }
}

// Make c_cfg hold h's configuration for launches on h's stream (the caller
// holds h's CfgLease).
int ensure_cfg(charm_gpu_handle_s *h)
{
    CfgSlot &s = cfg_slot(h->device);
    if (s.owner == h && s.live && s.stream == h->stream) return CHARM_GPU_OK;
    CUDA_TRY(cfg_takeover(s, h->stream));
    CUDA_TRY(cudaMemcpyToSymbolAsync(c_cfg, &h->dcfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(p2_upload_cfg(&h->dcfg, h->stream));
    CUDA_TRY(dw_upload_cfg(&h->dcfg, h->stream));
    CUDA_TRY(hex_upload_cfg(&h->dcfg, h->stream));
    s.owner = h;
    s.stream = h->stream;
    s.live = true;
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
    for (int d = 0; d < 3; d++) {
        m.tree_len[d] = h->tree_len[d];
        m.tree_len_f[d] = (float) h->tree_len[d];
    }
    return m;
}

HexDev hex_view(const charm_gpu_handle_s *h)
{
    HexDev x;
    x.g = h->d_hex_g;
    x.fg = h->d_hex_fg;
    x.face_face = h->d_hex_ff;
    x.vert = h->d_hex_vert;
    return x;
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
    if constexpr (std::is_same<T, double>::value) {
        if (h->hex) {
            hex_launch_face<NC>(h->cfg.flux, m, hex_view(h), u, slots, h->d_err, h->stream);
            end_launch(h, &t);
            CUDA_TRY(cudaGetLastError());
            return CHARM_GPU_OK;
        }
    }
    if constexpr (is_dw<T>) {
        dw_launch_face<NC>(h->cfg.flux, m, u, slots, nbi, (unsigned) (nbi + nbb), h->d_err, h->stream);
        end_launch(h, &t);
        CUDA_TRY(cudaGetLastError());
        return CHARM_GPU_OK;
    } else
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
                const double *dt_dev, double a_new, double a_old, int mode, const double *radd = nullptr,
                double *dt_next = nullptr)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 1, &t);
    if (h->hex) {
        if constexpr (std::is_same<T, double>::value)
            hex_launch_cell<NC>(m, hex_view(h), u, static_cast<const double *>(h->d_slots), u0, out, dt, dt_dev, a_new,
                                a_old, mode, h->d_err, reinterpret_cast<unsigned long long *>(dt_next), h->cfg.cfl,
                                h->stream);
    } else
    if constexpr (is_dw<T>)
        dw_launch_cell<NC>(m, u, static_cast<const T *>(h->d_slots), u0, out, dt, dt_dev, a_new, a_old, mode, h->d_err,
                           radd, reinterpret_cast<unsigned long long *>(dt_next), h->cfg.cfl, h->stream);
    else
    cell_kernel<T, NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, u, static_cast<const T *>(h->d_slots), u0, out, dt,
                                                            dt_dev, a_new, a_old, mode, h->d_err, radd,
                                                            reinterpret_cast<unsigned long long *>(dt_next), h->cfg.cfl);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_limit(charm_gpu_handle_s *h, const double *ua, const double *u0, double *out, double a_new, double a_old,
                 double *psi_out = nullptr, double *dt_next = nullptr)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 2, &t);
    if (h->hex)
        hex_launch_limit<NC>(m, hex_view(h), ua, u0, out, a_new, a_old, reinterpret_cast<unsigned long long *>(dt_next),
                             h->cfg.cfl, h->stream);
    else
    limit_kernel<NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, ua, u0, out, a_new, a_old, psi_out,
                                                          reinterpret_cast<unsigned long long *>(dt_next), h->cfg.cfl);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_cfl(charm_gpu_handle_s *h, const double *u)
{
    MeshDev m = mesh_view(h);
    // the reference's reduction starts from TAU (src/models/ns/charm_model.c:50)
    const double start = (h->cfg.tau > 0.0) ? h->cfg.tau : 1.0e300;
    CUDA_TRY(cudaMemcpyAsync(h->d_dt, &start, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const int bs = 256;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    if (h->hex)
        hex_launch_cfl<NC>(m, hex_view(h), u, reinterpret_cast<unsigned long long *>(h->d_dt), h->cfg.cfl, h->stream);
    else
    cfl_dt_kernel<NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, u, h->cfg.cfl, reinterpret_cast<unsigned long long *>(h->d_dt));
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// One stage: out = a_new*L(u - dt*M^-1*R(u)) + a_old*u0 (L = limiter or identity).
// ---- p2 basis -------------------------------------------------------------------

// Rule tables and the inverse mass matrix of the reference box for the p2
// kernels (3-point Gauss-Legendre per axis; the mass matrix by the 27-point
// rule, exact for the quadratic basis, inverted by Gauss-Jordan).
int upload_p2_tables(charm_gpu_handle_s *h)
{
    P2TabT<double> t;
    memset(&t, 0, sizeof(t));
    const double gx[3] = {-0.5 * sqrt(0.6), 0.0, 0.5 * sqrt(0.6)};
    const double gw[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};
    for (int i = 0; i < 27; i++) {
        const int ix = i % 3, iy = (i / 3) % 3, iz = i / 9;
        t.cxi[i][0] = gx[ix]; t.cxi[i][1] = gx[iy]; t.cxi[i][2] = gx[iz];
        t.cw[i] = gw[ix] * gw[iy] * gw[iz];
    }
    for (int i = 0; i < 9; i++) {
        t.fxi[i][0] = gx[i % 3]; t.fxi[i][1] = gx[i / 3];
        t.fw[i] = gw[i % 3] * gw[i / 3];
    }
    double a[kNB2][2 * kNB2];
    memset(a, 0, sizeof(a));
    for (int q = 0; q < 27; q++) {
        const double x = t.cxi[q][0], y = t.cxi[q][1], z = t.cxi[q][2];
        const double ph[kNB2] = {1.0, x, y, z, x * x, y * y, z * z, x * y, x * z, y * z};
        for (int i = 0; i < kNB2; i++) {
            t.mean[i] += t.cw[q] * ph[i];
            for (int j = 0; j < kNB2; j++) a[i][j] += t.cw[q] * ph[i] * ph[j];
        }
    }
    // odd moments vanish on the symmetric rule: keep them exact zeros, so that
    // M^-1 is exactly block-structured ({0, 4, 5, 6} coupled, the rest diagonal)
    auto coupled = [](int i, int j) {
        const bool bi = (i == 0 || (i >= 4 && i <= 6)), bj = (j == 0 || (j >= 4 && j <= 6));
        return i == j || (bi && bj);
    };
    for (int i = 0; i < kNB2; i++)
        for (int j = 0; j < kNB2; j++)
            if (!coupled(i, j)) a[i][j] = 0.0;
    for (int i = 0; i < kNB2; i++) a[i][kNB2 + i] = 1.0;
    for (int c = 0; c < kNB2; c++) {   // Gauss-Jordan, partial pivoting
        int piv = c;
        for (int r = c + 1; r < kNB2; r++)
            if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
        if (piv != c)
            for (int k = 0; k < 2 * kNB2; k++) std::swap(a[c][k], a[piv][k]);
        const double d = a[c][c];
        for (int k = 0; k < 2 * kNB2; k++) a[c][k] /= d;
        for (int r = 0; r < kNB2; r++) {
            if (r == c) continue;
            const double f = a[r][c];
            for (int k = 0; k < 2 * kNB2; k++) a[r][k] -= f * a[c][k];
        }
    }
    for (int i = 0; i < kNB2; i++)
        for (int j = 0; j < kNB2; j++) t.minv[i][j] = coupled(i, j) ? a[i][kNB2 + j] : 0.0;
    P2TabT<float> tf;
    for (int i = 0; i < 27; i++) {
        for (int k = 0; k < 3; k++) tf.cxi[i][k] = (float) t.cxi[i][k];
        tf.cw[i] = (float) t.cw[i];
    }
    for (int i = 0; i < 9; i++) {
        for (int k = 0; k < 2; k++) tf.fxi[i][k] = (float) t.fxi[i][k];
        tf.fw[i] = (float) t.fw[i];
    }
    for (int i = 0; i < kNB2; i++) {
        for (int j = 0; j < kNB2; j++) tf.minv[i][j] = (float) t.minv[i][j];
        tf.mean[i] = (float) t.mean[i];
    }
    CUDA_TRY(p2_upload_tables(t, tf));
    return CHARM_GPU_OK;
}

// p2 launchers, for T = double (FP64 form) and T = float (mixed form: u is
// the hi plane; the slot, lifting and volume-term buffers hold T).  The
// kernels are in charm_p2.cu.
template <typename T, int NC>
int launch_p2_face(charm_gpu_handle_s *h, const T *u)
{
    const int bs = 128;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    if (nbi + nbb == 0) return CHARM_GPU_OK;
    TimedLaunch t;
    begin_launch(h, 0, &t);
    p2_launch_face<T, NC>(h->cfg.flux, mesh_view(h), u, static_cast<T *>(h->d_slots), nbi, (unsigned) (nbi + nbb),
                          h->d_err, h->stream);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <typename T, int NC>
int launch_p2_cell(charm_gpu_handle_s *h, const T *u, const T *u0, T *out, const P2Upd &up, const T *radd)
{
    TimedLaunch t;
    begin_launch(h, 1, &t);
    p2_launch_cell<T, NC>(mesh_view(h), u, static_cast<const T *>(h->d_slots), u0, out, up, h->d_err, radd, h->stream);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// chemistry of the stage state (FP64 from the state S) -> h->d_uc, chem_rhs
template <typename S, int NC>
int launch_p2_chem(charm_gpu_handle_s *h, StIn<S> in, StOut<S> out)
{
    TimedLaunch t;
    begin_launch(h, 3, &t);
    p2_launch_chem<S, NC>(mesh_view(h), in, out, h->d_chem_rhs, h->stream);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// diffusion coefficients, lifting and the viscous volume terms -> h->d_radd
// (u_lo: the lo plane in the mixed form, for the FP64 diffusion coefficients)
template <typename T, int NC>
int launch_p2_visc(charm_gpu_handle_s *h, const T *u, const float *u_lo, const double *chem_rhs)
{
    const int bs = 128;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    p2_launch_visc<T, NC>(mesh_view(h), h->cfg.use_diff != 0, u, u_lo, reinterpret_cast<T *>(h->d_dif),
                          reinterpret_cast<T *>(h->d_s9), reinterpret_cast<T *>(h->d_vis), chem_rhs,
                          reinterpret_cast<T *>(h->d_radd), nbi, (unsigned) (nbi + nbb), h->stream);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <typename T, int NC>
int launch_p2_vflux(charm_gpu_handle_s *h, const T *u)
{
    const int bs = 128;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    if (nbi + nbb == 0) return CHARM_GPU_OK;
    TimedLaunch t;
    begin_launch(h, 0, &t);
    p2_launch_vflux<T, NC>(mesh_view(h), u, reinterpret_cast<const T *>(h->d_vis), static_cast<T *>(h->d_slots), nbi,
                           (unsigned) (nbi + nbb), h->stream);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// one FP64 p2 stage (or, with mode kCellResidual, the residual without chemistry)
template <int NC>
int launch_p2_limit(charm_gpu_handle_s *h, const double *ua, const double *u0, double *out, double a_new, double a_old)
{
    TimedLaunch t;
    begin_launch(h, 2, &t);
    p2_launch_limit<NC>(mesh_view(h), ua, u0, out, a_new, a_old, h->stream);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int p2_stage(charm_gpu_handle_s *h, const double *u, const double *u0, double *out, double dt, const double *dt_dev,
             double a_new, double a_old, int mode)
{
    int rc;
    const double *radd = nullptr;
    const bool upd = mode == kCellUpdate;
    if (h->cfg.model == CHARM_GPU_MODEL_NS) {
        if (upd && h->cfg.n_react) {
            if ((rc = launch_p2_chem<double, NC>(h, StIn<double>{u}, StOut<double>{h->d_uc}))) return rc;
            u = h->d_uc;   // the residual and the update act on the state after chemistry
        }
        if (h->cfg.use_visc) {
            if ((rc = launch_p2_visc<double, NC>(h, u, nullptr, upd ? h->d_chem_rhs : nullptr))) return rc;
            radd = h->d_radd;
        }
    }
    if ((rc = launch_p2_face<double, NC>(h, u))) return rc;
    if (radd && (rc = launch_p2_vflux<double, NC>(h, u))) return rc;
    P2Upd up{};
    up.dt = dt; up.a_new = a_new; up.a_old = a_old; up.dt_dev = dt_dev; up.mode = mode;
    return launch_p2_cell<double, NC>(h, u, u0, out, up, radd);
}

// ---- viscous terms and chemistry (charm_model_ns_timestep_single's stage,
//      src/models/ns/charm_model.c:242-253: chem, diff, conv, update) -------

bool has_visc_chem(const charm_gpu_handle_s *h)
{
    return h->cfg.model == CHARM_GPU_MODEL_NS && (h->cfg.use_visc || h->cfg.n_react);
}

// chemistry of the stage state u -> h->d_uc (when there are reactions)
template <int NC>
int launch_chem(charm_gpu_handle_s *h, const double *u)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    chem_kernel<NC><<<(unsigned) ((h->E + bs - 1) / bs), bs, 0, h->stream>>>(m, u, h->d_uc, h->d_chem_rhs);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// diffusion coefficients, lifting and the viscous volume terms of u
template <int NC>
int launch_visc(charm_gpu_handle_s *h, const double *u, const double *chem_rhs)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nbe = (h->E + bs - 1) / bs;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    if (h->cfg.use_diff && NC >= 2)
        diffcoef_kernel<NC, kNB, double, double><<<(unsigned) nbe, bs, 0, h->stream>>>(m, StIn<double>{u}, h->d_dif);
    if (nbi + nbb) vgrad_face_kernel<NC><<<(unsigned) (nbi + nbb), bs, 0, h->stream>>>(m, u, h->d_dif, h->d_s9, nbi);
    vgrad_cell_kernel<NC><<<(unsigned) nbe, bs, 0, h->stream>>>(m, u, h->d_dif, h->d_s9, h->d_vis);
    vvol_kernel<NC><<<(unsigned) nbe, bs, 0, h->stream>>>(m, u, h->d_vis, chem_rhs, h->d_radd);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// viscous face fluxes, added into the convective slots (after launch_face)
template <int NC>
int launch_vflux(charm_gpu_handle_s *h, const double *u)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    if (nbi + nbb == 0) return CHARM_GPU_OK;
    TimedLaunch t;
    begin_launch(h, 0, &t);
    vflux_face_kernel<NC><<<(unsigned) (nbi + nbb), bs, 0, h->stream>>>(m, u, h->d_vis,
                                                                       static_cast<double *>(h->d_slots), nbi);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <typename T, int NC>
int stage(charm_gpu_handle_s *h, const double *u, const double *u0, double *out, double dt, const double *dt_dev,
          double a_new, double a_old, double *dt_next = nullptr)
{
    int rc;
    const double *radd = nullptr;
    if constexpr (std::is_same<T, double>::value)
        if (h->nb == kNB2) {
            if (h->cfg.limiter == CHARM_GPU_LIM_BJ) {   // cell update -> ua, limiter + combination -> out
                if ((rc = p2_stage<NC>(h, u, nullptr, h->d_ua, dt, dt_dev, 1.0, 0.0, kCellUpdate))) return rc;
                return launch_p2_limit<NC>(h, h->d_ua, u0, out, a_new, a_old);
            }
            return p2_stage<NC>(h, u, u0, out, dt, dt_dev, a_new, a_old, kCellUpdate);
        }
    if constexpr (std::is_same<T, double>::value) {
        if (has_visc_chem(h)) {
            if (h->cfg.n_react) {
                if ((rc = launch_chem<NC>(h, u))) return rc;
                u = h->d_uc;   // the residual and the update act on the state after chemistry
            }
            if (h->cfg.use_visc) {
                if ((rc = launch_visc<NC>(h, u, h->d_chem_rhs))) return rc;
                radd = h->d_radd;
            }
        }
    }
    rc = launch_face<T, NC>(h, u);
    if (rc) return rc;
    if constexpr (std::is_same<T, double>::value)
        if (radd && (rc = launch_vflux<NC>(h, u))) return rc;
    if (h->cfg.limiter == CHARM_GPU_LIM_BJ) {
        rc = launch_cell<T, NC>(h, u, nullptr, h->d_ua, dt, dt_dev, 1.0, 0.0, kCellUpdate, radd);
        if (rc) return rc;
        return launch_limit<NC>(h, h->d_ua, u0, out, a_new, a_old, nullptr, dt_next);
    }
    return launch_cell<T, NC>(h, u, u0, out, dt, dt_dev, a_new, a_old, kCellUpdate, radd, dt_next);
}

// The last stage's kernel also reduces the next step's CFL step (CFL mode,
// FP64 p1): the reference's get_dt of the state this step ends with.
bool fused_cfl(const charm_gpu_handle_s *h)
{
    return h->cfg.dt_mode == CHARM_GPU_DT_CFL && h->cfg.precision != CHARM_GPU_PREC_MIXED && h->nb != kNB2;
}

template <typename T, int NC>
int step_impl(charm_gpu_handle_s *h, double dt, const double *dt_dev)
{
    int rc;
    const bool lim = h->cfg.limiter == CHARM_GPU_LIM_BJ;
    double *next = nullptr;
    if (fused_cfl(h)) {
        const double start = (h->cfg.tau > 0.0) ? h->cfg.tau : 1.0e300;
        CUDA_TRY(cudaMemcpyAsync(h->d_dt_next, &start, sizeof(double), cudaMemcpyHostToDevice, h->stream));
        next = h->d_dt_next;
    }
    if (h->cfg.model == CHARM_GPU_MODEL_EULER) {
        if (lim) rc = stage<T, NC>(h, h->d_u, nullptr, h->d_u, dt, dt_dev, 1.0, 0.0, next);   // cell -> ua, limiter -> u
        else if (!(rc = stage<T, NC>(h, h->d_u, nullptr, h->d_ub, dt, dt_dev, 1.0, 0.0, next)))
            std::swap(h->d_u, h->d_ub);
    } else if (lim) {
        // SSP-RK3 in the reference's order (charm_model.c:259-266).  A stage
        // never writes the buffer it reads its residual from.
        if (!(rc = stage<T, NC>(h, h->d_u, nullptr, h->d_ub, dt, dt_dev, 1.0, 0.0)) &&
            !(rc = stage<T, NC>(h, h->d_ub, h->d_u, h->d_ub, dt, dt_dev, 0.25, 0.75)))
            rc = stage<T, NC>(h, h->d_ub, h->d_u, h->d_u, dt, dt_dev, 2.0 / 3.0, 1.0 / 3.0, next);
    } else {
        if (!(rc = stage<T, NC>(h, h->d_u, nullptr, h->d_ub, dt, dt_dev, 1.0, 0.0)) &&
            !(rc = stage<T, NC>(h, h->d_ub, h->d_u, h->d_ua, dt, dt_dev, 0.25, 0.75)))
            rc = stage<T, NC>(h, h->d_ua, h->d_u, h->d_u, dt, dt_dev, 2.0 / 3.0, 1.0 / 3.0, next);
    }
    h->dt_next_valid = (rc == CHARM_GPU_OK) && next;
    return rc;
}

// ---- mixed form on FP32 hi/lo planes ---------------------------------------

int64_t n_state(const charm_gpu_handle_s *h) { return (int64_t) n_var(h) * h->nb * h->E; }

// hi/lo <- d_u (to_ff) or d_u <- hi/lo of buffer 0
int ff_convert(charm_gpu_handle_s *h, bool to_ff)
{
    const int64_t n = n_state(h);
    const int bs = 256;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    if (to_ff) ff_from_double_kernel<<<(unsigned) ((n + bs - 1) / bs), bs, 0, h->stream>>>(h->d_u, h->d_fh[0], h->d_fl[0], n);
    else ff_to_double_kernel<<<(unsigned) ((n + bs - 1) / bs), bs, 0, h->stream>>>(h->d_fh[0], h->d_fl[0], h->d_u, n);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

struct FFCoef {
    float h, l;
};
FFCoef ff_split(double x)
{
    const float hi = (float) x;
    return {hi, (float) (x - (double) hi)};
}

// One p2 stage of the mixed form on hi/lo buffers: out = a*(in - dt*M^-1*R) +
// b*u0 (u0 < 0: no combination), FP32 residual; chemistry in FP64 on hi + lo
// into d_uc (hi plane, then lo plane).  mode kCellResidual writes R (FP32)
// into the hi plane of out.
template <int NC>
int p2_ff_stage(charm_gpu_handle_s *h, int in, int u0, int out, FFCoef dt, FFCoef a, FFCoef b, int mode)
{
    int rc;
    const float *uh = h->d_fh[in], *ul = h->d_fl[in];
    const float *radd = nullptr;
    const bool upd = mode == kCellUpdate;
    if (h->cfg.model == CHARM_GPU_MODEL_NS) {
        if (upd && h->cfg.n_react) {
            float *ch = reinterpret_cast<float *>(h->d_uc), *cl = ch + n_state(h);
            if ((rc = launch_p2_chem<float, NC>(h, StIn<float>{uh, ul}, StOut<float>{ch, cl}))) return rc;
            uh = ch;
            ul = cl;
        }
        if (h->cfg.use_visc) {
            if ((rc = launch_p2_visc<float, NC>(h, uh, ul, upd ? h->d_chem_rhs : nullptr))) return rc;
            radd = reinterpret_cast<const float *>(h->d_radd);
        }
    }
    if ((rc = launch_p2_face<float, NC>(h, uh))) return rc;
    if (radd && (rc = launch_p2_vflux<float, NC>(h, uh))) return rc;
    P2Upd up{};
    up.mode = mode;
    up.u_lo = ul;
    up.u0_lo = (u0 >= 0) ? h->d_fl[u0] : nullptr;
    up.out_lo = h->d_fl[out];
    up.dt_h = dt.h; up.dt_l = dt.l; up.a_h = a.h; up.a_l = a.l; up.b_h = b.h; up.b_l = b.l;
    return launch_p2_cell<float, NC>(h, uh, (u0 >= 0) ? h->d_fh[u0] : nullptr, h->d_fh[out], up, radd);
}

template <int NC, int FLUX>
int launch_tile_stage(charm_gpu_handle_s *h, int in, int u0, int out, FFCoef dt, const double *dt_dev, FFCoef a,
                      FFCoef b, bool comb)
{
    MeshDev m = mesh_view(h);
    TileDev tl;
    tl.fptr = h->d_tile_fptr;
    tl.rec = h->d_tile_rec;
    tl.hptr = h->d_tile_hptr;
    tl.halo = h->d_tile_halo;
    tl.slot = h->d_tile_slot;
    tl.ncol = h->tile_ncol;
    tl.bulk = (h->E % 4 == 0) ? 1 : 0;
    // the dynamic shared memory limit is a per-device attribute of the kernel
    static int attr_smem[64] = {0};
    const int dev = h->device & 63;
    if ((size_t) attr_smem[dev] < h->tile_smem) {
        // the largest dynamic size: the opt-in limit less the kernel's static shared memory
        int max_optin = 0;
        cudaFuncAttributes fa;
        CUDA_TRY(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
        CUDA_TRY(cudaFuncGetAttributes(&fa, tile_stage_kernel<NC, FLUX>));
        const int dyn = max_optin - (int) fa.sharedSizeBytes;
        CUDA_TRY(cudaFuncSetAttribute(tile_stage_kernel<NC, FLUX>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
        attr_smem[dev] = dyn;
    }
    if ((size_t) attr_smem[dev] < h->tile_smem) return fail(CHARM_GPU_ENOTSUP, "tile stage: shared memory too small");
    const float *u0h = (u0 >= 0) ? h->d_fh[u0] : nullptr, *u0l = (u0 >= 0) ? h->d_fl[u0] : nullptr;
    TimedLaunch t;
    begin_launch(h, 1, &t);
    tile_stage_kernel<NC, FLUX><<<(unsigned) h->n_tiles, kTile, h->tile_smem, h->stream>>>(
        m, tl, h->d_fh[in], h->d_fl[in], u0h, u0l, h->d_fh[out], h->d_fl[out], dt.h, dt.l, dt_dev, a.h, a.l, b.h, b.l,
        comb ? 1 : 0, h->d_err);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_ff_stage(charm_gpu_handle_s *h, int in, int u0, int out, FFCoef dt, const double *dt_dev, FFCoef a, FFCoef b,
                    bool comb)
{
    if (h->tile_smem) {
        switch (h->cfg.flux) {
        case CHARM_GPU_FLUX_LF: return launch_tile_stage<NC, CHARM_GPU_FLUX_LF>(h, in, u0, out, dt, dt_dev, a, b, comb);
        case CHARM_GPU_FLUX_HLLC: return launch_tile_stage<NC, CHARM_GPU_FLUX_HLLC>(h, in, u0, out, dt, dt_dev, a, b, comb);
        case CHARM_GPU_FLUX_CD: return launch_tile_stage<NC, CHARM_GPU_FLUX_CD>(h, in, u0, out, dt, dt_dev, a, b, comb);
        default: return launch_tile_stage<NC, CHARM_GPU_FLUX_GODUNOV>(h, in, u0, out, dt, dt_dev, a, b, comb);
        }
    }
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const unsigned nb = (unsigned) ((h->E + bs - 1) / bs);
    const float *u0h = (u0 >= 0) ? h->d_fh[u0] : nullptr, *u0l = (u0 >= 0) ? h->d_fl[u0] : nullptr;
    TimedLaunch t;
    begin_launch(h, 1, &t);
#define FF_STAGE(FL) ff_stage_kernel<NC, FL><<<nb, bs, 0, h->stream>>>(m, h->d_fh[in], h->d_fl[in], u0h, u0l, \
        h->d_fh[out], h->d_fl[out], dt.h, dt.l, dt_dev, a.h, a.l, b.h, b.l, comb ? 1 : 0, h->d_err)
    switch (h->cfg.flux) {
    case CHARM_GPU_FLUX_LF: FF_STAGE(CHARM_GPU_FLUX_LF); break;
    case CHARM_GPU_FLUX_HLLC: FF_STAGE(CHARM_GPU_FLUX_HLLC); break;
    case CHARM_GPU_FLUX_CD: FF_STAGE(CHARM_GPU_FLUX_CD); break;
    default: FF_STAGE(CHARM_GPU_FLUX_GODUNOV); break;
    }
#undef FF_STAGE
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_ff_limit(charm_gpu_handle_s *h, int in, int u0, int out, FFCoef a, FFCoef b, bool comb)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const float *u0h = (u0 >= 0) ? h->d_fh[u0] : nullptr, *u0l = (u0 >= 0) ? h->d_fl[u0] : nullptr;
    TimedLaunch t;
    begin_launch(h, 2, &t);
    ff_limit_kernel<NC><<<(unsigned) ((h->E + bs - 1) / bs), bs, 0, h->stream>>>(
        m, h->d_fh[in], h->d_fl[in], u0h, u0l, h->d_fh[out], h->d_fl[out], a.h, a.l, b.h, b.l, comb ? 1 : 0);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// one stage of the mixed form: out = a*L(in - dt*M^-1*R(in)) + b*u0
template <int NC>
int ff_stage(charm_gpu_handle_s *h, int in, int u0, int out, FFCoef dt, const double *dt_dev, FFCoef a, FFCoef b,
             bool comb)
{
    const FFCoef one = {1.f, 0.f}, zero = {0.f, 0.f};
    int rc;
    if (h->nb == kNB2) return p2_ff_stage<NC>(h, in, comb ? u0 : -1, out, dt, a, b, kCellUpdate);   // fixed dt only
    if (h->cfg.limiter == CHARM_GPU_LIM_BJ) {
        // ua (1) holds the updated stage value before the limiter
        if ((rc = launch_ff_stage<NC>(h, in, -1, 1, dt, dt_dev, one, zero, false))) return rc;
        return launch_ff_limit<NC>(h, 1, u0, out, a, b, comb);
    }
    return launch_ff_stage<NC>(h, in, u0, out, dt, dt_dev, a, b, comb);
}

// buffers: 0 = u, 1 = ua, 2 = ub (same roles as the FP64 path)
template <int NC>
int ff_step_impl(charm_gpu_handle_s *h, double dt, const double *dt_dev)
{
    int rc;
    const FFCoef d = ff_split(dt), one = {1.f, 0.f}, zero = {0.f, 0.f};
    const FFCoef q1 = {0.25f, 0.f}, q3 = {0.75f, 0.f}, t2 = ff_split(2.0 / 3.0), t1 = ff_split(1.0 / 3.0);
    const bool lim = h->cfg.limiter == CHARM_GPU_LIM_BJ;
    if (h->cfg.model == CHARM_GPU_MODEL_EULER) {
        if (lim) return ff_stage<NC>(h, 0, -1, 0, d, dt_dev, one, zero, false);
        if ((rc = ff_stage<NC>(h, 0, -1, 2, d, dt_dev, one, zero, false))) return rc;
        std::swap(h->d_fh[0], h->d_fh[2]);
        std::swap(h->d_fl[0], h->d_fl[2]);
        return CHARM_GPU_OK;
    }
    if (lim) {
        if ((rc = ff_stage<NC>(h, 0, -1, 2, d, dt_dev, one, zero, false))) return rc;
        if ((rc = ff_stage<NC>(h, 2, 0, 2, d, dt_dev, q1, q3, true))) return rc;
        return ff_stage<NC>(h, 2, 0, 0, d, dt_dev, t2, t1, true);
    }
    if ((rc = ff_stage<NC>(h, 0, -1, 2, d, dt_dev, one, zero, false))) return rc;
    if ((rc = ff_stage<NC>(h, 2, 0, 1, d, dt_dev, q1, q3, true))) return rc;
    return ff_stage<NC>(h, 1, 0, 0, d, dt_dev, t2, t1, true);
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
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED) {
        switch (h->cfg.n_comp) {
        case 1: return ff_step_impl<1>(h, dt, dt_dev);
        case 2: return ff_step_impl<2>(h, dt, dt_dev);
        default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
        }
    }
    if (h->cfg.precision == CHARM_GPU_PREC_DW) return step_dispatch_t<dw>(h, dt, dt_dev);
    return step_dispatch_t<double>(h, dt, dt_dev);
}

int cfl_dispatch(charm_gpu_handle_s *h)
{
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED) {
        int rc = ff_convert(h, false);
        if (rc) return rc;
    }
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
    if (dt_in > 0) { *dt = dt_in; h->dt_next_valid = false; return CHARM_GPU_OK; }
    if (h->cfg.dt_mode == CHARM_GPU_DT_TAU) { *dt = h->cfg.tau; return CHARM_GPU_OK; }
    if (h->dt_next_valid) {
        // reduced by the last stage of the previous step from this state
        std::swap(h->d_dt, h->d_dt_next);
        h->dt_next_valid = false;
        *dt = 0.0;
        *dt_dev = h->d_dt;
        return CHARM_GPU_OK;
    }
    int rc = cfl_dispatch(h);
    if (rc) return rc;
    *dt = 0.0;
    *dt_dev = h->d_dt;
    return CHARM_GPU_OK;
}

// fn(lo, hi) over [0, n) on the host octree's worker pool (persistent
// threads; serial below its minimum chunk)
template <typename Fn>
void host_for(int64_t n, int64_t min_chunk, Fn &&fn)
{
    if (n <= 0) return;
    using F = typename std::remove_reference<Fn>::type;
    charm_forest_parallel_for_min(
        n, min_chunk, [](void *c, int64_t lo, int64_t hi) { (*static_cast<F *>(c))(lo, hi); }, (void *) &fn);
}

// the first error of a parallel check (code and a static message)
struct UploadError {
    int code = 0;
    const char *msg = "";
    bool set() const { return __atomic_load_n(&code, __ATOMIC_RELAXED) != 0; }
    void raise(int c, const char *m)
    {
        int expect = 0;
        if (__atomic_compare_exchange_n(&code, &expect, c, false, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED)) msg = m;
    }
};

// The state and stage buffers a step reads and writes (a step may swap them)
std::vector<void *> step_buffers(const charm_gpu_handle_s *h)
{
    return {h->d_u, h->d_ua, h->d_ub, h->d_fh[0], h->d_fh[1], h->d_fh[2], h->d_fl[0], h->d_fl[1], h->d_fl[2],
            h->d_slots, h->d_uc};
}

// Back-to-back steps with a fixed dt (given, or TAU) as a CUDA graph: two
// steps are captured once (a step that swaps its state buffers has swapped
// them back after two), kept for later runs with the same dt, buffers and
// stream, and replayed nsteps / 2 times; *done gets the steps launched.
// Not used when kernels are being timed one by one, when the error word is
// checked every few steps, or in CFL mode (the step then reads and swaps a
// device-side dt); a capture the driver refuses falls back to launches.
int run_as_graph(charm_gpu_handle_s *h, int nsteps, double dt_in, int *done)
{
    *done = 0;
    const bool fixed_dt = dt_in > 0.0 || h->cfg.dt_mode == CHARM_GPU_DT_TAU;
    if (nsteps < 4 || !fixed_dt || h->timing || h->cfg.check_every > 0) return CHARM_GPU_OK;
    const double dt = dt_in > 0.0 ? dt_in : h->cfg.tau;
    const std::vector<void *> bufs = step_buffers(h);
    if (!(h->run_graph && h->run_graph_dt == dt && h->run_graph_stream == h->stream && h->run_graph_bufs == bufs)) {
        drop_run_graph(h);
        int64_t l0[4];
        std::memcpy(l0, h->launches, sizeof(l0));
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return CHARM_GPU_OK;
        }
        int rc = 0;
        for (int s = 0; s < 2 && !rc; s++) {
            double d;
            const double *dd;
            if (!(rc = resolve_dt(h, dt, &d, &dd))) rc = step_dispatch(h, d, dd);
        }
        const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
        cudaGraphExec_t ge = nullptr;
        const bool ok = !rc && ec == cudaSuccess && g && step_buffers(h) == bufs &&
                        cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();   // a refused capture leaves no sticky error
        for (int k = 0; k < 4; k++) h->run_graph_launches[k] = h->launches[k] - l0[k];
        std::memcpy(h->launches, l0, sizeof(l0));   // nothing ran during the capture
        if (!ok) {
            // restore the buffers a captured step may have swapped
            h->d_u = (double *) bufs[0]; h->d_ua = (double *) bufs[1]; h->d_ub = (double *) bufs[2];
            for (int k = 0; k < 3; k++) { h->d_fh[k] = (float *) bufs[3 + k]; h->d_fl[k] = (float *) bufs[6 + k]; }
            if (ge) cudaGraphExecDestroy(ge);
            return CHARM_GPU_OK;
        }
        h->run_graph = ge;
        h->run_graph_dt = dt;
        h->run_graph_stream = h->stream;
        h->run_graph_bufs = bufs;
    }
    h->dt_next_valid = false;
    for (int i = 0; i + 2 <= nsteps; i += 2) {
        CUDA_TRY(cudaGraphLaunch(h->run_graph, h->stream));
        for (int k = 0; k < 4; k++) h->launches[k] += h->run_graph_launches[k];
        *done += 2;
    }
    return CHARM_GPU_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================

extern "C" {

const char *charm_gpu_version(void) { return "charm_gpu 0.1 (sm_103a)"; }
const char *charm_gpu_last_error(void) { return g_last_error.c_str(); }

// the message of charm_gpu_last_error() for the host C code (case reader)
void charm_internal_set_error(const char *msg) { g_last_error = msg ? msg : ""; }

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
    h->nb = (cfg->p_order == 2) ? kNB2 : CHARM_GPU_BASIS;
    build_devcfg(cfg, &h->dcfg);
    if (h->nb == kNB2 && upload_p2_tables(h) != CHARM_GPU_OK) {
        delete h;
        return CHARM_GPU_ECUDA;
    }
    if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(CHARM_GPU_ECUDA, "cudaStreamCreate failed");
    }
    h->stream = h->own_stream;
    if (cudaMalloc(&h->d_err, sizeof(unsigned)) != cudaSuccess || cudaMalloc(&h->d_dt, sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->d_dt_next, sizeof(double)) != cudaSuccess) {
        if (h->d_err) cudaFree(h->d_err);
        if (h->d_dt) cudaFree(h->d_dt);
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
    if (h->d_dt_next) cudaFree(h->d_dt_next);
    for (auto e : h->event_pool) cudaEventDestroy(e);
    {
        // the stream is idle: nothing queued reads c_cfg for this handle
        CfgLease lease(h);
        CfgSlot &s = cfg_slot(h->device);
        if (s.owner == h) s.owner = nullptr;
        if (s.live && s.stream == h->stream) s.live = false;
    }
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return CHARM_GPU_OK;
}

namespace {
// The upload of charm_gpu_upload_mesh; with hexff (general hexahedra: the
// face numbers of both sides of every interior record) the element faces
// that the records claim come from there instead of the box's dir bits.
int upload_impl(charm_gpu_handle_t h, const charm_gpu_mesh_t *mesh, const int8_t *hexff)
{
    if (!h || !mesh) return fail(CHARM_GPU_EINVAL, "null argument");
    const int64_t E = mesh->n_elem, F = mesh->n_face, Fb = mesh->n_bface;
    if (E <= 0 || F < 0 || Fb < 0) return fail(CHARM_GPU_EINVAL, "bad mesh sizes");
    if (E >= (int64_t) INT32_MAX) return fail(CHARM_GPU_EINVAL, "too many elements for int32 indices");
    if (!mesh->center || !mesh->level || (F && (!mesh->face_elem || !mesh->face_info)) ||
        (Fb && (!mesh->bface_elem || !mesh->bface_face || !mesh->bface_bnd)))
        return fail(CHARM_GPU_EINVAL, "null mesh array");
    // ---- validate indices and build the element tables on the host, on the
    // host octree's worker threads (the loops touch every face record and
    // element; serially they were most of an adapt's upload) ----
    std::vector<int32_t> cnt(E + 1, 0);
    std::vector<int32_t> lim_idx(6 * E, -1);
    std::vector<int8_t> lim_kind(6 * E, -1);
    UploadError uerr;
    // each element face takes exactly one record (the big side of a mortar:
    // its first sub-face record); a second claim is an error
    auto claim = [&](int f, int32_t e, int8_t k, int32_t idx) {
        int32_t expect = -1;
        if (!__atomic_compare_exchange_n(&lim_idx[(int64_t) f * E + e], &expect, idx, false, __ATOMIC_RELAXED,
                                         __ATOMIC_RELAXED))
            return false;
        lim_kind[(int64_t) f * E + e] = k;
        return true;
    };
    host_for(F, 4096, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi && !uerr.set(); i++) {
            const int32_t a = mesh->face_elem[i], b = mesh->face_elem[F + i];
            const unsigned info = mesh->face_info[i];
            const int d = info & 3, kind = (info >> 2) & 3;
            if (a < 0 || a >= E || b < 0 || b >= E || d > 2 || kind > 2) {
                uerr.raise(CHARM_GPU_EINVAL, "face record out of range");
                return;
            }
            if (kind && h->nb != CHARM_GPU_BASIS) { uerr.raise(CHARM_GPU_ENOTSUP, "p2: conforming meshes only"); return; }
            __atomic_fetch_add(&cnt[a], 1, __ATOMIC_RELAXED);
            __atomic_fetch_add(&cnt[b], 1, __ATOMIC_RELAXED);
            const int fa = hexff ? hexff[i] : 2 * d + 1, fb = hexff ? hexff[F + i] : 2 * d;   // side 0 / side 1
            if (fa < 0 || fa > 5 || fb < 0 || fb > 5) { uerr.raise(CHARM_GPU_EINVAL, "face number out of range"); return; }
            if (kind == 0) {
                if (!claim(fa, a, 0, b) || !claim(fb, b, 0, a)) {
                    uerr.raise(CHARM_GPU_EINVAL, "element face with more than one face record");
                    return;
                }
                continue;
            }
            const int sub = (info >> 4) & 3;
            const int32_t small = (kind == 1) ? a : b, big = (kind == 1) ? b : a;
            const int fs = (kind == 1) ? fa : fb, fbig = (kind == 1) ? fb : fa;
            if (!claim(fs, small, (int8_t) (3 | (sub << 4)), big)) {
                uerr.raise(CHARM_GPU_EINVAL, "element face with more than one face record");
                return;
            }
            if (sub == 0) {
                // the 4 sub-faces of one big face must be consecutive records
                if (i + 3 >= F) { uerr.raise(CHARM_GPU_EINVAL, "incomplete mortar"); return; }
                for (int k = 1; k < 4; k++) {
                    const unsigned ik = mesh->face_info[i + k];
                    const int32_t bigk = (((ik >> 2) & 3) == 1) ? mesh->face_elem[F + i + k] : mesh->face_elem[i + k];
                    if (((ik >> 4) & 3) != (unsigned) k || bigk != big || (ik & 3) != (unsigned) d ||
                        ((ik >> 2) & 3) != (unsigned) kind) {
                        uerr.raise(CHARM_GPU_EINVAL, "mortar sub-faces not consecutive");
                        return;
                    }
                }
                if (!claim(fbig, big, 2, (int32_t) i)) {
                    uerr.raise(CHARM_GPU_EINVAL, "element face with more than one face record");
                    return;
                }
            }
        }
    });
    if (uerr.set()) return fail(uerr.code, uerr.msg);
    host_for(Fb, 4096, [&](int64_t lo, int64_t hi) {
        for (int64_t j = lo; j < hi && !uerr.set(); j++) {
            const int32_t e = mesh->bface_elem[j];
            const int f = mesh->bface_face[j], bnd = mesh->bface_bnd[j];
            if (e < 0 || e >= E || f < 0 || f > 5 || bnd < 0 || bnd >= h->cfg.n_bnd) {
                uerr.raise(CHARM_GPU_EINVAL, "boundary face record out of range");
                return;
            }
            __atomic_fetch_add(&cnt[e], 1, __ATOMIC_RELAXED);
            if (!claim(f, e, 1, (int32_t) j)) {
                uerr.raise(CHARM_GPU_EINVAL, "element face with more than one face record");
                return;
            }
        }
    });
    if (uerr.set()) return fail(uerr.code, uerr.msg);
    host_for(6 * E, 16384, [&](int64_t lo, int64_t hi) {
        for (int64_t k = lo; k < hi; k++)
            if (lim_idx[k] < 0) { uerr.raise(CHARM_GPU_EINVAL, "element face without a face record"); return; }
    });
    if (uerr.set()) return fail(uerr.code, uerr.msg);
    std::vector<int32_t> ptr(E + 1, 0);
    for (int64_t e = 0; e < E; e++) ptr[e + 1] = ptr[e] + cnt[e];
    // the element-owned gather: every element's slots in increasing slot
    // order (interior sides 2i, 2i+1 by face, then boundary 2F + j), the
    // order in which the cell kernels add them
    std::vector<int32_t> slot(ptr[E] > 0 ? ptr[E] : 1);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    host_for(F, 4096, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; i++) {
            slot[__atomic_fetch_add(&fill[mesh->face_elem[i]], 1, __ATOMIC_RELAXED)] = (int32_t) (2 * i);
            slot[__atomic_fetch_add(&fill[mesh->face_elem[F + i]], 1, __ATOMIC_RELAXED)] = (int32_t) (2 * i + 1);
        }
    });
    host_for(Fb, 4096, [&](int64_t lo, int64_t hi) {
        for (int64_t j = lo; j < hi; j++)
            slot[__atomic_fetch_add(&fill[mesh->bface_elem[j]], 1, __ATOMIC_RELAXED)] = (int32_t) (2 * F + j);
    });
    host_for(E, 4096, [&](int64_t lo, int64_t hi) {
        for (int64_t e = lo; e < hi; e++) std::sort(slot.begin() + ptr[e], slot.begin() + ptr[e + 1]);
    });
    int64_t S = 2 * F + Fb;
    S += (S & 1);

    CUDA_TRY(cudaSetDevice(h->device));
    cudaStreamSynchronize(h->stream);
    reset_mesh(h);
    int arc;
    const int V = n_var(h);
    const size_t st = (size_t) V * h->nb * E * sizeof(double);
    const size_t sl = (size_t) V * h->nb * (S > 0 ? S : 2) *
                      (h->cfg.precision == CHARM_GPU_PREC_MIXED ? sizeof(float) : sizeof(double));
    if ((arc = ensure_buf(h, &h->d_center, 3 * E * sizeof(double)))) return arc;
    if ((arc = ensure_buf(h, &h->d_level, E))) return arc;
    if ((arc = ensure_buf(h, &h->d_face_elem, 2 * (F ? F : 1) * sizeof(int32_t)))) return arc;
    if ((arc = ensure_buf(h, &h->d_face_info, F ? F : 1))) return arc;
    if ((arc = ensure_buf(h, &h->d_bface_elem, (Fb ? Fb : 1) * sizeof(int32_t)))) return arc;
    if ((arc = ensure_buf(h, &h->d_bface_face, Fb ? Fb : 1))) return arc;
    if ((arc = ensure_buf(h, &h->d_bface_bnd, Fb ? Fb : 1))) return arc;
    if ((arc = ensure_buf(h, &h->d_gather_ptr, (E + 1) * sizeof(int32_t)))) return arc;
    if ((arc = ensure_buf(h, &h->d_gather_slot, (ptr[E] ? ptr[E] : 1) * sizeof(int32_t)))) return arc;
    if ((arc = ensure_buf(h, &h->d_lim_idx, 6 * E * sizeof(int32_t)))) return arc;
    if ((arc = ensure_buf(h, &h->d_lim_kind, 6 * E))) return arc;
    if ((arc = ensure_buf(h, &h->d_u, st))) return arc;
    if ((arc = ensure_buf(h, &h->d_ua, st))) return arc;
    if ((arc = ensure_buf(h, &h->d_ub, st))) return arc;
    if ((arc = ensure_buf(h, &h->d_slots, sl))) return arc;
    if (h->cfg.model == CHARM_GPU_MODEL_NS && (h->cfg.use_visc || h->cfg.n_react)) {
        if ((arc = ensure_buf(h, &h->d_chem_rhs, sizeof(double) * E))) return arc;
        CUDA_TRY(cudaMemset(h->d_chem_rhs, 0, sizeof(double) * E));
        if (h->cfg.n_react) if ((arc = ensure_buf(h, &h->d_uc, st))) return arc;
        if (h->cfg.use_visc) {
            if ((arc = ensure_buf(h, &h->d_s9, sizeof(double) * 9 * h->nb * S))) return arc;
            if ((arc = ensure_buf(h, &h->d_vis, sizeof(double) * 9 * h->nb * E))) return arc;
            if ((arc = ensure_buf(h, &h->d_radd, sizeof(double) * 4 * h->nb * E))) return arc;
            if ((arc = ensure_buf(h, &h->d_dif, sizeof(double) * V * E))) return arc;
            CUDA_TRY(cudaMemset(h->d_dif, 0, sizeof(double) * V * E));
        }
    }
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED) {
        for (int k = 0; k < 3; k++) {
            if ((arc = ensure_buf(h, &h->d_fh[k], st / 2))) return arc;
            if ((arc = ensure_buf(h, &h->d_fl[k], st / 2))) return arc;
            CUDA_TRY(cudaMemset(h->d_fh[k], 0, st / 2));
            CUDA_TRY(cudaMemset(h->d_fl[k], 0, st / 2));
        }
        // tiles of kTile consecutive elements: every face touching a tile, in
        // global face order (keeps the 4 records of a mortar consecutive),
        // as records with the shared-memory columns of both sides; the
        // tile's halo (outside elements that share one of its faces); for
        // every element face its record position and kind
        const int64_t nt = (E + kTile - 1) / kTile;
        // a tile's records: every record of its elements (from their gather
        // slots), sorted (interior faces by index, then boundary records as
        // F + j: the 4 records of a mortar stay consecutive), each once; its
        // halo: the outside elements of those records, sorted
        auto rec_of = [&](int32_t sl) -> int32_t { return sl < 2 * F ? sl >> 1 : (int32_t) (F + (sl - 2 * F)); };
        auto tile_lists = [&](int64_t t, std::vector<int32_t> &list, std::vector<int32_t> &hl) {
            const int64_t e0 = t * kTile, e1 = std::min<int64_t>(E, e0 + kTile);
            list.clear();
            hl.clear();
            for (int64_t e = e0; e < e1; e++)
                for (int32_t j = ptr[e]; j < ptr[e + 1]; j++) list.push_back(rec_of(slot[j]));
            std::sort(list.begin(), list.end());
            list.erase(std::unique(list.begin(), list.end()), list.end());
            for (const int32_t r : list) {
                if (r >= F) continue;   // a boundary record's element is in the tile
                for (int side = 0; side < 2; side++) {
                    const int32_t e = mesh->face_elem[side * F + r];
                    if (e < e0 || e >= e1) hl.push_back(e);
                }
            }
            std::sort(hl.begin(), hl.end());
            hl.erase(std::unique(hl.begin(), hl.end()), hl.end());
        };
        // each tile's lists once, kept for the fill below
        std::vector<int32_t> tptr(nt + 1, 0), hptr(nt + 1, 0);
        std::vector<std::vector<int32_t>> lists((size_t) nt), halos((size_t) nt);
        host_for(nt, 64, [&](int64_t lo, int64_t hi) {
            for (int64_t t = lo; t < hi; t++) {
                tile_lists(t, lists[t], halos[t]);
                tptr[t + 1] = (int32_t) lists[t].size();
                hptr[t + 1] = (int32_t) halos[t].size();
            }
        });
        int64_t max_list = 0, max_halo = 0;
        for (int64_t t = 0; t < nt; t++) {
            max_list = std::max<int64_t>(max_list, tptr[t + 1]);
            max_halo = std::max<int64_t>(max_halo, hptr[t + 1]);
            tptr[t + 1] += tptr[t];
            hptr[t + 1] += hptr[t];
        }
        std::vector<int4> trec(tptr[nt] > 0 ? tptr[nt] : 1);
        std::vector<int32_t> tslot(6 * E, -1), halo(hptr[nt] > 0 ? hptr[nt] : 1, 0);
        host_for(nt, 64, [&](int64_t lo, int64_t hi) {
            for (int64_t t = lo; t < hi; t++) {
                const std::vector<int32_t> &list = lists[t], &hl = halos[t];
                const int64_t e0 = t * kTile, e1 = std::min<int64_t>(E, e0 + kTile);
                std::copy(hl.begin(), hl.end(), halo.begin() + hptr[t]);
                auto column = [&](int32_t e) -> int32_t {
                    if (e >= e0 && e < e1) return (int32_t) (e - e0);
                    return kTile + (int32_t) (std::lower_bound(hl.begin(), hl.end(), e) - hl.begin());
                };
                for (size_t loc = 0; loc < list.size(); loc++) {
                    const int32_t r = list[loc];
                    int4 rec;
                    if (r < F) {
                        const int32_t a = mesh->face_elem[r], b = mesh->face_elem[F + r];
                        const unsigned info = mesh->face_info[r];
                        const int d = info & 3, kind = (info >> 2) & 3, sub = (info >> 4) & 3;
                        rec.x = column(a);
                        rec.y = column(b);
                        rec.z = (int) info;
                        rec.w = mesh->level[(kind == 2) ? b : a];
                        for (int side = 0; side < 2; side++) {
                            const int32_t e = side ? b : a;
                            if (e < e0 || e >= e1) continue;
                            const int f = side ? 2 * d : 2 * d + 1;
                            const bool big = (kind == 1 && side == 1) || (kind == 2 && side == 0);
                            const bool small = (kind == 1 && side == 0) || (kind == 2 && side == 1);
                            if (!big) tslot[(int64_t) f * E + e] = ((int32_t) loc << 2) | (small ? 3 : 0);
                            else if (sub == 0) tslot[(int64_t) f * E + e] = ((int32_t) loc << 2) | 2;
                        }
                    } else {
                        const int64_t j = r - F;
                        const int32_t e = mesh->bface_elem[j];
                        rec.x = column(e);
                        rec.y = -1;
                        rec.z = (int) mesh->bface_face[j] | ((int) mesh->bface_bnd[j] << 8) | kRecBoundary;
                        rec.w = mesh->level[e];
                        tslot[(int64_t) mesh->bface_face[j] * E + e] = ((int32_t) loc << 2) | 1;
                    }
                    trec[tptr[t] + loc] = rec;
                }
            }
        });
        host_for(6 * E, 16384, [&](int64_t lo, int64_t hi) {
            for (int64_t k = lo; k < hi; k++)
                if (tslot[k] < 0) { uerr.raise(CHARM_GPU_EINVAL, "element face without a tile face slot"); return; }
        });
        if (uerr.set()) return fail(uerr.code, uerr.msg);
        if (halo.empty()) halo.push_back(0);
        const int ncol = (int) ((kTile + max_halo + 3) & ~(int64_t) 3);   // 16-byte aligned planes
        const size_t smem = sizeof(float) * ((size_t) V * CHARM_GPU_BASIS * ncol + (size_t) max_list * 3 * V);
        int max_optin = 0;
        CUDA_TRY(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
        if (smem + 1024 <= (size_t) max_optin) {   // 1 KB left for the kernel's static shared memory
            if ((arc = ensure_buf(h, &h->d_tile_fptr, (nt + 1) * sizeof(int32_t)))) return arc;
            if ((arc = ensure_buf(h, &h->d_tile_rec, trec.size() * sizeof(int4)))) return arc;
            if ((arc = ensure_buf(h, &h->d_tile_slot, (size_t) 6 * E * sizeof(int32_t)))) return arc;
            if ((arc = ensure_buf(h, &h->d_tile_hptr, (nt + 1) * sizeof(int32_t)))) return arc;
            if ((arc = ensure_buf(h, &h->d_tile_halo, halo.size() * sizeof(int32_t)))) return arc;
            CUDA_TRY(cudaMemcpy(h->d_tile_fptr, tptr.data(), (nt + 1) * sizeof(int32_t), cudaMemcpyHostToDevice));
            CUDA_TRY(cudaMemcpy(h->d_tile_rec, trec.data(), trec.size() * sizeof(int4), cudaMemcpyHostToDevice));
            CUDA_TRY(cudaMemcpy(h->d_tile_slot, tslot.data(), (size_t) 6 * E * sizeof(int32_t), cudaMemcpyHostToDevice));
            CUDA_TRY(cudaMemcpy(h->d_tile_hptr, hptr.data(), (nt + 1) * sizeof(int32_t), cudaMemcpyHostToDevice));
            CUDA_TRY(cudaMemcpy(h->d_tile_halo, halo.data(), halo.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
            h->n_tiles = nt;
            h->tile_smem = smem;
            h->tile_ncol = ncol;
        }
    }
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

// Jacobian of the trilinear map at the 8 Gauss points of every element, on
// the host, before anything changes (the same map as hex_map in dg_hex.cuh).
bool hex_jacobians_positive(const double *vert, int64_t E)
{
    const double s3 = 0.57735026918962576451;
    for (int64_t e = 0; e < E; e++)
        for (int q = 0; q < 8; q++) {
            const double r[3] = {(q & 1) ? s3 : -s3, (q & 2) ? s3 : -s3, (q & 4) ? s3 : -s3};
            double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int k = 0; k < 8; k++) {
                const double sx = (k & 1) ? 1.0 : -1.0, sy = (k & 2) ? 1.0 : -1.0, sz = (k & 4) ? 1.0 : -1.0;
                const double wx = 1.0 + sx * r[0], wy = 1.0 + sy * r[1], wz = 1.0 + sz * r[2];
                for (int d = 0; d < 3; d++) {
                    const double v = vert[(int64_t) (3 * k + d) * E + e];
                    J[d][0] += wz * wy * sx * 0.125 * v;
                    J[d][1] += wz * wx * sy * 0.125 * v;
                    J[d][2] += wy * wx * sz * 0.125 * v;
                }
            }
            const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
            if (!(det > 0.0)) return false;
        }
    return true;
}
}  // namespace

int charm_gpu_upload_mesh(charm_gpu_handle_t h, const charm_gpu_mesh_t *mesh)
{
    return upload_impl(h, mesh, nullptr);
}

int charm_gpu_upload_mesh_hex(charm_gpu_handle_t h, const charm_gpu_mesh_t *mesh, const charm_gpu_hex_t *hex)
{
    if (!h || !mesh || !hex || !hex->vertex || (mesh->n_face > 0 && !hex->face_face))
        return fail(CHARM_GPU_EINVAL, "null argument");
    if (h->cfg.precision != CHARM_GPU_PREC_FP64 || h->nb != CHARM_GPU_BASIS)
        return fail(CHARM_GPU_ENOTSUP, "general hexahedra: FP64, p1");
    if (h->cfg.model == CHARM_GPU_MODEL_NS && (h->cfg.use_visc || h->cfg.n_react))
        return fail(CHARM_GPU_ENOTSUP, "general hexahedra: convective terms only");
    if (mesh->n_elem > 0 && mesh->n_elem < (int64_t) INT32_MAX && !hex_jacobians_positive(hex->vertex, mesh->n_elem))
        return fail(CHARM_GPU_EINVAL, "element with a non-positive Jacobian");
    int rc = upload_impl(h, mesh, hex->face_face);
    if (rc) return rc;
    const int64_t E = h->E, F = h->F, NR = h->F + h->Fb;
    int arc;
    if ((arc = ensure_buf(h, &h->d_hex_vert, 24 * E * sizeof(double))) ||
        (arc = ensure_buf(h, &h->d_hex_g, (size_t) kHexG * E * sizeof(double))) ||
        (arc = ensure_buf(h, &h->d_hex_fg, (size_t) kHexF * (NR ? NR : 1) * sizeof(double))) ||
        (arc = ensure_buf(h, &h->d_hex_ff, 2 * (F ? F : 1)))) {
        h->mesh_ready = false;
        return arc;
    }
    CUDA_TRY(cudaMemcpy(h->d_hex_vert, hex->vertex, 24 * E * sizeof(double), cudaMemcpyHostToDevice));
    if (F) CUDA_TRY(cudaMemcpy(h->d_hex_ff, hex->face_face, 2 * F, cudaMemcpyHostToDevice));
    HexDev x = hex_view(h);
    CUDA_TRY(cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), h->stream));
    CUDA_TRY(hex_launch_geom(mesh_view(h), x, h->d_hex_g, h->d_hex_fg, h->d_err, h->stream));
    unsigned err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, h->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (err) {
        h->mesh_ready = false;
        return fail(CHARM_GPU_EINVAL, "element with a non-positive Jacobian");
    }
    h->hex = true;
    return CHARM_GPU_OK;
}

// ---- adapt with the state on the device ------------------------------------

// rho[e] = sum of the species' coefficient-0 planes (0 + s_0 + s_1 ..., the
// host criterion's order)
__global__ void __launch_bounds__(256) density_means_kernel(const double *__restrict__ u, int64_t E, int nb, int nc,
                                                            double *__restrict__ rho)
{
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double r = 0.0;
    for (int s = 0; s < nc; s++) r += u[(int64_t) ((4 + s) * nb) * E + e];
    rho[e] = r;
}

// One pass of an adapt plan (charm_gpu_adapt_plan_t): output leaf k of the
// state [V][4][Eo] from the input state [V][4][Ei].  The parent <-> child
// projections of charm_replace_quads (src/charm_amr.c:206-307) with the
// operations, and their order, of the host octree's project_down /
// project_up, rounded one by one (no contraction into FMA): the result is
// the host's, bit for bit.
__global__ void __launch_bounds__(256) adapt_project_kernel(const double *__restrict__ src, int64_t Ei,
                                                            double *__restrict__ dst, int64_t Eo,
                                                            const int32_t *__restrict__ map, int V)
{
    const int64_t k = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Eo) return;
    const int64_t s = map[2 * k];
    const int op = map[2 * k + 1];
    for (int v = 0; v < V; v++) {
        const double *P = src + (int64_t) v * 4 * Ei;
        double *Cn = dst + (int64_t) v * 4 * Eo;
        if (op < 0) {
            for (int b = 0; b < 4; b++) Cn[(int64_t) b * Eo + k] = P[(int64_t) b * Ei + s];
        } else if (op < 8) {
            const double o0 = (op & 1) ? 0.25 : -0.25, o1 = (op & 2) ? 0.25 : -0.25, o2 = (op & 4) ? 0.25 : -0.25;
            double x = __dadd_rn(P[s], __dmul_rn(o0, P[Ei + s]));
            x = __dadd_rn(x, __dmul_rn(o1, P[2 * Ei + s]));
            x = __dadd_rn(x, __dmul_rn(o2, P[3 * Ei + s]));
            Cn[k] = x;
            for (int b = 1; b < 4; b++) Cn[(int64_t) b * Eo + k] = __dmul_rn(0.5, P[(int64_t) b * Ei + s]);
        } else {
            double m = 0.0, sk[3] = {0.0, 0.0, 0.0};
            for (int i = 0; i < 8; i++) {
                const double c0 = P[s + i];
                m = __dadd_rn(m, c0);
                for (int d = 0; d < 3; d++) {
                    const double sg = ((i >> d) & 1) ? 0.375 : -0.375;
                    sk[d] = __dadd_rn(sk[d], __dadd_rn(__dmul_rn(sg, c0),
                                                       __dmul_rn(P[(int64_t) (d + 1) * Ei + s + i], 1. / 16.)));
                }
            }
            Cn[k] = __dmul_rn(m, 0.125);
            for (int d = 0; d < 3; d++) Cn[(int64_t) (d + 1) * Eo + k] = sk[d];
        }
    }
}

int charm_gpu_cell_fields(charm_gpu_handle_t h, double *out)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (!out) return fail(CHARM_GPU_EINVAL, "null argument");
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED && (rc = ff_convert(h, false))) return rc;   // d_u <- hi + lo
    const int nf = 8 + h->cfg.n_comp;
    if ((rc = ensure_buf(h, &h->d_proj[1], sizeof(double) * (size_t) nf * h->E))) return rc;
    const unsigned nb = (unsigned) ((h->E + 255) / 256);
    if (h->cfg.n_comp == 1) cell_fields_kernel<1><<<nb, 256, 0, h->stream>>>(h->d_u, h->E, h->nb, h->d_proj[1]);
    else cell_fields_kernel<2><<<nb, 256, 0, h->stream>>>(h->d_u, h->E, h->nb, h->d_proj[1]);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, h->d_proj[1], sizeof(double) * (size_t) nf * h->E, cudaMemcpyDeviceToHost,
                             h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_density_means(charm_gpu_handle_t h, double *rho)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (!rho) return fail(CHARM_GPU_EINVAL, "null argument");
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED && (rc = ff_convert(h, false))) return rc;   // d_u <- hi + lo
    if ((rc = ensure_buf(h, &h->d_proj[0], sizeof(double) * (size_t) h->E))) return rc;
    density_means_kernel<<<(unsigned) ((h->E + 255) / 256), 256, 0, h->stream>>>(h->d_u, h->E, h->nb, h->cfg.n_comp,
                                                                                  h->d_proj[0]);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(rho, h->d_proj[0], sizeof(double) * (size_t) h->E, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_refine_flags_relative(charm_gpu_handle_t h, double threshold, int per_cell, int8_t *flags,
                                    double *grad_out)
{
    if (!h || !flags) return fail(CHARM_GPU_EINVAL, "null argument");
    if (!(threshold > 0.0)) return fail(CHARM_GPU_EINVAL, "threshold must be positive");
    if (!h->mesh_ready) return fail(CHARM_GPU_ESTATE, "no mesh uploaded");
    const int64_t E = h->E;
    std::vector<double> g(grad_out ? 0 : (size_t) (3 * E)), rho((size_t) E), vol((size_t) E);
    double *hg = grad_out ? grad_out : g.data();
    int rc = charm_gpu_refine_flags(h, 1.0, nullptr, hg);   // the gradient estimate of charm_adapt
    if (!rc) rc = charm_gpu_density_means(h, rho.data());
    if (rc) return rc;
    if (per_cell) {
        CUDA_TRY(cudaSetDevice(h->device));
        if (h->hex) {
            CUDA_TRY(cudaMemcpy(vol.data(), h->d_hex_g + (size_t) kGvol * E, sizeof(double) * E, cudaMemcpyDeviceToHost));
        } else {
            std::vector<int8_t> lev((size_t) E);
            CUDA_TRY(cudaMemcpy(lev.data(), h->d_level, (size_t) E, cudaMemcpyDeviceToHost));
            for (int64_t e = 0; e < E; e++) {
                double v = 1.0;
                for (int d = 0; d < 3; d++) v *= ldexp(h->tree_len[d], -lev[e]);
                vol[e] = v;
            }
        }
    }
    for (int64_t e = 0; e < E; e++) {
        const double gn = sqrt(hg[e] * hg[e] + hg[E + e] * hg[E + e] + hg[2 * E + e] * hg[2 * E + e]);
        const double r = rho[e] > 1.0e-12 ? rho[e] : 1.0e-12;
        const double ind = gn * (per_cell ? cbrt(vol[e]) : 1.0) / r;
        flags[e] = (ind > threshold) ? 1 : (ind <= 0.5 * threshold ? -1 : 0);
    }
    return CHARM_GPU_OK;
}

int charm_gpu_adapt_upload(charm_gpu_handle_t h, const charm_gpu_adapt_plan_t *plan, const charm_gpu_mesh_t *mesh)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->hex) return fail(CHARM_GPU_ENOTSUP, "adapt projection: box meshes only");
    h->dt_next_valid = false;
    if (!plan || !mesh || (plan->n_pass > 0 && (!plan->n_out || !plan->map))) return fail(CHARM_GPU_EINVAL, "null argument");
    if (h->nb != CHARM_GPU_BASIS) return fail(CHARM_GPU_ENOTSUP, "adapt projection: p1 only");
    if (plan->n_in != h->E) return fail(CHARM_GPU_EINVAL, "adapt plan: input leaves differ from the uploaded mesh");
    const int64_t n_last = plan->n_pass ? plan->n_out[plan->n_pass - 1] : plan->n_in;
    if (n_last != mesh->n_elem) return fail(CHARM_GPU_EINVAL, "adapt plan: output leaves differ from the mesh");
    const bool mixed = h->cfg.precision == CHARM_GPU_PREC_MIXED;
    if (mixed && (rc = ff_convert(h, false))) return rc;   // d_u <- hi + lo
    const int V = n_var(h);
    int64_t nmax = plan->n_in;
    for (int p = 0; p < plan->n_pass; p++) {
        if (plan->n_out[p] < 1 || plan->n_out[p] > INT32_MAX) return fail(CHARM_GPU_EINVAL, "adapt plan: bad pass size");
        nmax = std::max(nmax, plan->n_out[p]);
    }
    const size_t sb = sizeof(double) * (size_t) V * 4 * (size_t) nmax;
    if ((rc = ensure_buf(h, &h->d_proj[0], sb)) || (rc = ensure_buf(h, &h->d_proj[1], sb)) ||
        (rc = ensure_buf(h, &h->d_pmap, sizeof(int32_t) * 2 * (size_t) nmax)))
        return rc;
    const double *src = h->d_u;
    int64_t Ei = plan->n_in;
    double *dst = h->d_proj[0];
    if (plan->n_pass == 0)
        CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * (size_t) V * 4 * (size_t) Ei, cudaMemcpyDeviceToDevice,
                                 h->stream));
    for (int p = 0; p < plan->n_pass; p++) {
        const int64_t Eo = plan->n_out[p];
        // the map's sources must lie in the pass's input (a bad plan must not
        // send the kernel out of bounds)
        const int32_t *mp = plan->map[p];
        for (int64_t k = 0; k < Eo; k++) {
            const int32_t sidx = mp[2 * k], op = mp[2 * k + 1];
            if (op < -1 || op > 8 || sidx < 0 || (int64_t) sidx + (op == 8 ? 8 : 1) > Ei)
                return fail(CHARM_GPU_EINVAL, "adapt plan: map entry out of range");
        }
        dst = h->d_proj[p & 1];
        CUDA_TRY(cudaMemcpyAsync(h->d_pmap, mp, sizeof(int32_t) * 2 * (size_t) Eo, cudaMemcpyHostToDevice, h->stream));
        adapt_project_kernel<<<(unsigned) ((Eo + 255) / 256), 256, 0, h->stream>>>(src, Ei, dst, Eo, h->d_pmap, V);
        CUDA_TRY(cudaGetLastError());
        src = dst;
        Ei = Eo;
    }
    if ((rc = charm_gpu_upload_mesh(h, mesh))) return rc;
    CUDA_TRY(cudaMemcpyAsync(h->d_u, dst, sizeof(double) * (size_t) V * 4 * (size_t) h->E, cudaMemcpyDeviceToDevice,
                             h->stream));
    if (mixed && (rc = ff_convert(h, true))) return rc;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_set_state(charm_gpu_handle_t h, const double *u, int on_device)
{
    if (!h || !u) return fail(CHARM_GPU_EINVAL, "null argument");
    if (!h->mesh_ready) return fail(CHARM_GPU_ESTATE, "no mesh uploaded");
    h->dt_next_valid = false;
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t st = (size_t) n_var(h) * h->nb * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(h->d_u, u, st, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED) {
        int rc = ff_convert(h, true);
        if (rc) return rc;
    }
    if (!on_device) CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_get_state(charm_gpu_handle_t h, double *u, int on_device)
{
    if (!h || !u) return fail(CHARM_GPU_EINVAL, "null argument");
    if (!h->mesh_ready) return fail(CHARM_GPU_ESTATE, "no mesh uploaded");
    CUDA_TRY(cudaSetDevice(h->device));
    const size_t st = (size_t) n_var(h) * h->nb * h->E * sizeof(double);
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED) {
        int rc = ff_convert(h, false);
        if (rc) return rc;
    }
    CUDA_TRY(cudaMemcpyAsync(u, h->d_u, st, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    if (!on_device) CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_step(charm_gpu_handle_t h, double dt_in, double *dt_out)
{
    CfgLease lease(h);
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
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    int done = 0;
    if ((rc = run_as_graph(h, nsteps, dt_in, &done))) return rc;
    for (int s = done; s < nsteps; s++) {
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
    CfgLease lease(h);
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
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (!res) return fail(CHARM_GPU_EINVAL, "null argument");
    const bool mixed = h->cfg.precision == CHARM_GPU_PREC_MIXED;
    if (mixed && (rc = ff_convert(h, false))) return rc;   // d_u <- hi + lo
    if (h->nb == kNB2 && mixed) {
        // FP32 residual into the hi plane of buffer 1, widened into d_ua
        const FFCoef z = {0.f, 0.f}, one = {1.f, 0.f};
        rc = (h->cfg.n_comp == 1) ? p2_ff_stage<1>(h, 0, -1, 1, z, one, z, kCellResidual)
                                  : p2_ff_stage<2>(h, 0, -1, 1, z, one, z, kCellResidual);
        if (rc) return rc;
        const int64_t n = n_state(h);
        CUDA_TRY(cudaMemsetAsync(h->d_fl[1], 0, n * sizeof(float), h->stream));
        ff_to_double_kernel<<<(unsigned) ((n + 255) / 256), 256, 0, h->stream>>>(h->d_fh[1], h->d_fl[1], h->d_ua, n);
        CUDA_TRY(cudaGetLastError());
    } else if (h->nb == kNB2) {
        switch (h->cfg.n_comp) {
        case 1: rc = p2_stage<1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
        default: rc = p2_stage<2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
        }
    } else if (!mixed && h->cfg.model == CHARM_GPU_MODEL_NS && h->cfg.use_visc) {
        // with the viscous terms (no chemistry outside a step: chem_rhs = 0)
        switch (h->cfg.n_comp) {
        case 1:
            if (!(rc = launch_visc<1>(h, h->d_u, nullptr)) && !(rc = launch_face<double, 1>(h, h->d_u)) &&
                !(rc = launch_vflux<1>(h, h->d_u)))
                rc = launch_cell<double, 1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual, h->d_radd);
            break;
        default:
            if (!(rc = launch_visc<2>(h, h->d_u, nullptr)) && !(rc = launch_face<double, 2>(h, h->d_u)) &&
                !(rc = launch_vflux<2>(h, h->d_u)))
                rc = launch_cell<double, 2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual, h->d_radd);
            break;
        }
    } else if (h->cfg.precision == CHARM_GPU_PREC_DW) {
        switch (h->cfg.n_comp) {
        case 1: rc = launch_face<dw, 1>(h, h->d_u); if (!rc) rc = launch_cell<dw, 1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
        default: rc = launch_face<dw, 2>(h, h->d_u); if (!rc) rc = launch_cell<dw, 2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
        }
    } else switch (h->cfg.n_comp * 2 + (mixed ? 1 : 0)) {
    case 2: rc = launch_face<double, 1>(h, h->d_u); if (!rc) rc = launch_cell<double, 1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    case 3: rc = launch_face<float, 1>(h, h->d_u); if (!rc) rc = launch_cell<float, 1>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    case 4: rc = launch_face<double, 2>(h, h->d_u); if (!rc) rc = launch_cell<double, 2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    case 5: rc = launch_face<float, 2>(h, h->d_u); if (!rc) rc = launch_cell<float, 2>(h, h->d_u, nullptr, h->d_ua, 0, nullptr, 1, 0, kCellResidual); break;
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
    if (rc) return rc;
    const size_t st = (size_t) n_var(h) * h->nb * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(res, h->d_ua, st, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return CHARM_GPU_OK;
}

int charm_gpu_limit(charm_gpu_handle_t h)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    h->dt_next_valid = false;
    if (h->cfg.limiter != CHARM_GPU_LIM_BJ) return CHARM_GPU_OK;
    const size_t st = (size_t) n_var(h) * h->nb * h->E * sizeof(double);
    const bool mixed = h->cfg.precision == CHARM_GPU_PREC_MIXED;
    if (mixed && (rc = ff_convert(h, false))) return rc;   // d_u <- hi + lo
    CUDA_TRY(cudaMemcpyAsync(h->d_ua, h->d_u, st, cudaMemcpyDeviceToDevice, h->stream));
    if (h->nb == kNB2) {
        rc = (h->cfg.n_comp == 1) ? launch_p2_limit<1>(h, h->d_ua, nullptr, h->d_u, 1.0, 0.0)
                                  : launch_p2_limit<2>(h, h->d_ua, nullptr, h->d_u, 1.0, 0.0);
        return rc;
    }
    switch (h->cfg.n_comp) {
    case 1: rc = launch_limit<1>(h, h->d_ua, nullptr, h->d_u, 1.0, 0.0); break;
    case 2: rc = launch_limit<2>(h, h->d_ua, nullptr, h->d_u, 1.0, 0.0); break;
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
    if (!rc && mixed) rc = ff_convert(h, true);
    return rc;
}

int charm_gpu_refine_flags(charm_gpu_handle_t h, double max_err, int8_t *flags, double *grad_out)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->nb != CHARM_GPU_BASIS) return fail(CHARM_GPU_ENOTSUP, "refine flags: p1 only");
    if (!flags && !grad_out) return fail(CHARM_GPU_EINVAL, "null argument");
    if (h->hex) {
        // general hexahedra: the estimate from the face tables, the criterion
        // with each element's own (quadrature) volume
        double *d_grad = h->d_ua;
        TimedLaunch t;
        begin_launch(h, 3, &t);
        if (h->cfg.n_comp == 1) hex_launch_amr_grad<1>(mesh_view(h), hex_view(h), h->d_u, d_grad, h->stream);
        else hex_launch_amr_grad<2>(mesh_view(h), hex_view(h), h->d_u, d_grad, h->stream);
        end_launch(h, &t);
        CUDA_TRY(cudaGetLastError());
        std::vector<double> g(grad_out ? 0 : (size_t) (3 * h->E)), vol((size_t) h->E);
        double *hg = grad_out ? grad_out : g.data();
        CUDA_TRY(cudaMemcpyAsync(hg, d_grad, sizeof(double) * 3 * h->E, cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaMemcpyAsync(vol.data(), h->d_hex_g + (size_t) kGvol * h->E, sizeof(double) * h->E,
                                 cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        if (flags) {
            const double err2_max = max_err * max_err;
            for (int64_t e = 0; e < h->E; e++) {   // charm_refine_err_estimate (src/charm_amr.c:12-48)
                double diff2 = 0.0;
                for (int d = 0; d < 3; d++) diff2 += hg[d * h->E + e] * hg[d * h->E + e];
                const double err2 = diff2 * (1. / 12.) * exp(log(vol[e]) * 5. / 3.);
                flags[e] = (err2 > err2_max * vol[e]) ? 1 : 0;
            }
        }
        return CHARM_GPU_OK;
    }
    if (h->cfg.precision == CHARM_GPU_PREC_MIXED && (rc = ff_convert(h, false))) return rc;   // d_u <- hi + lo
    // the gradient goes through the (idle) slot buffer: 3*E doubles fit in it
    MeshDev m = mesh_view(h);
    double *d_grad = h->d_ua;
    const int bs = 128;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    switch (h->cfg.n_comp) {
    case 1: amr_grad_kernel<1><<<(unsigned) ((h->E + bs - 1) / bs), bs, 0, h->stream>>>(m, h->d_u, d_grad); break;
    case 2: amr_grad_kernel<2><<<(unsigned) ((h->E + bs - 1) / bs), bs, 0, h->stream>>>(m, h->d_u, d_grad); break;
    default: return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    }
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    std::vector<double> g(grad_out ? 0 : (size_t) (3 * h->E));
    double *hg = grad_out ? grad_out : g.data();
    CUDA_TRY(cudaMemcpyAsync(hg, d_grad, sizeof(double) * 3 * h->E, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (flags) {
        // charm_refine_err_estimate (src/charm_amr.c:12-48), on the host with
        // the same libm calls, so the flags follow the reference's rounding
        std::vector<int8_t> lev((size_t) h->E);
        CUDA_TRY(cudaMemcpy(lev.data(), h->d_level, (size_t) h->E, cudaMemcpyDeviceToHost));
        const double err2_max = max_err * max_err;
        // the box volume and vol^(5/3) depend on the level only: the same
        // expressions, evaluated once per level instead of once per element
        double lvol[128], lpow[128];
        for (int l = 0; l < 128; l++) {
            double hh[3];
            for (int d = 0; d < 3; d++) hh[d] = ldexp(h->tree_len[d], -l);
            lvol[l] = hh[0] * hh[1] * hh[2];
            lpow[l] = exp(log(lvol[l]) * 5. / 3.);
        }
        for (int64_t e = 0; e < h->E; e++) {
            const int l = lev[e] & 127;   // leaf levels are 0..CHARM_FOREST_MAXLEVEL
            double diff2 = 0.0;
            for (int d = 0; d < 3; d++) diff2 += hg[d * h->E + e] * hg[d * h->E + e];
            const double err2 = diff2 * (1. / 12.) * lpow[l];
            flags[e] = (err2 > err2_max * lvol[l]) ? 1 : 0;
        }
    }
    return CHARM_GPU_OK;
}

int charm_gpu_set_stream(charm_gpu_handle_t h, void *stream)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    CfgLease lease(h);
    CfgSlot &s = cfg_slot(h->device);
    cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    if (s.live && s.stream == h->stream && next != h->stream) {
        // the caller may destroy the old stream: mark its queued work now
        CUDA_TRY(cudaSetDevice(h->device));
        if (!s.fence) CUDA_TRY(cudaEventCreateWithFlags(&s.fence, cudaEventDisableTiming));
        CUDA_TRY(cudaEventRecord(s.fence, h->stream));
        s.fence_pending = true;
        s.live = false;
        s.owner = nullptr;   // re-upload the constants on the new stream
    }
    h->stream = next;
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
        if (err & kErrWait) return fail(CHARM_GPU_ETIMEDOUT, "a bounded device wait (bulk copy) ran out");
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
    CfgLease lease(h);
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

int charm_gpu_abi_sizes(int64_t out[6])
{
    if (!out) return fail(CHARM_GPU_EINVAL, "null argument");
    out[0] = sizeof(charm_gpu_config_t);
    out[1] = sizeof(charm_gpu_mesh_t);
    out[2] = sizeof(charm_gpu_comp_t);
    out[3] = sizeof(charm_gpu_bnd_t);
    out[4] = sizeof(charm_gpu_objective_t);
    out[5] = sizeof(charm_gpu_adjoint_info_t);
    return CHARM_GPU_OK;
}

int charm_gpu_dims(charm_gpu_handle_t h, int64_t *n_elem, int *nv, int *nb)
{
    if (!h) return fail(CHARM_GPU_EINVAL, "null handle");
    if (n_elem) *n_elem = h->E;
    if (nv) *nv = n_var(h);
    if (nb) *nb = h->nb;
    return CHARM_GPU_OK;
}

}  // extern "C"

// ============================================================================
// Allocation-free residual: charm_gpu_residual_static (include/charm_gpu.h)
// ============================================================================
//
// For callers that cannot allocate device memory themselves or let a library
// do it for them -- code that runs where cudaMalloc is forbidden or unsafe,
// such as a host framework that owns all device memory through its own pool
// allocator, or a step inside a real-time loop that must not allocate.
// They pass the mesh, the state and the output as device buffers they own;
// the face projections this computation needs between its kernels live in
// one file-scope __device__ array of CHARM_GPU_STATIC_SCRATCH_BYTES, which
// every GPU that loads the library holds until the process exits.
//
// Set-up: the first call on a device, with that device current, resolves
// the array's device address with cudaGetSymbolAddress.  Make that first
// call before any stream capture.  All calls share the one array and each
// call rewrites what it uses (control words cleared, face table reset at the
// start of every call), so calls that overlap on the GPU (different streams
// or host threads, or a handle's kernels running at the same time) race:
// serialise them.
//
// Kernels: a table kernel (validates the face records and writes, per
// element face, where its flux projection will be), the regular path's face
// kernel writing into the scratch, and a gather kernel (volume integral +
// the element's projections -> residual).

namespace {

constexpr size_t kScratchBytes = CHARM_GPU_STATIC_SCRATCH_BYTES;
constexpr size_t kCtrlBytes = 256;      // control words at the start of the scratch
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

void *g_scratch_addr[kMaxDevices];
std::mutex g_setup_mutex;

// control words
enum : int { kCtlBadRecord = 0, kCtlMissingFace = 1, kCtlDeviceErr = 2 };

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Per element face: (slot << 2) | tag; tag 0 = one slot, tag 1 = big side of
// a mortar whose 4 sub-face records start at the face of `slot >> 1`.
// Entries start at -1 (memset 0xff) and every element face must be written.
// Element face slot idx takes its record's code; a second record for the
// same element face marks the mesh invalid.
__device__ __forceinline__ void static_claim(int32_t *ef, unsigned *ctl, int64_t idx, int32_t code)
{
    if (atomicCAS(reinterpret_cast<int *>(ef + idx), -1, (int) code) != -1) atomicOr(&ctl[kCtlBadRecord], 16u);
}

__global__ void static_table_kernel(MeshDev m, int n_bnd, int32_t *ef, unsigned *ctl)
{
    const int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem, F = m.n_face;
    if (t < F) {
        const int a = m.face_elem[t], b = m.face_elem[F + t];
        const unsigned info = m.face_info[t];
        const int d = info & 3, kind = (info >> 2) & 3, sub = (info >> 4) & 3;
        if (a < 0 || a >= E || b < 0 || b >= E || d > 2 || kind > 2) { atomicOr(&ctl[kCtlBadRecord], 1u); return; }
        const int fa = 2 * d + 1, fb = 2 * d;
        if (kind == 0) {
            static_claim(ef, ctl, (int64_t) fa * E + a, (int32_t) ((2 * t) << 2));
            static_claim(ef, ctl, (int64_t) fb * E + b, (int32_t) ((2 * t + 1) << 2));
            return;
        }
        const int small = (kind == 1) ? a : b, big = (kind == 1) ? b : a;
        const int fs = (kind == 1) ? fa : fb, fbig = (kind == 1) ? fb : fa;
        const int64_t ss = (kind == 1) ? 2 * t : 2 * t + 1, sb = (kind == 1) ? 2 * t + 1 : 2 * t;
        static_claim(ef, ctl, (int64_t) fs * E + small, (int32_t) (ss << 2));
        if (sub == 0) {
            if (t + 3 >= F) { atomicOr(&ctl[kCtlBadRecord], 2u); return; }
            for (int k = 1; k < 4; k++) {
                const unsigned ik = m.face_info[t + k];
                const int bk = (((ik >> 2) & 3) == 1) ? m.face_elem[F + t + k] : m.face_elem[t + k];
                if (((ik >> 4) & 3) != (unsigned) k || (ik & 3) != (unsigned) d || bk != big || ((ik >> 2) & 3) != (unsigned) kind) {
                    atomicOr(&ctl[kCtlBadRecord], 4u);
                    return;
                }
            }
            static_claim(ef, ctl, (int64_t) fbig * E + big, (int32_t) ((sb << 2) | 1));
        }
    } else if (t < F + m.n_bface) {
        const int64_t j = t - F;
        const int e = m.bface_elem[j], f = m.bface_face[j], bid = m.bface_bnd[j];
        if (e < 0 || e >= E || f < 0 || f > 5 || bid < 0 || bid >= n_bnd) { atomicOr(&ctl[kCtlBadRecord], 8u); return; }
        static_claim(ef, ctl, (int64_t) f * E + e, (int32_t) ((2 * F + j) << 2));
    }
}

// Volume integral of element e plus its face projections -> res[V][B][E].
template <typename T, int NC>
__global__ void __launch_bounds__(128)
static_gather_kernel(MeshDev m, const double *__restrict__ u, const T *__restrict__ slots,
                     const int32_t *__restrict__ ef, double *__restrict__ res, unsigned *ctl)
{
    constexpr int V = 4 + NC;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t E = m.n_elem, S = m.n_slot;
    if (e >= E) return;
    const int lev = m.level[e];
    const double hx = level_h(m, lev, 0), hy = level_h(m, lev, 1), hz = level_h(m, lev, 2);
    const double vol = hx * hy * hz;
    T c[V][kNB];
    load_coef<T, V>(u, E, e, c);
    T F[V], G[V], H[V];
#pragma unroll
    for (int v = 0; v < V; v++) F[v] = G[v] = H[v] = T(0);
    T gr[3][kNB];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int k = 0; k < kNB; k++) gr[a][k] = T(0);
    const bool grav = c_cfg.has_grav != 0;
#pragma unroll 1
    for (int g = 0; g < 8; g++) {
        const T px = T((g & 1) ? kGaussPhi : -kGaussPhi);
        const T py = T((g & 2) ? kGaussPhi : -kGaussPhi);
        const T pz = T((g & 4) ? kGaussPhi : -kGaussPhi);
        T U[V];
#pragma unroll
        for (int v = 0; v < V; v++) U[v] = c[v][0] + px * c[v][1] + py * c[v][2] + pz * c[v][3];
        Prim<T, NC> p;
        cons_to_prim<T, NC>(U, p);
        // the state check of cell_kernel: density and pressure at the Gauss points
        if (!(p.r > T(0)) || !(p.p > T(0)))
            set_error(&ctl[kCtlDeviceErr], isfinite((double) p.r) && isfinite((double) p.p) ? kErrNegative : kErrNonFinite);
        const auto hp = U[3] + p.p;   // r e_tot + p: the energy fluxes are u hp, v hp, w hp
        F[0] += U[0] * p.u + p.p; F[1] += U[0] * p.v; F[2] += U[0] * p.w; F[3] += p.u * hp;
        G[0] += U[1] * p.u; G[1] += U[1] * p.v + p.p; G[2] += U[1] * p.w; G[3] += p.v * hp;
        H[0] += U[2] * p.u; H[1] += U[2] * p.v; H[2] += U[2] * p.w + p.p; H[3] += p.w * hp;
#pragma unroll
        for (int i = 0; i < NC; i++) {
            F[4 + i] += U[0] * p.c[i];
            G[4 + i] += U[1] * p.c[i];
            H[4 + i] += U[2] * p.c[i];
        }
        if (grav) {
            const T phi[4] = {T(1), px, py, pz};
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int k = 0; k < kNB; k++) gr[a][k] += p.r * T(c_cfg.grav[a]) * phi[k];
        }
    }
    const double w8 = vol * 0.125;
    double R[V][kNB];
#pragma unroll
    for (int v = 0; v < V; v++) {
        R[v][0] = 0.0;
        R[v][1] = -(double) F[v] * (w8 / hx);
        R[v][2] = -(double) G[v] * (w8 / hy);
        R[v][3] = -(double) H[v] * (w8 / hz);
    }
    if (grav) {
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int k = 0; k < kNB; k++) R[a][k] -= (double) gr[a][k] * w8;
    }
#pragma unroll 1
    for (int f = 0; f < 6; f++) {
        const int32_t code = ef[(int64_t) f * E + e];
        if (code < 0) { atomicOr(&ctl[kCtlMissingFace], 1u); return; }
        const int64_t slot = code >> 2;
        const int nsub = (code & 1) ? 4 : 1;
        for (int k = 0; k < nsub; k++) {
            const int64_t sl = slot + 2 * k;
#pragma unroll
            for (int v = 0; v < V; v++)
#pragma unroll
                for (int b = 0; b < kNB; b++) R[v][b] += (double) slots[(int64_t) (v * kNB + b) * S + sl];
        }
    }
#pragma unroll
    for (int v = 0; v < V; v++)
#pragma unroll
        for (int b = 0; b < kNB; b++) res[(int64_t) (v * kNB + b) * E + e] = R[v][b];
}

template <typename T, int NC>
void launch_face_static(const charm_gpu_config_t *cfg, const MeshDev &m, const double *u, T *slots, unsigned *err,
                        cudaStream_t st)
{
    const int bs = 128;
    const int64_t nbi = (m.n_face + bs - 1) / bs, nbb = (m.n_bface + bs - 1) / bs;
    if (nbi + nbb == 0) return;
    const unsigned g = (unsigned) (nbi + nbb);
    switch (cfg->flux) {
    case CHARM_GPU_FLUX_LF: face_kernel<T, NC, CHARM_GPU_FLUX_LF><<<g, bs, 0, st>>>(m, u, slots, nbi, err); break;
    case CHARM_GPU_FLUX_HLLC: face_kernel<T, NC, CHARM_GPU_FLUX_HLLC><<<g, bs, 0, st>>>(m, u, slots, nbi, err); break;
    case CHARM_GPU_FLUX_CD: face_kernel<T, NC, CHARM_GPU_FLUX_CD><<<g, bs, 0, st>>>(m, u, slots, nbi, err); break;
    default: face_kernel<T, NC, CHARM_GPU_FLUX_GODUNOV><<<g, bs, 0, st>>>(m, u, slots, nbi, err); break;
    }
}

template <typename T, int NC>
void run_static(const charm_gpu_config_t *cfg, const MeshDev &m, const double *u, unsigned char *base, size_t ef_off,
                size_t slot_off, double *res, cudaStream_t st)
{
    unsigned *ctl = reinterpret_cast<unsigned *>(base);
    int32_t *ef = reinterpret_cast<int32_t *>(base + ef_off);
    T *slots = reinterpret_cast<T *>(base + slot_off);
    launch_face_static<T, NC>(cfg, m, u, slots, &ctl[kCtlDeviceErr], st);
    const int bs = 128;
    static_gather_kernel<T, NC><<<(unsigned) ((m.n_elem + bs - 1) / bs), bs, 0, st>>>(m, u, slots, ef, res, ctl);
}

}  // namespace

extern "C" int charm_gpu_residual_static(const charm_gpu_config_t *cfg, const charm_gpu_mesh_t *mesh, const double *u,
                                         double *res, void *stream)
{
    if (!cfg || !mesh || !u || !res) return fail(CHARM_GPU_EINVAL, "null argument");
    if (cfg->n_comp < 1 || cfg->n_comp > 2) return fail(CHARM_GPU_ENOTSUP, "1 or 2 species only");
    if (cfg->flux < 0 || cfg->flux > 3 || cfg->n_bnd < 0 || cfg->n_bnd > CHARM_GPU_MAX_BND || cfg->use_visc || cfg->p_order == 2 ||
        (cfg->precision != CHARM_GPU_PREC_FP64 && cfg->precision != CHARM_GPU_PREC_MIXED) ||
        (cfg->eos != CHARM_GPU_EOS_IDEAL && cfg->eos != CHARM_GPU_EOS_MIX))
        return fail(CHARM_GPU_EINVAL, "invalid configuration");
    for (int i = 0; i < cfg->n_comp; i++)
        if (!(cfg->comp[i].m > 0) || cfg->comp[i].n_cp < 1 || cfg->comp[i].n_cp > CHARM_GPU_MAX_CP)
            return fail(CHARM_GPU_EINVAL, "invalid component");
    const int64_t E = mesh->n_elem, F = mesh->n_face, Fb = mesh->n_bface;
    if (E <= 0 || F < 0 || Fb < 0 || E >= (int64_t) INT32_MAX) return fail(CHARM_GPU_EINVAL, "bad mesh sizes");
    if (!mesh->level || (F && (!mesh->face_elem || !mesh->face_info)) ||
        (Fb && (!mesh->bface_elem || !mesh->bface_face || !mesh->bface_bnd)))
        return fail(CHARM_GPU_EINVAL, "null mesh array");
    const int V = 4 + cfg->n_comp;
    const size_t tsize = cfg->precision == CHARM_GPU_PREC_MIXED ? sizeof(float) : sizeof(double);
    int64_t S = 2 * F + Fb;
    S += (S & 1);
    const size_t ef_off = kCtrlBytes;
    const size_t slot_off = align256(ef_off + (size_t) 6 * (size_t) E * sizeof(int32_t));
    const size_t need = slot_off + (size_t) V * CHARM_GPU_BASIS * (size_t) (S > 0 ? S : 2) * tsize;
    if (need > kScratchBytes)
        return fail(CHARM_GPU_EINVAL, "mesh too large for charm_gpu_residual_static: needs " + std::to_string(need) +
                                          " bytes of scratch, the static array holds " + std::to_string(kScratchBytes));
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(CHARM_GPU_ECUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return fail(CHARM_GPU_ENOTSUP, "device index above 63");
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess || !p)
                return fail(CHARM_GPU_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = p;
        }
    }
    unsigned char *base = static_cast<unsigned char *>(g_scratch_addr[dev]);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevCfg dcfg;
    build_devcfg(cfg, &dcfg);
    cudaError_t e;
    // take c_cfg over from any handle on this device (their queued launches
    // finish first); every path below ends with st synchronised, so nothing
    // of this call reads c_cfg after it returns
    CfgLease lease(dev);
    CfgSlot &cs = cfg_slot(dev);
    struct Release {
        CfgSlot &s;
        ~Release() { s.owner = nullptr; s.live = false; }
    } release{cs};
    if ((e = cfg_takeover(cs, st)) != cudaSuccess) return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    cs.owner = nullptr;
    cs.stream = st;
    cs.live = true;
    if ((e = cudaMemcpyToSymbolAsync(c_cfg, &dcfg, sizeof(DevCfg), 0, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    // clear the control words, and mark every element face unset
    if ((e = cudaMemsetAsync(base, 0, kCtrlBytes, st)) != cudaSuccess) return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    if ((e = cudaMemsetAsync(base + ef_off, 0xff, (size_t) 6 * E * sizeof(int32_t), st)) != cudaSuccess)
        return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    MeshDev m;
    memset(&m, 0, sizeof(m));
    m.n_elem = E; m.n_face = F; m.n_bface = Fb; m.n_slot = S;
    m.center = mesh->center; m.level = mesh->level;
    m.face_elem = mesh->face_elem; m.face_info = mesh->face_info;
    m.bface_elem = mesh->bface_elem; m.bface_face = mesh->bface_face; m.bface_bnd = mesh->bface_bnd;
    for (int d = 0; d < 3; d++) {
        m.tree_len[d] = mesh->tree_len[d];
        m.tree_len_f[d] = (float) mesh->tree_len[d];
    }
    const int bs = 256;
    const int64_t nt = F + Fb;
    unsigned *ctl = reinterpret_cast<unsigned *>(base);
    if (nt > 0)
        static_table_kernel<<<(unsigned) ((nt + bs - 1) / bs), bs, 0, st>>>(m, cfg->n_bnd,
                                                                           reinterpret_cast<int32_t *>(base + ef_off), ctl);
    unsigned h_ctl[4] = {0, 0, 0, 0};
    if ((e = cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    if (h_ctl[kCtlBadRecord])
        return fail(CHARM_GPU_EINVAL, "face record out of range, mortar records not consecutive, or an element face "
                                      "with more than one record");
    const bool mixed = cfg->precision == CHARM_GPU_PREC_MIXED;
    switch (cfg->n_comp * 2 + (mixed ? 1 : 0)) {
    case 2: run_static<double, 1>(cfg, m, u, base, ef_off, slot_off, res, st); break;
    case 3: run_static<float, 1>(cfg, m, u, base, ef_off, slot_off, res, st); break;
    case 4: run_static<double, 2>(cfg, m, u, base, ef_off, slot_off, res, st); break;
    default: run_static<float, 2>(cfg, m, u, base, ef_off, slot_off, res, st); break;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    if ((e = cudaMemcpyAsync(h_ctl, ctl, sizeof(h_ctl), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    if (h_ctl[kCtlMissingFace]) return fail(CHARM_GPU_EINVAL, "an element face has no face record");
    if (h_ctl[kCtlDeviceErr] & kErrNonFinite) return fail(CHARM_GPU_ENONFINITE, "non-finite state");
    if (h_ctl[kCtlDeviceErr] & kErrNegative) return fail(CHARM_GPU_ENEGATIVE, "non-positive density or pressure");
    if (h_ctl[kCtlDeviceErr] & kErrHllc) return fail(CHARM_GPU_EHLLC, "HLLC: SL <= S* <= SR violated");
    return CHARM_GPU_OK;
}

extern "C" int charm_gpu_point_flux(const charm_gpu_config_t *cfg, int64_t n, const double *U2, const double *normals,
                                    double *q)
{
    if (!cfg || n < 0 || (n > 0 && (!U2 || !normals || !q))) return fail(CHARM_GPU_EINVAL, "null argument");
    int rc = validate_config(cfg);
    if (rc) return rc;
    if (n == 0) return CHARM_GPU_OK;
    if (n > ((int64_t) 1 << 30)) return fail(CHARM_GPU_EINVAL, "too many points");
    const int V = 4 + cfg->n_comp;
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    DevCfg dcfg;
    build_devcfg(cfg, &dcfg);
    struct Bufs {
        cudaStream_t st = nullptr;
        double *U2 = nullptr, *nrm = nullptr, *q = nullptr;
        unsigned *err = nullptr;
        ~Bufs()
        {
            if (st) cudaStreamSynchronize(st);
            cudaFree(U2); cudaFree(nrm); cudaFree(q); cudaFree(err);
            if (st) cudaStreamDestroy(st);
        }
    } b;
    CUDA_TRY(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
    const size_t su = (size_t) n * 2 * V * sizeof(double), sn = (size_t) n * 3 * sizeof(double),
                 sq = (size_t) n * V * sizeof(double);
    if (cudaMalloc(&b.U2, su) != cudaSuccess || cudaMalloc(&b.nrm, sn) != cudaSuccess ||
        cudaMalloc(&b.q, sq) != cudaSuccess || cudaMalloc(&b.err, sizeof(unsigned)) != cudaSuccess)
        return fail(CHARM_GPU_ENOMEM, "cudaMalloc failed");
    CUDA_TRY(cudaMemcpyAsync(b.U2, U2, su, cudaMemcpyHostToDevice, b.st));
    CUDA_TRY(cudaMemcpyAsync(b.nrm, normals, sn, cudaMemcpyHostToDevice, b.st));
    CUDA_TRY(cudaMemsetAsync(b.err, 0, sizeof(unsigned), b.st));
    unsigned herr = 0;
    {
        // the point kernels have their own translation unit and so their own
        // copy of the configuration constants: calls of this entry point
        // take turns, handles are not affected
        static std::mutex point_mu;
        std::lock_guard<std::mutex> lock(point_mu);
        const bool mixed = cfg->precision == CHARM_GPU_PREC_MIXED;
        const bool dword = cfg->precision == CHARM_GPU_PREC_DW;
        cudaError_t e = point_launch_flux(&dcfg, cfg->flux, cfg->n_comp, mixed, dword, n, b.U2, b.nrm, b.q, b.err, b.st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(q, b.q, sq, cudaMemcpyDeviceToHost, b.st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, b.err, sizeof(unsigned), cudaMemcpyDeviceToHost, b.st);
        cudaError_t e2 = cudaStreamSynchronize(b.st);
        if (e == cudaSuccess) e = e2;
        if (e != cudaSuccess) return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    }
    if (herr & kErrHllc) return fail(CHARM_GPU_EHLLC, "HLLC: SL <= S* <= SR violated");
    return CHARM_GPU_OK;
}

extern "C" int charm_gpu_math_check(int which, int64_t n, const double *a, const double *b, double *out)
{
    if (which < 0 || which > 1 || n < 0 || (n > 0 && (!b || !out || (which == 1 && !a))))
        return fail(CHARM_GPU_EINVAL, "bad argument");
    if (n == 0) return CHARM_GPU_OK;
    if (n > ((int64_t) 1 << 28)) return fail(CHARM_GPU_EINVAL, "too many operands");
    struct Bufs {
        double *a = nullptr, *b = nullptr, *o = nullptr;
        ~Bufs() { cudaFree(a); cudaFree(b); cudaFree(o); }
    } d;
    const size_t sz = (size_t) n * sizeof(double);
    if (cudaMalloc(&d.a, sz) != cudaSuccess || cudaMalloc(&d.b, sz) != cudaSuccess || cudaMalloc(&d.o, sz) != cudaSuccess)
        return fail(CHARM_GPU_ENOMEM, "cudaMalloc failed");
    CUDA_TRY(cudaMemcpy(d.b, b, sz, cudaMemcpyHostToDevice));
    if (which == 1) CUDA_TRY(cudaMemcpy(d.a, a, sz, cudaMemcpyHostToDevice));
    CUDA_TRY(point_launch_math(which, n, d.a, d.b, d.o, nullptr));
    CUDA_TRY(cudaMemcpy(out, d.o, sz, cudaMemcpyDeviceToHost));
    return CHARM_GPU_OK;
}

#include "adjoint_host.cuh"
