// Host side of the discrete adjoint (part of the charm_gpu.cu translation
// unit): buffers, the reverse of one time step, binomial checkpointing of the
// step states, the objective, and the C entry points declared in charm_gpu.h.
#pragma once

namespace {

int adj_check(charm_gpu_handle_s *h)
{
    if (h->cfg.precision != CHARM_GPU_PREC_FP64) return fail(CHARM_GPU_ENOTSUP, "adjoint: FP64 precision only");
    if (h->hex) return fail(CHARM_GPU_ENOTSUP, "adjoint: box meshes only");
    if (h->nb != CHARM_GPU_BASIS) return fail(CHARM_GPU_ENOTSUP, "adjoint: p1 basis only");
    if (!h->dcfg.ideal_fast) return fail(CHARM_GPU_ENOTSUP, "adjoint: ideal gas with constant cp only");
    if (h->cfg.dt_mode != CHARM_GPU_DT_TAU) return fail(CHARM_GPU_ENOTSUP, "adjoint: fixed time step (TAU) only");
    if (h->cfg.flux == CHARM_GPU_FLUX_GODUNOV) return fail(CHARM_GPU_ENOTSUP, "adjoint: Godunov flux not supported");
    for (int b = 0; b < h->cfg.n_bnd; b++)
        if (h->cfg.bnd[b].type == CHARM_GPU_BND_MASS_FLOW)
            return fail(CHARM_GPU_ENOTSUP, "adjoint: MASS_FLOW boundary not supported");
    if (h->cfg.n_comp < 1 || h->cfg.n_comp > 2) return fail(CHARM_GPU_ENOTSUP, "species count not instantiated");
    if (h->cfg.model == CHARM_GPU_MODEL_NS && (h->cfg.use_visc || h->cfg.n_react))
        return fail(CHARM_GPU_ENOTSUP, "adjoint: viscous terms and reactions not supported");
    return CHARM_GPU_OK;
}

int adj_alloc(charm_gpu_handle_s *h, int n_snap)
{
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    double **bufs[] = {&h->d_adj_lam, &h->d_adj_s, &h->d_adj_acc, &h->d_adj_u1, &h->d_adj_u2, &h->d_adj_fin};
    for (double **q : bufs)
        if (!*q && cudaMalloc(q, st) != cudaSuccess) { *q = nullptr; return fail(CHARM_GPU_ENOMEM, "adjoint buffers"); }
    if (!h->d_adj_psi && cudaMalloc(&h->d_adj_psi, 3 * (size_t) n_var(h) * h->E * sizeof(double)) != cudaSuccess) {
        h->d_adj_psi = nullptr;
        return fail(CHARM_GPU_ENOMEM, "adjoint buffers");
    }
    if (!h->d_obj_part && cudaMalloc(&h->d_obj_part, ((h->E + 127) / 128) * sizeof(double)) != cudaSuccess) {
        h->d_obj_part = nullptr;
        return fail(CHARM_GPU_ENOMEM, "adjoint buffers");
    }
    while ((int) h->d_snap.size() < n_snap) {
        double *q = nullptr;
        if (cudaMalloc(&q, st) != cudaSuccess) return fail(CHARM_GPU_ENOMEM, "adjoint checkpoints");
        h->d_snap.push_back(q);
    }
    return CHARM_GPU_OK;
}

double *adj_psi(charm_gpu_handle_s *h, double *psi, int stage)
{
    return psi + (size_t) stage * n_var(h) * h->E;
}

template <int NC>
int launch_adj_face(charm_gpu_handle_s *h, const double *u, const double *sh, double coef, int scale_minv)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nbi = (h->F + bs - 1) / bs, nbb = (h->Fb + bs - 1) / bs;
    if (nbi + nbb == 0) return CHARM_GPU_OK;
    double *slots = static_cast<double *>(h->d_slots);
    TimedLaunch t;
    begin_launch(h, 0, &t);
    const unsigned nb = (unsigned) (nbi + nbb);
    switch (h->cfg.flux) {
    case CHARM_GPU_FLUX_LF:
        adj_face_kernel<NC, CHARM_GPU_FLUX_LF><<<nb, bs, 0, h->stream>>>(m, u, sh, coef, scale_minv, slots, nbi);
        break;
    case CHARM_GPU_FLUX_CD:
        adj_face_kernel<NC, CHARM_GPU_FLUX_CD><<<nb, bs, 0, h->stream>>>(m, u, sh, coef, scale_minv, slots, nbi);
        break;
    default:
        adj_face_kernel<NC, CHARM_GPU_FLUX_HLLC><<<nb, bs, 0, h->stream>>>(m, u, sh, coef, scale_minv, slots, nbi);
        break;
    }
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

template <int NC>
int launch_adj_cell(charm_gpu_handle_s *h, const double *u, const double *sh, double coef, int scale_minv, double base,
                    int mode, const double *psi, double a_next, double b_next, double *acc, double *out)
{
    MeshDev m = mesh_view(h);
    const int bs = 128;
    TimedLaunch t;
    begin_launch(h, 1, &t);
    adj_cell_kernel<NC><<<(unsigned) ((h->E + bs - 1) / bs), bs, 0, h->stream>>>(
        m, u, sh, coef, scale_minv, static_cast<const double *>(h->d_slots), base, mode, psi, a_next, b_next, acc, out);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

int launch_adj_init(charm_gpu_handle_s *h, const double *psi, double a, double b, bool with_acc)
{
    const int64_t n = (int64_t) n_var(h) * CHARM_GPU_BASIS * h->E;
    const int bs = 256;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    adj_init_kernel<<<(unsigned) ((n + bs - 1) / bs), bs, 0, h->stream>>>(h->d_adj_lam, psi, a, b, n_var(h), h->E,
                                                                          h->d_adj_s, with_acc ? h->d_adj_acc : nullptr);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    return CHARM_GPU_OK;
}

// Recompute the stage states of one step from `in`: u1, u2, the limiter
// scalings of the stages -> psi ([3][V][E]), and the new state -> out when out
// is not null.  The stage that only produces the new state is skipped when
// neither it nor its limiter scaling is needed.
template <int NC>
int adj_forward_step(charm_gpu_handle_s *h, const double *in, double *u1, double *u2, double *psi, double *out)
{
    const double dt = h->cfg.tau;
    const bool lim = h->cfg.limiter == CHARM_GPU_LIM_BJ;
    int rc;
    auto stage = [&](const double *u, const double *u0, double *dst, double a, double b, int k) -> int {
        int r = launch_face<double, NC>(h, u);
        if (r) return r;
        if (lim) {
            if ((r = launch_cell<double, NC>(h, u, nullptr, h->d_ua, dt, nullptr, 1.0, 0.0, kCellUpdate))) return r;
            return launch_limit<NC>(h, h->d_ua, u0, dst, a, b, adj_psi(h, psi, k));
        }
        return launch_cell<double, NC>(h, u, u0, dst, dt, nullptr, a, b, kCellUpdate);
    };
    if (h->cfg.model == CHARM_GPU_MODEL_EULER) {
        if (!out && !lim) return CHARM_GPU_OK;
        return stage(in, nullptr, out ? out : h->d_ub, 1.0, 0.0, 0);
    }
    if ((rc = stage(in, nullptr, u1, 1.0, 0.0, 0))) return rc;
    if ((rc = stage(u1, in, u2, 0.25, 0.75, 1))) return rc;
    if (!out && !lim) return CHARM_GPU_OK;
    return stage(u2, in, out ? out : h->d_ub, 2.0 / 3.0, 1.0 / 3.0, 2);
}

// d_adj_lam: dJ/du(n+1) -> dJ/du(n), with u(n) = in and the stage states
// (u1, u2, psi) of adj_forward_step.
template <int NC>
int adj_reverse_step(charm_gpu_handle_s *h, const double *in, const double *u1, const double *u2, double *psi)
{
    const double dt = h->cfg.tau;
    const bool lim = h->cfg.limiter == CHARM_GPU_LIM_BJ;
    int rc;
    if (h->cfg.model == CHARM_GPU_MODEL_EULER) {
        if ((rc = launch_adj_init(h, lim ? adj_psi(h, psi, 0) : nullptr, 1.0, 0.0, false))) return rc;
        if ((rc = launch_adj_face<NC>(h, in, h->d_adj_s, -dt, 1))) return rc;
        return launch_adj_cell<NC>(h, in, h->d_adj_s, -dt, 1, 1.0, kAdjFinal, nullptr, 0, 0, nullptr, h->d_adj_lam);
    }
    // u3 = 2/3 L(s3) + 1/3 u0
    if ((rc = launch_adj_init(h, lim ? adj_psi(h, psi, 2) : nullptr, 2.0 / 3.0, 1.0 / 3.0, true))) return rc;
    // stage 3 from u2; its u2^ feeds u2 = 1/4 L(s2) + 3/4 u0
    if ((rc = launch_adj_face<NC>(h, u2, h->d_adj_s, -dt, 1))) return rc;
    if ((rc = launch_adj_cell<NC>(h, u2, h->d_adj_s, -dt, 1, 1.0, kAdjStage, lim ? adj_psi(h, psi, 1) : nullptr,
                                  0.25, 0.75, h->d_adj_acc, h->d_adj_s)))
        return rc;
    // stage 2 from u1; u1 = L(s1)
    if ((rc = launch_adj_face<NC>(h, u1, h->d_adj_s, -dt, 1))) return rc;
    if ((rc = launch_adj_cell<NC>(h, u1, h->d_adj_s, -dt, 1, 1.0, kAdjStage, lim ? adj_psi(h, psi, 0) : nullptr,
                                  1.0, 0.0, nullptr, h->d_adj_s)))
        return rc;
    // stage 1 from u0, plus the u0 terms of the combinations
    if ((rc = launch_adj_face<NC>(h, in, h->d_adj_s, -dt, 1))) return rc;
    return launch_adj_cell<NC>(h, in, h->d_adj_s, -dt, 1, 1.0, kAdjFinal, nullptr, 0, 0, h->d_adj_acc, h->d_adj_lam);
}

// J and dJ/du (into grad, device) of the state u.
template <int NC>
int objective_eval(charm_gpu_handle_s *h, const double *u, const charm_gpu_objective_t *obj, double *J, double *grad)
{
    if (obj->kind != CHARM_GPU_OBJ_PRESSURE_BOX) return fail(CHARM_GPU_EINVAL, "unknown objective");
    MeshDev m = mesh_view(h);
    const int bs = 128;
    const int64_t nb = (h->E + bs - 1) / bs;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    adj_objective_kernel<NC><<<(unsigned) nb, bs, 0, h->stream>>>(m, u, obj->lo[0], obj->lo[1], obj->lo[2],
                                                                   obj->hi[0], obj->hi[1], obj->hi[2], h->d_obj_part,
                                                                   grad);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    std::vector<double> part((size_t) nb);
    CUDA_TRY(cudaMemcpyAsync(part.data(), h->d_obj_part, (size_t) nb * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (double x : part) s += x;
    *J = s;
    return CHARM_GPU_OK;
}

// Binomial checkpointing (the optimal schedule of Griewank's revolve): with
// s checkpoint buffers (including the one holding the state at step a),
// reversing n steps costs the fewest forward steps when the next checkpoint
// goes at a + m, m = max(beta(s, t-2), n - beta(s-1, t)), t the smallest
// repetition number with beta(s, t) = C(s + t, s) >= n.
double binom(int64_t n, int64_t k)
{
    double r = 1.0;
    for (int64_t i = 1; i <= k; i++) r = r * (double) (n - k + i) / (double) i;
    return r;
}

int64_t revolve_split(int64_t n, int s)
{
    int64_t t = 0;
    while (binom(s + t, s) < (double) n) t++;
    double m = (t >= 2) ? binom(s + t - 2, s) : 1.0;
    m = std::max(m, (double) n - binom(s - 1 + t, s - 1));
    int64_t mi = (int64_t) m;
    return std::min(std::max<int64_t>(mi, 1), n - 1);
}

struct AdjRun {
    charm_gpu_handle_s *h;
    int64_t n_steps;
    const charm_gpu_objective_t *obj;
    const double *dJdu_final;
    std::vector<int> free_slots;
    bool have_final = false;
    double J = 0.0;
    int64_t forward_steps = 0, reverse_steps = 0;
    int max_slots_used = 1, slots_used = 1;
};

template <int NC>
int adj_restore_and_advance(AdjRun &r, int slot, int64_t k)
{
    charm_gpu_handle_s *h = r.h;
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(h->d_u, h->d_snap[slot], st, cudaMemcpyDeviceToDevice, h->stream));
    for (int64_t i = 0; i < k; i++) {
        int rc = step_impl<double, NC>(h, h->cfg.tau, nullptr);
        if (rc) return rc;
    }
    r.forward_steps += k;
    return CHARM_GPU_OK;
}

// the adjoint step of step a, with u(a) in h->d_u
template <int NC>
int adj_leaf(AdjRun &r, int64_t a)
{
    charm_gpu_handle_s *h = r.h;
    int rc;
    const bool last = (a == r.n_steps - 1) && !r.have_final;
    if ((rc = adj_forward_step<NC>(h, h->d_u, h->d_adj_u1, h->d_adj_u2, h->d_adj_psi,
                                   last ? h->d_adj_fin : nullptr)))
        return rc;
    r.forward_steps += 1;
    if (last) {
        const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
        if (r.dJdu_final) {
            CUDA_TRY(cudaMemcpyAsync(h->d_adj_lam, r.dJdu_final, st, cudaMemcpyHostToDevice, h->stream));
        } else if ((rc = objective_eval<NC>(h, h->d_adj_fin, r.obj, &r.J, h->d_adj_lam))) {
            return rc;
        }
        r.have_final = true;
    }
    if ((rc = adj_reverse_step<NC>(h, h->d_u, h->d_adj_u1, h->d_adj_u2, h->d_adj_psi))) return rc;
    r.reverse_steps += 1;
    if (h->cfg.check_every > 0 && r.reverse_steps % h->cfg.check_every == 0) return charm_gpu_sync(h, 600.0);
    return CHARM_GPU_OK;
}

template <int NC>
int adj_revolve(AdjRun &r, int64_t a, int64_t b, int slot_a, int s)
{
    int rc;
    if (b - a == 1) {
        if ((rc = adj_restore_and_advance<NC>(r, slot_a, 0))) return rc;
        return adj_leaf<NC>(r, a);
    }
    if (s <= 1 || r.free_slots.empty()) {
        for (int64_t k = b - 1; k >= a; k--) {
            if ((rc = adj_restore_and_advance<NC>(r, slot_a, k - a))) return rc;
            if ((rc = adj_leaf<NC>(r, k))) return rc;
        }
        return CHARM_GPU_OK;
    }
    const int64_t m = a + revolve_split(b - a, s);
    if ((rc = adj_restore_and_advance<NC>(r, slot_a, m - a))) return rc;
    const int slot_m = r.free_slots.back();
    r.free_slots.pop_back();
    r.slots_used++;
    r.max_slots_used = std::max(r.max_slots_used, r.slots_used);
    const size_t st = (size_t) n_var(r.h) * CHARM_GPU_BASIS * r.h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(r.h->d_snap[slot_m], r.h->d_u, st, cudaMemcpyDeviceToDevice, r.h->stream));
    if ((rc = adj_revolve<NC>(r, m, b, slot_m, s - 1))) return rc;
    r.free_slots.push_back(slot_m);
    r.slots_used--;
    return adj_revolve<NC>(r, a, m, slot_a, s);
}

// Number of state buffers per step that keep every stage state of it.
int stage_states(const charm_gpu_handle_s *h) { return h->cfg.model == CHARM_GPU_MODEL_EULER ? 1 : 3; }

// Enough buffers for every stage state of the run: one forward sweep keeps
// them all and the reverse sweep recomputes nothing.
template <int NC>
int adjoint_all_stages(charm_gpu_handle_s *h, int n_steps, const charm_gpu_objective_t *obj,
                       const double *dJdu_final, AdjRun &r)
{
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    const int k = stage_states(h);
    const bool lim = h->cfg.limiter == CHARM_GPU_LIM_BJ;
    const size_t psi_n = (size_t) 3 * n_var(h) * h->E;   // per step
    if (lim && h->n_psi_all < (size_t) n_steps * psi_n) {
        if (h->d_adj_psi_all) cudaFree(h->d_adj_psi_all);
        h->n_psi_all = 0;
        if (cudaMalloc(&h->d_adj_psi_all, (size_t) n_steps * psi_n * sizeof(double)) != cudaSuccess) {
            h->d_adj_psi_all = nullptr;
            return fail(CHARM_GPU_ENOMEM, "adjoint limiter scalings");
        }
        h->n_psi_all = (size_t) n_steps * psi_n;
    }
    auto psi_of = [&](int64_t n) { return lim ? h->d_adj_psi_all + (size_t) n * psi_n : h->d_adj_psi; };
    auto u1_of = [&](int64_t n) { return k == 3 ? h->d_snap[k * n + 1] : h->d_adj_u1; };
    auto u2_of = [&](int64_t n) { return k == 3 ? h->d_snap[k * n + 2] : h->d_adj_u2; };
    CUDA_TRY(cudaMemcpyAsync(h->d_snap[0], h->d_u, st, cudaMemcpyDeviceToDevice, h->stream));
    int rc;
    for (int64_t n = 0; n < n_steps; n++) {
        double *out = (n + 1 < n_steps) ? h->d_snap[k * (n + 1)] : h->d_adj_fin;
        if ((rc = adj_forward_step<NC>(h, h->d_snap[k * n], u1_of(n), u2_of(n), psi_of(n), out))) return rc;
        r.forward_steps++;
        if (h->cfg.check_every > 0 && (n + 1) % h->cfg.check_every == 0 && (rc = charm_gpu_sync(h, 600.0))) return rc;
    }
    if (dJdu_final) {
        CUDA_TRY(cudaMemcpyAsync(h->d_adj_lam, dJdu_final, st, cudaMemcpyHostToDevice, h->stream));
    } else if ((rc = objective_eval<NC>(h, h->d_adj_fin, obj, &r.J, h->d_adj_lam))) {
        return rc;
    }
    for (int64_t n = n_steps - 1; n >= 0; n--) {
        if ((rc = adj_reverse_step<NC>(h, h->d_snap[k * n], u1_of(n), u2_of(n), psi_of(n)))) return rc;
        r.reverse_steps++;
        if (h->cfg.check_every > 0 && r.reverse_steps % h->cfg.check_every == 0 && (rc = charm_gpu_sync(h, 600.0)))
            return rc;
    }
    r.max_slots_used = k * n_steps;
    CUDA_TRY(cudaMemcpyAsync(h->d_u, h->d_adj_fin, st, cudaMemcpyDeviceToDevice, h->stream));
    return CHARM_GPU_OK;
}

template <int NC>
int adjoint_impl(charm_gpu_handle_s *h, int n_steps, int n_snap, const charm_gpu_objective_t *obj,
                 const double *dJdu_final, AdjRun &r)
{
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    r.h = h;
    r.n_steps = n_steps;
    r.obj = obj;
    r.dJdu_final = dJdu_final;
    if (n_snap >= stage_states(h) * n_steps) return adjoint_all_stages<NC>(h, n_steps, obj, dJdu_final, r);
    for (int k = n_snap - 1; k >= 1; k--) r.free_slots.push_back(k);
    CUDA_TRY(cudaMemcpyAsync(h->d_snap[0], h->d_u, st, cudaMemcpyDeviceToDevice, h->stream));
    int rc = adj_revolve<NC>(r, 0, n_steps, 0, n_snap);
    if (rc) return rc;
    // the handle ends at the final state, as after charm_gpu_run
    CUDA_TRY(cudaMemcpyAsync(h->d_u, h->d_adj_fin, st, cudaMemcpyDeviceToDevice, h->stream));
    return CHARM_GPU_OK;
}

}  // namespace

extern "C" {

int charm_gpu_objective(charm_gpu_handle_t h, const charm_gpu_objective_t *obj, double *J, double *dJdu)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (!obj || !J) return fail(CHARM_GPU_EINVAL, "null argument");
    if ((rc = adj_check(h)) || (rc = adj_alloc(h, 0))) return rc;
    h->adj_valid = false;
    switch (h->cfg.n_comp) {
    case 1: rc = objective_eval<1>(h, h->d_u, obj, J, h->d_adj_lam); break;
    default: rc = objective_eval<2>(h, h->d_u, obj, J, h->d_adj_lam); break;
    }
    if (rc) return rc;
    if (dJdu) {
        const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
        CUDA_TRY(cudaMemcpyAsync(dJdu, h->d_adj_lam, st, cudaMemcpyDeviceToHost, h->stream));
    }
    return charm_gpu_sync(h, 600.0);
}

int charm_gpu_residual_adjoint(charm_gpu_handle_t h, const double *rbar, double *ubar)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (!rbar || !ubar) return fail(CHARM_GPU_EINVAL, "null argument");
    if ((rc = adj_check(h)) || (rc = adj_alloc(h, 0))) return rc;
    h->adj_valid = false;
    const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
    CUDA_TRY(cudaMemcpyAsync(h->d_adj_s, rbar, st, cudaMemcpyHostToDevice, h->stream));
    switch (h->cfg.n_comp) {
    case 1:
        if (!(rc = launch_adj_face<1>(h, h->d_u, h->d_adj_s, 1.0, 0)))
            rc = launch_adj_cell<1>(h, h->d_u, h->d_adj_s, 1.0, 0, 0.0, kAdjResidual, nullptr, 0, 0, nullptr,
                                    h->d_adj_lam);
        break;
    default:
        if (!(rc = launch_adj_face<2>(h, h->d_u, h->d_adj_s, 1.0, 0)))
            rc = launch_adj_cell<2>(h, h->d_u, h->d_adj_s, 1.0, 0, 0.0, kAdjResidual, nullptr, 0, 0, nullptr,
                                    h->d_adj_lam);
        break;
    }
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(ubar, h->d_adj_lam, st, cudaMemcpyDeviceToHost, h->stream));
    return charm_gpu_sync(h, 600.0);
}

int charm_gpu_refine_flags_adjoint(charm_gpu_handle_t h, double max_err, int8_t *flags, double *grad_out)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    if (!flags && !grad_out) return fail(CHARM_GPU_EINVAL, "null argument");
    if (!h->adj_valid) return fail(CHARM_GPU_ESTATE, "no adjoint: call charm_gpu_adjoint first");
    std::vector<double> grad((size_t) (3 * h->E)), w((size_t) h->E);
    if ((rc = charm_gpu_refine_flags(h, max_err, nullptr, grad.data()))) return rc;
    MeshDev m = mesh_view(h);
    const int bs = 256;
    TimedLaunch t;
    begin_launch(h, 3, &t);
    adj_weight_kernel<<<(unsigned) ((h->E + bs - 1) / bs), bs, 0, h->stream>>>(m, h->d_adj_lam, h->cfg.n_comp,
                                                                               h->d_ub);
    end_launch(h, &t);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(w.data(), h->d_ub, sizeof(double) * h->E, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    double mean = 0.0;
    for (double x : w) mean += x;
    mean /= (double) h->E;
    // grad * sqrt(w / mean(w)): the reference criterion |grad|^2/12 V^(5/3) >
    // max_err^2 V applied to this weighted gradient is the criterion scaled by
    // the relative adjoint weight, so that charm_host_forest_adapt_state (the
    // refine/coarsen callbacks) can take it unchanged
    for (int64_t e = 0; e < h->E; e++) {
        const double s = (mean > 0.0) ? sqrt(w[e] / mean) : 0.0;
        for (int d = 0; d < 3; d++) grad[d * h->E + e] *= s;
    }
    if (grad_out) memcpy(grad_out, grad.data(), sizeof(double) * 3 * h->E);
    if (flags) {
        std::vector<int8_t> lev((size_t) h->E);
        CUDA_TRY(cudaMemcpy(lev.data(), h->d_level, (size_t) h->E, cudaMemcpyDeviceToHost));
        const double err2_max = max_err * max_err;
        for (int64_t e = 0; e < h->E; e++) {
            double hh[3];
            for (int d = 0; d < 3; d++) hh[d] = ldexp(h->tree_len[d], -lev[e]);
            const double vol = hh[0] * hh[1] * hh[2];
            double diff2 = 0.0;
            for (int d = 0; d < 3; d++) diff2 += grad[d * h->E + e] * grad[d * h->E + e];
            const double err2 = diff2 * (1. / 12.) * exp(log(vol) * 5. / 3.);
            flags[e] = (err2 > err2_max * vol) ? 1 : 0;
        }
    }
    return CHARM_GPU_OK;
}

int charm_gpu_adjoint(charm_gpu_handle_t h, int n_steps, int n_snapshots, const charm_gpu_objective_t *obj,
                      const double *dJdu_final, double *dJdu0, charm_gpu_adjoint_info_t *info)
{
    CfgLease lease(h);
    int rc = check_ready(h);
    if (rc) return rc;
    h->dt_next_valid = false;
    if (n_steps < 1 || n_snapshots < 1) return fail(CHARM_GPU_EINVAL, "n_steps and n_snapshots must be >= 1");
    if (!obj && !dJdu_final) return fail(CHARM_GPU_EINVAL, "adjoint: need an objective or dJ/du at the final state");
    if ((rc = adj_check(h))) return rc;
    const int n_snap = (n_snapshots >= stage_states(h) * n_steps) ? stage_states(h) * n_steps
                                                                   : std::min(n_snapshots, n_steps);
    if ((rc = adj_alloc(h, n_snap))) return rc;
    h->adj_valid = false;
    const auto t0 = std::chrono::steady_clock::now();
    AdjRun r;
    switch (h->cfg.n_comp) {
    case 1: rc = adjoint_impl<1>(h, n_steps, n_snap, obj, dJdu_final, r); break;
    default: rc = adjoint_impl<2>(h, n_steps, n_snap, obj, dJdu_final, r); break;
    }
    if (rc) return rc;
    if ((rc = charm_gpu_sync(h, 3600.0))) return rc;
    if (dJdu0) {
        const size_t st = (size_t) n_var(h) * CHARM_GPU_BASIS * h->E * sizeof(double);
        CUDA_TRY(cudaMemcpy(dJdu0, h->d_adj_lam, st, cudaMemcpyDeviceToHost));
    }
    h->adj_valid = true;
    if (info) {
        info->J = r.J;
        info->forward_steps = r.forward_steps;
        info->reverse_steps = r.reverse_steps;
        info->snapshots = r.max_slots_used;
        info->pad = 0;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return CHARM_GPU_OK;
}

}  // extern "C"
