/*
 * charm_gpu.h - C ABI of the GB300 DG time-step library (libcharm_gpu.so).
 *
 * The library replaces CHARM_3D's per-step model plugin, i.e. the pair
 *   charm_timestep_single_fn_t  (reference include/charm_globals.h:239)
 *   charm_get_timestep_fn_t     (reference include/charm_globals.h:240)
 * registered by charm_model_ns_init / charm_model_euler_init
 * (reference src/models/ns/charm_model_ns_init.cpp:79-88,
 *  src/models/euler/charm_model_euler_init.cpp:14-18) and called once per
 * step by charm_timesteps (reference src/charm_timesteps.c:42).
 *
 * The host keeps the octree (refine, 2:1 balance, coarsen) on the CPU.  After
 * each adapt it flattens leaves and faces into the structure-of-arrays mesh
 * below and uploads it; the conserved state then stays resident in HBM.
 * The plugin function pointers of the reference (flux_fn, lim_fn, eos_fn,
 * bnd_fn; reference include/charm_globals.h:122,236-238) become enum
 * selectors in charm_gpu_config_t.
 *
 * Conventions
 *   - Every entry point returns an int status (CHARM_GPU_OK == 0); none of
 *     them exits the process (the reference's charm_abort calls exit(1),
 *     src/charm_globals.c:459-470).
 *   - State arrays are double [V][B][E]: variable-major, then basis
 *     coefficient, then element (Morton order of the uploaded mesh).
 *     V = 4 + n_comp in the reference's order (ru, rv, rw, re, rc_0..);
 *     density is the sum of the partial densities rc_i.
 *   - A handle is used by one host thread at a time; calls are ordered on the
 *     handle's CUDA stream.  `stream` arguments are cudaStream_t values passed
 *     as void* (NULL = the handle's own stream).  Several handles may run
 *     from several threads and streams at once: the kernels read the
 *     configuration from one constant-memory copy per device, and a call
 *     that switches it to another handle's configuration first waits (on
 *     the GPU) for the launches still queued with the previous one.
 */
#ifndef CHARM_GPU_H
#define CHARM_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define CHARM_GPU_OK          0
#define CHARM_GPU_EINVAL      1   /* bad argument or configuration */
#define CHARM_GPU_ENOMEM      2   /* device or host allocation failed */
#define CHARM_GPU_ECUDA       3   /* CUDA runtime error */
#define CHARM_GPU_ENONFINITE  4   /* device error word: non-finite state */
#define CHARM_GPU_ENEGATIVE   5   /* device error word: density or pressure <= 0 */
#define CHARM_GPU_EHLLC       6   /* device error word: HLLC wave-speed order broken
                                     (reference src/charm_fluxes.c:354-357 aborts) */
#define CHARM_GPU_ETIMEDOUT   7   /* bounded host wait ran out */
#define CHARM_GPU_ESTATE      8   /* call order (e.g. step before upload) */
#define CHARM_GPU_ENOTSUP     9   /* configuration not implemented on the GPU */

/* ---- selectors (reference strings in src/charm_init_yaml.cpp) ------------- */
enum { CHARM_GPU_MODEL_EULER = 0,   /* "EULER": one forward-Euler stage
                                       (src/models/euler/charm_model.c:454-540) */
       CHARM_GPU_MODEL_NS    = 1 }; /* "NS": 3-stage SSP-RK with limiter per stage
                                       (src/models/ns/charm_model.c:187-273) */

enum { CHARM_GPU_FLUX_LF = 0, CHARM_GPU_FLUX_GODUNOV = 1, CHARM_GPU_FLUX_HLLC = 2,
       CHARM_GPU_FLUX_CD = 3 };                        /* :352-368 */
enum { CHARM_GPU_LIM_NONE = 0, CHARM_GPU_LIM_BJ = 1 };  /* :370-380 */
enum { CHARM_GPU_EOS_IDEAL = 0, CHARM_GPU_EOS_MIX = 1 };/* :174-186 */
enum { CHARM_GPU_PREC_FP64 = 0,     /* drop-in: all arithmetic in FP64 */
       CHARM_GPU_PREC_MIXED = 1,    /* FP32 residual, FP32 hi/lo state, FP64 dt */
       CHARM_GPU_PREC_DW = 2 };     /* FP64 state; residual (fluxes, volume terms) in double-word
                                       arithmetic on the FP32 pipe (two floats, ~48 bits), within
                                       ~1e-13 of FP64; p1 convective terms (no viscous terms or
                                       chemistry), no adjoint, no allocation-free residual */
enum { CHARM_GPU_DT_TAU = 0,        /* fixed TAU: the reference's get_dt_fn
                                       (src/models/ns/charm_model.c:49) */
       CHARM_GPU_DT_CFL = 1 };      /* CFL*volume/(|u|+c) at the cell centres,
                                       min over cells and TAU (the reference's
                                       unreachable code, :21-36, 50-59) */

/* boundary types, same numbering as charm_bnd_types_t
 * (reference include/charm_globals.h:432-439) */
enum { CHARM_GPU_BND_INLET = 0, CHARM_GPU_BND_OUTLET = 1, CHARM_GPU_BND_WALL_SLIP = 2,
       CHARM_GPU_BND_WALL_NO_SLIP = 3, CHARM_GPU_BND_MASS_FLOW = 4 };

/* component property laws (reference include/charm_globals.h:206-221) */
enum { CHARM_GPU_CP_CONST = 0, CHARM_GPU_CP_POLYNOM = 1 };
enum { CHARM_GPU_LAW_CONST = 0, CHARM_GPU_LAW_SUTHERLAND = 1 };

#define CHARM_GPU_MAX_COMP   8    /* species on the device (reference: 128 slots) */
#define CHARM_GPU_MAX_CP     8    /* cp polynomial coefficients */
#define CHARM_GPU_MAX_BND   16    /* boundary-condition table entries */
#define CHARM_GPU_BASIS      4    /* p1 Taylor basis (CHARM_BASE_FN_COUNT, charm_def.h:177) */
#define CHARM_GPU_BASIS_P2  10    /* p2 Taylor basis (p_order = 2); state arrays are then [V][10][E] */

typedef struct charm_gpu_comp {      /* charm_comp_t, include/charm_globals.h:224-240 */
    double m, ml0, kp0, t0, ts, sig, ek, h0;
    int    cp_type, kp_type, ml_type;
    int    n_cp;
    double cp[CHARM_GPU_MAX_CP];
} charm_gpu_comp_t;

typedef struct charm_gpu_bnd {       /* charm_bnd_t, include/charm_globals.h:441-448 */
    int    type;
    /* inlet: V.x V.y V.z T P; wall_no_slip: T; mass_flow: M P T CosX CosY CosZ P c_0.. */
    double params[7 + CHARM_GPU_MAX_COMP];
} charm_gpu_bnd_t;

#define CHARM_GPU_MAX_REACT  8    /* reactions (charm_ctx_t.reactions) */

typedef struct charm_gpu_reaction {  /* charm_reaction_t, include/charm_globals.h:280-287 */
    int32_t left[3], right[3];       /* component indices, -1 = none (always 3 entries) */
    double  a, e, n;                 /* k = a * T^n * exp(-e / (T R)) */
} charm_gpu_reaction_t;

typedef struct charm_gpu_config {
    int    model, flux, limiter, eos, precision, dt_mode;
    int    n_comp;
    charm_gpu_comp_t comp[CHARM_GPU_MAX_COMP];
    int    n_bnd;
    charm_gpu_bnd_t bnd[CHARM_GPU_MAX_BND];
    double grav[3];      /* region gravity (charm_reg_t.grav), uniform over the mesh */
    double tau;          /* control.TAU */
    double cfl;          /* control.CFL */
    double t_ref;        /* control.MODEL.t_ref */
    int    use_visc;     /* MODEL.use_visc: viscous and heat-conduction terms (FP64 only) */
    int    check_every;  /* steps between device error-word checks (0 = only at sync) */
    int    use_diff;     /* MODEL.use_diffusion: species diffusion (needs use_visc, >= 2 species) */
    int    n_react;      /* reactions, evaluated per RK stage on cell means */
    charm_gpu_reaction_t react[CHARM_GPU_MAX_REACT];
    int    p_order;      /* basis order: 1 (0 = 1), the reference's p1 Taylor basis with its 8/6-point
                            rules; 2: the p2 Taylor basis (10 functions, charm_base_func) with
                            27-point cell and 9-point face Gauss rules (uniform meshes, FP64) */
} charm_gpu_config_t;

/*
 * Flattened mesh.  Elements are the octree leaves in Morton order.  Each leaf
 * is an axis-aligned box; `level` with `tree_len` gives its edge lengths
 * h = tree_len / 2^level (the reference's dh, src/charm_geom.c:157-169).
 *
 * Interior faces join side 0 (lower coordinate along `dir`, its face 2*dir+1)
 * and side 1 (its face 2*dir); this is p4est_iterate's side order.  A hanging
 * face of a 2:1 mesh is stored as 4 sub-face records ("1-to-4 mortar"), each
 * joining one small leaf with the big one; quadrature points then lie on the
 * small leaf's face (src/models/euler/charm_model.c:282-285).
 *
 * face_info bits: 0-1 dir | 2-3 kind (0 conforming, 1 side 0 is the small
 * leaf, 2 side 1 is the small leaf) | 4-5 sub (position of the small face in
 * the big face: bit 4 along the lower tangential axis, bit 5 along the upper)
 * | 6 periodic wrap.
 */
typedef struct charm_gpu_mesh {
    int64_t        n_elem;
    const double  *center;      /* [3][n_elem] */
    const int8_t  *level;       /* [n_elem] */
    double         tree_len[3];
    int64_t        n_face;
    const int32_t *face_elem;   /* [2][n_face] */
    const uint8_t *face_info;   /* [n_face] */
    int64_t        n_bface;
    const int32_t *bface_elem;  /* [n_bface] */
    const int8_t  *bface_face;  /* [n_bface] 0..5 (-x,+x,-y,+y,-z,+z) */
    const int8_t  *bface_bnd;   /* [n_bface] index into charm_gpu_config_t.bnd */
} charm_gpu_mesh_t;

/*
 * General (trilinear) hexahedra: the leaves of a forest over an unstructured
 * hexahedral mesh (one tree per hexahedron of a gmsh file, reference
 * src/charm_connectivity.c:315-519), mapped into space through each tree's
 * corner vertices (p4est_qcoord_to_vertex, as src/charm_geom.c:12-31 uses
 * it).  With a mesh of such elements, charm_gpu_mesh_t's center holds the
 * element centres (informative), level and tree_len are not used, face_info
 * keeps its kind and sub bits (dir: side 0's face / 2), and for every
 * interior face record the faces of both sides are given here; quadrature
 * points, weights, normals, the Taylor basis centre and scale and the mass
 * matrix of every element are computed from the corners as the reference
 * computes them (charm_geom_quad_calc, src/charm_geom.c:496-530).
 */
typedef struct charm_gpu_hex {
    const double *vertex;      /* [8][3][n_elem]: corner k (p4est order, k = ix + 2 iy + 4 iz),
                                  coordinate d of element e at vertex[(3 k + d) n_elem + e] */
    const int8_t *face_face;   /* [2][n_face]: face number (0..5) of interior face record i on
                                  side 0 (face_face[i]) and side 1 (face_face[n_face + i]) */
} charm_gpu_hex_t;

typedef struct charm_gpu_handle_s *charm_gpu_handle_t;

/* Library version and the text of the last error on this thread. */
const char *charm_gpu_version(void);
const char *charm_gpu_last_error(void);

/* Create a solver on CUDA device `device` (replaces charm_model_*_init). */
int charm_gpu_create(charm_gpu_handle_t *h, const charm_gpu_config_t *cfg, int device);
int charm_gpu_destroy(charm_gpu_handle_t h);

/* Upload a flattened mesh (after each adapt).  The caller owns the arrays;
 * the library copies them.  Resets the state to zero.  Invalid records
 * (indices out of range, mortar sub-faces that are not 4 consecutive
 * records, an element face without a record or with two) return
 * CHARM_GPU_EINVAL before anything changes: the previous mesh and state
 * stay as they were. */
int charm_gpu_upload_mesh(charm_gpu_handle_t h, const charm_gpu_mesh_t *mesh);

/* Upload a mesh of general hexahedra (see charm_gpu_hex_t); otherwise as
 * charm_gpu_upload_mesh, with the same record checks, and also
 * CHARM_GPU_EINVAL for an element whose corners give a non-positive
 * Jacobian at a quadrature point (the reference asserts gj != 0,
 * src/charm_geom.c:124).  FP64, p1, convective terms: CHARM_GPU_ENOTSUP for
 * the mixed and double-word forms, p2, viscous terms and chemistry. */
int charm_gpu_upload_mesh_hex(charm_gpu_handle_t h, const charm_gpu_mesh_t *mesh, const charm_gpu_hex_t *hex);

/* State in/out, layout [V][B][E] (reference charm_data_t.par.c,
 * include/charm_globals.h:329-338).  `on_device` != 0: `u` is a device pointer. */
int charm_gpu_set_state(charm_gpu_handle_t h, const double *u, int on_device);
int charm_gpu_get_state(charm_gpu_handle_t h, double *u, int on_device);

/* One time step (1 stage for EULER, 3 SSP-RK stages for NS, each followed by
 * the limiter).  dt_in > 0 is used as the step; dt_in <= 0 takes the step
 * from the configured dt mode.  *dt_out (may be NULL) receives the step
 * taken.  Replaces charm_timestep_single_fn_t. */
int charm_gpu_step(charm_gpu_handle_t h, double dt_in, double *dt_out);

/* n steps back to back (no host round trip between them).  With a fixed
 * step (dt_in > 0, or the TAU mode), no per-kernel timing and no periodic
 * error-word check, the steps are replayed as a CUDA graph of two steps,
 * captured on the handle's stream by the first such run and kept for later
 * runs with the same step, stream and mesh (an upload drops it); results
 * and launch counts are those of the steps launched one by one. */
int charm_gpu_run(charm_gpu_handle_t h, int nsteps, double dt_in);

/* Time step of the configured mode (replaces charm_get_timestep_fn_t). */
int charm_gpu_get_dt(charm_gpu_handle_t h, double *dt);

/* Residual int_*[V][B][E] of the current state: volume plus surface
 * integrals, before M^-1 (reference int_ru..int_rc, charm_globals.h:403-407). */
int charm_gpu_residual(charm_gpu_handle_t h, double *res, int on_device);

/* Apply the configured limiter once to the current state. */
int charm_gpu_limit(charm_gpu_handle_t h);

/* Density-gradient refinement indicator of charm_adapt
 * (reference src/charm_amr.c:12-48, 350-573): flags[e] = 1 where
 * |grad rho|^2/12 * V^(5/3) > max_err^2 * V.  grad_out ([3][E], may be NULL)
 * receives the gradient estimate.  On general hexahedra V is each element's
 * quadrature volume and the estimate uses the faces' own normals. */
int charm_gpu_refine_flags(charm_gpu_handle_t h, double max_err, int8_t *flags, double *grad_out);

/* Stream control and synchronisation.  charm_gpu_sync waits at most
 * timeout_s seconds (bounded polling) and then reports the device error word. */
int charm_gpu_set_stream(charm_gpu_handle_t h, void *stream);
int charm_gpu_sync(charm_gpu_handle_t h, double timeout_s);

/* Kernel accounting for measurement: launches since the last reset, and the
 * summed CUDA-event duration per kernel class when timing is enabled.
 * Classes: 0 face, 1 cell (volume + gather + update), 2 limiter, 3 other. */
int charm_gpu_set_timing(charm_gpu_handle_t h, int enable);
int charm_gpu_kernel_stats(charm_gpu_handle_t h, int64_t launches[4], double ms[4]);
int charm_gpu_reset_stats(charm_gpu_handle_t h);

/* Run nsteps (as charm_gpu_run) between two CUDA events recorded on the
 * handle's stream and return the elapsed device time in *ms. */
int charm_gpu_time_run(charm_gpu_handle_t h, int nsteps, double dt_in, double *ms);

/* Measured arithmetic peak of this GPU's CUDA cores, for roofline
 * denominators: which = 0 FP64 FMA, 1 FP32 FMA; *tflops in TFLOP/s. */
int charm_gpu_probe_peak(int device, int which, double *tflops);

/* sizeof of the ABI structs as compiled into the library, for binding checks:
 * out[0] config, out[1] mesh, out[2] comp, out[3] bnd, out[4] objective,
 * out[5] adjoint info. */
int charm_gpu_abi_sizes(int64_t out[6]);

/*
 * Residual R(u) (as charm_gpu_residual) without allocating any device
 * memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc, or have a library call it for them -- code whose
 * device memory is owned by another allocator (a framework's memory pool)
 * or that runs in a loop where allocation is not allowed.  The caller
 * passes device buffers it owns: the mesh arrays (mesh holds DEVICE
 * pointers, same layout as for charm_gpu_upload_mesh), the state u
 * [V][B][E] and the output res [V][B][E].  The face projections between the
 * kernels live in one static device array of CHARM_GPU_STATIC_SCRATCH_BYTES
 * (about 1 KB per element in FP64, so up to ~65,000 elements); larger
 * meshes are rejected with CHARM_GPU_EINVAL and a message.  The first call
 * on a device (with that device current) looks up the array's address:
 * make it before any stream capture.  All calls share the array, so calls
 * that overlap on the GPU race; serialise them.  Synchronises `stream` to
 * read its error words, so no call can be captured into a CUDA graph.
 * Errors as charm_gpu_sync reports them for a handle (non-finite state,
 * non-positive density or pressure at a Gauss point, HLLC wave order), and
 * CHARM_GPU_EINVAL for face records that point outside the mesh, mortar
 * records that are not 4 consecutive sub-faces, an element face without a
 * record or with two; `res` is then not written.
 */
#define CHARM_GPU_STATIC_SCRATCH_BYTES ((size_t) 64 << 20)
int charm_gpu_residual_static(const charm_gpu_config_t *cfg, const charm_gpu_mesh_t *mesh, const double *u, double *res,
                              void *stream);

/*
 * Numerical flux between n pairs of conserved states, evaluated by the same
 * device functions as the face kernels (verification entry; the reference's
 * counterpart is the configured flux_fn, include/charm_globals.h:238, as
 * charm_calc_flux_{lf,hllc,godunov,cd} in src/charm_fluxes.c).  Host arrays:
 * U2 [n][2][V] (side 0, side 1), normals [n][3] (unit, from side 0 to side
 * 1), q [n][V].  An axis-aligned normal takes the face kernels' axis path,
 * any other normal the general rotation.  cfg gives flux, EOS and
 * components (precision FP64: double arithmetic; MIXED: the float
 * instantiation of the mixed form).  Allocates and synchronises.
 */
int charm_gpu_point_flux(const charm_gpu_config_t *cfg, int64_t n, const double *U2, const double *normals, double *q);

/* The FP64 division helpers of the flux kernels on n host operands
 * (verification entry; no counterpart in the reference): which = 0:
 * out = the Newton-refined reciprocal of b; 1: out = the quotient a / b as
 * the kernels form it.  Allocates and synchronises. */
int charm_gpu_math_check(int which, int64_t n, const double *a, const double *b, double *out);

/* The p2 basis contraction (values of n_var = 5 or 6 variables' 10 Taylor
 * coefficients at the 27 cell Gauss points, the first step of every p2 cell
 * stage; reference src/charm_base_func.c:139-196) as a measurement entry with
 * no counterpart in the reference: method 0 on FP32 FMAs, method 1 on the
 * tensor cores (tcgen05.mma, BF16 operands split in three terms each, six
 * products, FP32 accumulation in tensor memory).  coef: host float
 * [n_var][10][E]; sum[e] = sum_q w_q sum_v U_v(q)^2 (host double [E]);
 * vals (optional) the values, host float [E][n_var][27].  The kernel runs
 * once, then `reps` times timed with CUDA events: *ms is the time of one
 * launch.  Allocates and synchronises. */
int charm_gpu_p2_interp(int method, int64_t E, int n_var, const float *coef, double *sum, float *vals, int reps,
                        double *ms);

/* Element count, variables and basis size of the uploaded mesh. */
int charm_gpu_dims(charm_gpu_handle_t h, int64_t *n_elem, int *n_var, int *n_basis);

/* ---- discrete adjoint ------------------------------------------------------
 * No counterpart in the reference (it has no adjoint).  The transpose of the
 * exact derivative of the FP64 time step as the GPU computes it: face fluxes
 * (LF, CD, HLLC), boundary states (inlet, outlet, slip and no-slip walls),
 * volume fluxes, gravity, the RK stages and their combinations; the BJ
 * limiter enters with its scaling frozen at the forward value (the active
 * set is not differentiated).  Requires an FP64 handle, an ideal gas with
 * constant cp and a fixed step (TAU); other configurations return
 * CHARM_GPU_ENOTSUP.  Arrays are host [V][B][E] like the state. */

enum { CHARM_GPU_OBJ_PRESSURE_BOX = 1 };

/* J = integral of the pressure over the elements whose centre lies in
 * [lo, hi) (8-point Gauss rule per element). */
typedef struct {
    int32_t kind;       /* CHARM_GPU_OBJ_* */
    int32_t pad;
    double  lo[3], hi[3];
} charm_gpu_objective_t;

typedef struct {
    double  J;               /* objective at the final state (0 when dJ/du was given) */
    int64_t forward_steps;   /* forward time steps taken, recomputation included */
    int64_t reverse_steps;   /* adjoint steps (= n_steps) */
    int32_t snapshots;       /* checkpoints held at most, the initial state included */
    int32_t pad;
    double  seconds;         /* wall time of the call */
} charm_gpu_adjoint_info_t;

/* J and dJ/du (dJdu may be NULL) of the current state. */
int charm_gpu_objective(charm_gpu_handle_t h, const charm_gpu_objective_t *obj, double *J, double *dJdu);

/* ubar = (dR/du)^T rbar at the current state, R the residual of
 * charm_gpu_residual. */
int charm_gpu_residual_adjoint(charm_gpu_handle_t h, const double *rbar, double *ubar);

/* Gradient of J(u(n_steps)) with respect to the current state u(0), through
 * n_steps time steps of the handle's scheme.  J is `obj` at the final state,
 * or, when dJdu_final is not NULL, the linear functional with that gradient.
 * Step states are checkpointed in n_snapshots device buffers (the initial
 * state included) and recomputed by binomial checkpointing (Griewank's
 * revolve schedule), so any run length fits the memory given.  With
 * n_snapshots >= 3 * n_steps (1 * n_steps for the forward-Euler model) every
 * stage state is kept instead and nothing is recomputed (one forward sweep).  dJdu0 (may be
 * NULL: the gradient stays on the device for charm_gpu_refine_flags_adjoint)
 * receives dJ/du(0).  The handle ends at the final state, as after
 * charm_gpu_run(h, n_steps, 0). */
int charm_gpu_adjoint(charm_gpu_handle_t h, int n_steps, int n_snapshots, const charm_gpu_objective_t *obj,
                      const double *dJdu_final, double *dJdu0, charm_gpu_adjoint_info_t *info);

/* Adjoint-weighted refinement indicator: the density-gradient estimate of
 * charm_gpu_refine_flags scaled by sqrt(w_e / mean(w)), w_e = |dJ/d(density
 * mean of e)| / V_e from the last charm_gpu_adjoint call, and the reference
 * criterion applied to it (flags[e] = 1: refine).  grad_out ([3][E], may be
 * NULL) receives the weighted gradient, which charm_host_forest_adapt_state
 * takes in place of the plain one, so the octree's refine and coarsen
 * callbacks follow the weighted criterion.  The gradient is that of the
 * current state: set the state the adjoint started from to weight it at
 * that time.  CHARM_GPU_ESTATE when no adjoint has been computed. */
int charm_gpu_refine_flags_adjoint(charm_gpu_handle_t h, double max_err, int8_t *flags, double *grad_out);

/* Projection plan of an adapt, for carrying a device-resident state through
 * it (charm_gpu_adapt_upload).  Pass p maps the leaves before it to its
 * n_out[p] output leaves; for output leaf k, map[p][2k] is a leaf of the
 * pass's input and map[p][2k+1] the operation: -1 copy; 0..7 the child with
 * that Morton child id of that leaf (charm_replace_quads' parent -> child
 * projection); 8 the parent of the family of 8 consecutive input leaves
 * starting there (children -> parent).  The passes are refine, coarsen (when
 * some family merged) and one per 2:1 balance ripple, in order. */
typedef struct {
    int32_t n_pass, pad;
    int64_t n_in;                 /* leaves before the adapt */
    const int64_t *n_out;         /* [n_pass] */
    const int32_t *const *map;    /* [n_pass] -> int32 [2 * n_out[p]] */
} charm_gpu_adapt_plan_t;

/* rho[e] = sum over the species of their mean coefficient in the current
 * state: the centre density that the reference's coarsening criterion reads
 * (before its clamp). */
int charm_gpu_density_means(charm_gpu_handle_t h, double *rho);

/* The refine criterion of the benchmark configuration's AMR case (no
 * counterpart in the reference, whose criterion is charm_gpu_refine_flags'):
 * the indicator |grad rho| * L / rho with the gradient estimate of
 * charm_gpu_refine_flags, rho the centre density (charm_gpu_density_means)
 * and L = 1 (the domain's units) or, with per_cell != 0, the element's edge
 * V^(1/3); flags[e] = +1 where it is above threshold, -1 where it is at most
 * threshold / 2 (a coarsening candidate), else 0.  The flags drive
 * charm_host_forest_adapt_plan_flags.  grad_out ([3][E]) may be NULL. */
int charm_gpu_refine_flags_relative(charm_gpu_handle_t h, double threshold, int per_cell, int8_t *flags,
                                    double *grad_out);

/* Carry the device state through `plan` (p1 projections of
 * charm_replace_quads, src/charm_amr.c:206-307, the arithmetic of
 * charm_host_forest_adapt_state) and upload `mesh`, the flattened forest
 * after that adapt: the state stays on the device across the adapt. */
int charm_gpu_adapt_upload(charm_gpu_handle_t h, const charm_gpu_adapt_plan_t *plan, const charm_gpu_mesh_t *mesh);

/* Cell-centre primitive fields of the current state: the values the
 * reference's output writes per cell (charm_write_solution,
 * src/charm_output.c:10-52: charm_get_fields at the centre, then
 * charm_param_cons_to_prim).  out[f * E + e] for f = 0..7: R, P, E, E_TOT,
 * U, V, W, T, then f = 8 + i: the mass fraction C_i of species i. */
int charm_gpu_cell_fields(charm_gpu_handle_t h, double *out);

/* ---- case file ------------------------------------------------------------
 * CHARM_3D's task.yaml read into the solver configuration, with the same
 * keys, names and checks as the reference's charm_init_context_yaml
 * (reference src/charm_init_yaml.cpp:333-428) and model initialisers
 * (src/models/ns/charm_model_ns_init.cpp:14-89,
 * src/models/euler/charm_model_euler_init.cpp:14-18), which need yaml-cpp.
 * A reader of the YAML subset these files use (block and flow maps and
 * lists, plain and quoted scalars, comments) is built in.  cfg gets the
 * choices the step takes (flux, limiter, EOS of the material, model,
 * components, boundaries in file order, TAU, CFL, gravity, reactions);
 * precision FP64, p_order 1 and dt_mode TAU are set and may be changed
 * before charm_gpu_create.  The rest of the file (time loop, AMR and output
 * controls, mesh file, regions) is returned beside it.  Errors:
 * CHARM_GPU_EINVAL (syntax, missing key, unknown name, the reference's
 * checks) or CHARM_GPU_ENOTSUP (TABLE EOS, more components, boundaries or
 * reactions than the device holds, regions with different gravity), with
 * the message in charm_gpu_last_error(). */
#define CHARM_CASE_MAX_REG 16

typedef struct charm_case_region {   /* charm_reg_t, include/charm_globals.h */
    char   name[64];
    int    id, material_id;
    double v[3], t, p, grav[3];
    double c[CHARM_GPU_MAX_COMP];      /* concentration of each component (file order) */
} charm_case_region_t;

typedef struct charm_case {
    charm_gpu_config_t cfg;
    double tmax, max_error;              /* control.TMAX, MAX_ERROR */
    int    refine_period, repartition_period, min_level, max_level, file_output_step, log_output_step;
    char   mesh_type[32], mesh_name[256];          /* mesh.files_type, mesh.name */
    char   bnd_name[CHARM_GPU_MAX_BND][64];        /* boundaries[i].name (cfg.bnd[i]) */
    char   comp_name[CHARM_GPU_MAX_COMP][64];      /* components[i].name (cfg.comp[i]) */
    int    comp_id[CHARM_GPU_MAX_COMP];
    int    n_reg;
    charm_case_region_t reg[CHARM_CASE_MAX_REG];
} charm_case_t;

int charm_case_read_yaml(const char *path, charm_case_t *out);
int charm_case_parse_yaml(const char *text, charm_case_t *out);

/* ---- host octree (the CPU side of the boundary) -------------------------- */

typedef struct charm_host_forest_s *charm_host_forest_t;

/* Brick of ntree[0]*ntree[1]*ntree[2] cubic trees, uniform `level`. */
int charm_host_forest_new(charm_host_forest_t *f, const int32_t ntree[3], const int32_t periodic[3],
                          const double origin[3], const double tree_len[3], int level);
int charm_host_forest_free(charm_host_forest_t f);
int64_t charm_host_forest_count(charm_host_forest_t f);

/* Forest over an unstructured hexahedral mesh, one tree per hexahedron,
 * uniform `level` (the reference's charm_conn_reader_msh +
 * p4est_connectivity_complete + p4est_new_ext, src/charm_connectivity.c:315-519,
 * src/charm_3d.c:36).  From arrays: n_vert vertices [3], n_tree hexahedra
 * with their corner vertices in p4est order [8], and tree_bnd [6*n_tree],
 * the boundary index of every tree face that has no neighbour.  Tree faces
 * are matched by their vertex sets; a face shared by more than two trees
 * or whose corners do not match as a square's symmetry returns
 * CHARM_GPU_EINVAL. */
int charm_host_forest_new_hex(charm_host_forest_t *f, int32_t n_vert, const double *vert, int32_t n_tree,
                              const int32_t *t2v, const int8_t *tree_bnd, int level);

/* The same from a gmsh 2.x ASCII file: 8-node hexahedra are the trees, and
 * 4-node quadrangles name boundary faces by physical tag; a boundary face
 * takes the configured boundary whose name (bnd_names[k] for
 * charm_gpu_config_t.bnd[k]) is its patch's physical name
 * (charm_conn_bnd_find_by_id, src/charm_connectivity.c:176-203).  A
 * boundary face without a quadrangle or whose name is not configured
 * returns CHARM_GPU_EINVAL with the face in the error text. */
int charm_host_forest_new_gmsh(charm_host_forest_t *f, const char *path, int level, int n_bnd,
                               const char *const *bnd_names);

/* Trees of the forest, and for an unstructured mesh the physical tag of
 * each tree's hexahedron (its region). */
int charm_host_forest_tree_count(charm_host_forest_t f);
int charm_host_forest_tree_region(charm_host_forest_t f, int32_t *reg_tag);

/* Flatten an unstructured forest (charm_host_forest_flatten is for bricks):
 * the same records, interior faces by leaf and face (side 0: the lower
 * coordinate inside a tree, the lower tree across a tree face), plus the
 * corners and face numbers of charm_gpu_hex_t.  Arrays stay owned by f. */
int charm_host_forest_flatten_hex(charm_host_forest_t f, charm_gpu_mesh_t *mesh, charm_gpu_hex_t *hex);

/* Boundary id per domain side (-x,+x,-y,+y,-z,+z) used when flattening. */
int charm_host_forest_set_bnd(charm_host_forest_t f, const int8_t bnd_of_side[6]);

/* Refine flagged leaves (level < maxlevel), then coarsen complete families
 * whose 8 flags are all -1 (level > minlevel), then 2:1 face-balance.
 * Returns the new leaf count via *n_new. */
int charm_host_forest_adapt(charm_host_forest_t f, const int8_t *flags, int minlevel, int maxlevel,
                            int64_t *n_new);

/* One adapt of charm_adapt (reference src/charm_amr.c:575-610) with the
 * state carried along: refine (level < maxlevel) where
 * |grad rho|^2/12 * vol^(5/3) > max_err^2 * vol, coarsen complete families by
 * the reference's family criterion (children's estimates plus the spread of
 * their centre densities; level > minlevel; families refined in this same
 * adapt are not coarsened), then 2:1 face balance.  The state is projected
 * parent <-> children as charm_replace_quads does (:206-307; exact for p1
 * on boxes; on an unstructured forest by the quadrature of the trilinear
 * cells, each leaf's own volume in the criteria, and the first child's for
 * a family as the reference takes it).  grad: [3][E] from
 * charm_gpu_refine_flags; u_in: [V][B][E]
 * of the leaves before the adapt.  The new state ([V][B][n_new]) is returned
 * by charm_host_forest_state and stays valid until the next adapt or free. */
int charm_host_forest_adapt_state(charm_host_forest_t f, const double *grad, double max_err, int minlevel, int maxlevel,
                                  int n_comp, const double *u_in, int64_t *n_new);
int charm_host_forest_state(charm_host_forest_t f, const double **u_out);

/* The adapt of charm_host_forest_adapt_state without the state: the family
 * coarsening criterion reads the centre densities rho ([E], the sum of the
 * species' mean coefficients: charm_gpu_density_means) in place of the
 * state, and the projections are recorded in *plan (valid until the next
 * adapt or free of f).  Same forest as charm_host_forest_adapt_state. */
int charm_host_forest_adapt_plan(charm_host_forest_t f, const double *grad, const double *rho, double max_err,
                                 int minlevel, int maxlevel, int64_t *n_new, charm_gpu_adapt_plan_t *plan);

/* The adapt of charm_host_forest_adapt_plan driven by caller's flags instead
 * of the reference's criteria (e.g. from charm_gpu_refine_flags_relative):
 * refine the leaves flagged +1 (level < maxlevel), coarsen complete families
 * whose 8 flags are -1 (level > minlevel; families refined in this adapt
 * are not coarsened), then 2:1 face balance; the projections are recorded
 * as the plan, as there.  Bricks only (CHARM_GPU_ENOTSUP otherwise). */
int charm_host_forest_adapt_plan_flags(charm_host_forest_t f, const int8_t *flags, int minlevel, int maxlevel,
                                       int64_t *n_new, charm_gpu_adapt_plan_t *plan);

/* Flatten into a mesh view whose arrays live inside the forest object and
 * stay valid until the next adapt/flatten/free. */
int charm_host_forest_flatten(charm_host_forest_t f, charm_gpu_mesh_t *mesh);

/* Write the leaves as a VTK XML unstructured grid (ASCII .vtu): one
 * hexahedron per leaf, cell data "level", "mpirank" (0) and the n_fields
 * arrays fields[f * E + e] under names[f] (the layout of
 * charm_gpu_cell_fields with the reference's names R, P, E, E_TOT, U, V, W,
 * T, C_<component>). */
int charm_host_forest_write_vtu(charm_host_forest_t f, const char *path, int n_fields, const char *const *names,
                                const double *fields);

/* Leaf coordinates: qcoord[4*i..] = x, y, z, tree; level[i]. */
int charm_host_forest_leaves(charm_host_forest_t f, int32_t *qcoord, int8_t *level);

#ifdef __cplusplus
}
#endif

#endif /* CHARM_GPU_H */
