// Tensor-core (tcgen05) form of the p2 basis contraction, and the FMA form
// it is measured against (charm_gpu_p2_interp).
//
// The contraction: the p2 Taylor basis (10 functions, charm_base_func) of V
// state variables evaluated at the 27 cell Gauss points of every element,
// U_v(q) = sum_i c_{v,i} phi_i(q) -- the interpolation every p2 cell-kernel
// stage starts with (reference src/charm_base_func.c:139-196, charm_get_fields).
// As a matrix product per tile of 128 elements and per variable:
// D[e][q] = sum_k A[e][k] B[q][k], M = 128, N = 32 (27 points, padded), on
// tcgen05.mma kind::f16 with BF16 operands and FP32 accumulation in tensor
// memory.  BF16 holds 8 significant bits, so both operands are split into
// three BF16 terms, c = c1 + c2 + c3, phi = p1 + p2 + p3 (24 bits each), and
// the six products that carry weight to 2^-24 are stacked along K:
//   A row e = [c1 | c1 | c2 | c1 | c2 | c3]   (10 columns each, 4 of padding)
//   B row q = [p1 | p2 | p1 | p3 | p2 | p1]
// K = 64 = four MMA steps of 16.  Operands live in shared memory in the
// no-swizzle K-major layout of 8x8 "core matrices" (8 rows of 16 bytes,
// 128 contiguous bytes); the MMA is issued by one thread, completion comes
// back on an mbarrier (tcgen05.commit), and each thread reads its element's
// row of D from tensor memory (tcgen05.ld, lane = element).
//
// Both kernels reduce what they computed to one number per element,
// S_e = sum_q w_q sum_v U_v(q)^2 (w: the Gauss weights), so that the timing
// compares the contraction and not the write-back; with `vals` the full
// U_v(q) are written as well, for the accuracy check.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <cstdint>

#include "charm_gpu.h"

namespace {

constexpr int kNB2 = 10;            // p2 Taylor basis
constexpr int kQ = 27;              // cell Gauss points (3 x 3 x 3)
constexpr int kTileE = 128;         // elements per tile (MMA M)
constexpr int kN = 32;              // points padded (MMA N)
constexpr int kK = 64;              // 6 split products x 10 functions, padded (4 MMA steps of K = 16)
constexpr int kMaxV = 6;

__constant__ float c_phi[kQ][kNB2];   // basis at the Gauss points (reference box [-1/2, 1/2]^3)
__constant__ float c_w[kQ];           // Gauss weights, sum 1

// ---- tcgen05 / mbarrier helpers ------------------------------------------------

__device__ __forceinline__ unsigned saddr(const void *p) { return (unsigned) __cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (between core matrices adjacent along K), stride byte offset
// (between 8-row groups), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(unsigned addr, unsigned lbo, unsigned sbo)
{
    uint64_t d = 0;
    d |= (uint64_t) ((addr >> 4) & 0x3FFFu);
    d |= (uint64_t) ((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t) ((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t) 1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init1(uint64_t *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_wait0(uint64_t *bar, unsigned tries)
{
    for (unsigned i = 0; i < tries; i++) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(saddr(bar)) : "memory");
        if (done) return true;
    }
    return false;
}

// Byte offset of element (r, k) of a K-major operand of kK columns in the
// no-swizzle core-matrix layout: core matrix (r/8, k/8) at ((r/8)*(kK/8) +
// k/8) * 128, row r%8 at 16 bytes, column k%8 at 2 bytes.
__device__ __forceinline__ int core_off(int r, int k)
{
    return ((r >> 3) * (kK / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ void split3(float x, __nv_bfloat16 &a, __nv_bfloat16 &b, __nv_bfloat16 &c)
{
    a = __float2bfloat16_rn(x);
    const float r = x - __bfloat162float(a);
    b = __float2bfloat16_rn(r);
    c = __float2bfloat16_rn(r - __bfloat162float(b));
}

// which split term of A (0, 1, 2 = c1, c2, c3) and of B sits in K group g
__device__ __forceinline__ int a_term(int g) { return (g == 2 || g == 4) ? 1 : (g == 5 ? 2 : 0); }
__device__ __forceinline__ int b_term(int g) { return (g == 1 || g == 4) ? 1 : (g == 3 ? 2 : 0); }

template <int V>
__global__ void __launch_bounds__(kTileE)
p2_interp_tc_kernel(const float *__restrict__ coef, int64_t E, double *__restrict__ sum, float *__restrict__ vals,
                    unsigned *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(sm);                        // V x [128][64]
    __nv_bfloat16 *sB = reinterpret_cast<__nv_bfloat16 *>(sm + V * kTileE * kK * 2);  // [32][64]
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t e0 = (int64_t) blockIdx.x * kTileE;
    const int64_t e = e0 + tid;

    // ---- tensor memory: V x 32 columns (power of two >= 32) ----
    constexpr unsigned ncols = (V * kN <= 32) ? 32 : (V * kN <= 64) ? 64 : (V * kN <= 128) ? 128 : 256;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(saddr(&tmem_base)), "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) mbar_init1(&bar);

    // ---- operands in shared memory ----
    // A: element tid's row of every variable (zeros past the end of the mesh)
    for (int v = 0; v < V; v++) {
        __nv_bfloat16 t[3][kNB2];
#pragma unroll
        for (int i = 0; i < kNB2; i++) {
            const float x = (e < E) ? __ldg(coef + (int64_t) (v * kNB2 + i) * E + e) : 0.f;
            split3(x, t[0][i], t[1][i], t[2][i]);
        }
        __nv_bfloat16 *a = sA + (size_t) v * kTileE * kK;
        unsigned char *ab = reinterpret_cast<unsigned char *>(a);
#pragma unroll
        for (int g = 0; g < 6; g++)
#pragma unroll
            for (int i = 0; i < kNB2; i++)
                *reinterpret_cast<__nv_bfloat16 *>(ab + core_off(tid, g * kNB2 + i)) = t[a_term(g)][i];
        for (int k = 6 * kNB2; k < kK; k++)
            *reinterpret_cast<__nv_bfloat16 *>(ab + core_off(tid, k)) = __float2bfloat16_rn(0.f);
    }
    // B: row q (< 32) by thread q; points past 27 are zero
    if (tid < kN) {
        __nv_bfloat16 t[3][kNB2];
#pragma unroll
        for (int i = 0; i < kNB2; i++) split3((tid < kQ) ? c_phi[tid][i] : 0.f, t[0][i], t[1][i], t[2][i]);
        unsigned char *bb = reinterpret_cast<unsigned char *>(sB);
#pragma unroll
        for (int g = 0; g < 6; g++)
#pragma unroll
            for (int i = 0; i < kNB2; i++)
                *reinterpret_cast<__nv_bfloat16 *>(bb + core_off(tid, g * kNB2 + i)) = t[b_term(g)][i];
        for (int k = 6 * kNB2; k < kK; k++)
            *reinterpret_cast<__nv_bfloat16 *>(bb + core_off(tid, k)) = __float2bfloat16_rn(0.f);
    }
    // shared-memory writes visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    // ---- MMA: one thread issues V x 4 steps, commit to the mbarrier ----
    if (tid == 0) {
        constexpr uint32_t idesc = idesc_bf16(kTileE, kN);
        const unsigned bA = saddr(sA), bB = saddr(sB);
        for (int v = 0; v < V; v++) {
            for (int kb = 0; kb < kK / 16; kb++) {
                // a K step of 16 = 2 core matrices along K = 256 bytes further
                const uint64_t da = smem_desc(bA + (unsigned) (v * kTileE * kK * 2) + kb * 256, 128, (kK / 8) * 128);
                const uint64_t db = smem_desc(bB + kb * 256, 128, (kK / 8) * 128);
                const uint32_t acc = kb ? 1u : 0u;
                asm volatile("{\n\t.reg .pred p;\n\t"
                             "setp.ne.b32 p, %4, 0;\n\t"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                             ::"r"(tmem + (uint32_t) (v * kN)), "l"(da), "l"(db), "r"(idesc), "r"(acc) : "memory");
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     ::"r"(saddr(&bar)) : "memory");
    }
    // every thread waits; the read-back is warp-collective, so all take the
    // same branch
    const bool ok = __syncthreads_and(mbar_wait0(&bar, 1u << 20) ? 1 : 0) != 0;
    if (!ok) {
        // the products did not complete: report, wait (bounded) once more,
        // free the tensor memory and stop
        if (tid == 0) atomicOr(err, 1u);
        mbar_wait0(&bar, 1u << 20);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // ---- read back: thread tid = lane tid = element e ----
        double s = 0.0;
        const uint32_t lane_base = (uint32_t) (warp * 32) << 16;
        for (int v = 0; v < V; v++) {
            uint32_t r[32];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                         "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                         "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                           "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
                           "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
                           "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                         : "r"(tmem + lane_base + (uint32_t) (v * kN)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float sv = 0.f;
#pragma unroll
            for (int q = 0; q < kQ; q++) {
                const float u = __uint_as_float(r[q]);
                sv += c_w[q] * u * u;
                if (vals && e < E) vals[((int64_t) e * V + v) * kQ + q] = u;
            }
            s += sv;
        }
        if (e < E) sum[e] = s;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// The same contraction with FP32 FMAs from registers.
template <int V>
__global__ void __launch_bounds__(kTileE)
p2_interp_fma_kernel(const float *__restrict__ coef, int64_t E, double *__restrict__ sum, float *__restrict__ vals)
{
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double s = 0.0;
    for (int v = 0; v < V; v++) {
        float c[kNB2];
#pragma unroll
        for (int i = 0; i < kNB2; i++) c[i] = __ldg(coef + (int64_t) (v * kNB2 + i) * E + e);
        float sv = 0.f;
#pragma unroll
        for (int q = 0; q < kQ; q++) {
            float u = 0.f;
#pragma unroll
            for (int i = 0; i < kNB2; i++) u = fmaf(c[i], c_phi[q][i], u);
            sv += c_w[q] * u * u;
            if (vals) vals[((int64_t) e * V + v) * kQ + q] = u;
        }
        s += sv;
    }
    sum[e] = s;
}

template <int V>
cudaError_t launch(int method, const float *coef, int64_t E, double *sum, float *vals, unsigned *err, cudaStream_t st)
{
    const unsigned nb = (unsigned) ((E + kTileE - 1) / kTileE);
    if (method == 1) {
        const int smem = V * kTileE * kK * 2 + kN * kK * 2;
        cudaError_t e = cudaFuncSetAttribute(p2_interp_tc_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        p2_interp_tc_kernel<V><<<nb, kTileE, smem, st>>>(coef, E, sum, vals, err);
    } else {
        p2_interp_fma_kernel<V><<<nb, kTileE, 0, st>>>(coef, E, sum, vals);
    }
    return cudaGetLastError();
}

}  // namespace

// Declared in charm_gpu.h.  Errors set the message of charm_gpu_last_error
// through the library's setter.
extern "C" void charm_internal_set_error(const char *msg);

extern "C" int charm_gpu_p2_interp(int method, int64_t E, int n_var, const float *coef, double *sum, float *vals,
                                   int reps, double *ms)
{
    auto fail = [](int code, const char *msg) {
        charm_internal_set_error(msg);
        return code;
    };
    if ((method != 0 && method != 1) || E <= 0 || n_var < 5 || n_var > kMaxV || !coef || !sum || reps < 1)
        return fail(CHARM_GPU_EINVAL, "charm_gpu_p2_interp: bad argument");
    if (E > ((int64_t) 1 << 26)) return fail(CHARM_GPU_EINVAL, "charm_gpu_p2_interp: too many elements");
    // basis and weights at the 27 Gauss points (3 per axis at 0, +-sqrt(3/5)/2)
    static bool tables = false;
    if (!tables) {
        float phi[kQ][kNB2], w[kQ];
        const double g[3] = {-0.5 * 0.7745966692414834, 0.0, 0.5 * 0.7745966692414834};
        const double gw[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};
        for (int q = 0; q < kQ; q++) {
            const int ix = q % 3, iy = (q / 3) % 3, iz = q / 9;
            const double x = g[ix], y = g[iy], z = g[iz];
            const double p[kNB2] = {1.0, x, y, z, x * x, y * y, z * z, x * y, x * z, y * z};
            for (int i = 0; i < kNB2; i++) phi[q][i] = (float) p[i];
            w[q] = (float) (gw[ix] * gw[iy] * gw[iz]);
        }
        if (cudaMemcpyToSymbol(c_phi, phi, sizeof(phi)) != cudaSuccess || cudaMemcpyToSymbol(c_w, w, sizeof(w)) != cudaSuccess)
            return fail(CHARM_GPU_ECUDA, "charm_gpu_p2_interp: constant upload failed");
        tables = true;
    }
    struct Bufs {
        float *c = nullptr, *v = nullptr;
        double *s = nullptr;
        unsigned *err = nullptr;
        cudaEvent_t a = nullptr, b = nullptr;
        ~Bufs()
        {
            cudaFree(c); cudaFree(v); cudaFree(s); cudaFree(err);
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } d;
    const size_t sc = (size_t) n_var * kNB2 * E * sizeof(float), ss = (size_t) E * sizeof(double),
                 sv = (size_t) E * n_var * kQ * sizeof(float);
    if (cudaMalloc(&d.c, sc) != cudaSuccess || cudaMalloc(&d.s, ss) != cudaSuccess ||
        cudaMalloc(&d.err, sizeof(unsigned)) != cudaSuccess || (vals && cudaMalloc(&d.v, sv) != cudaSuccess))
        return fail(CHARM_GPU_ENOMEM, "charm_gpu_p2_interp: cudaMalloc failed");
    if (cudaMemcpy(d.c, coef, sc, cudaMemcpyHostToDevice) != cudaSuccess || cudaMemset(d.err, 0, sizeof(unsigned)) != cudaSuccess ||
        cudaEventCreate(&d.a) != cudaSuccess || cudaEventCreate(&d.b) != cudaSuccess)
        return fail(CHARM_GPU_ECUDA, "charm_gpu_p2_interp: set-up failed");
    cudaError_t e = (n_var == 5) ? launch<5>(method, d.c, E, d.s, d.v, d.err, nullptr)
                                 : launch<6>(method, d.c, E, d.s, d.v, d.err, nullptr);   // warm-up, values
    if (e == cudaSuccess) e = cudaEventRecord(d.a, nullptr);
    for (int r = 0; e == cudaSuccess && r < reps; r++)
        e = (n_var == 5) ? launch<5>(method, d.c, E, d.s, nullptr, d.err, nullptr)
                         : launch<6>(method, d.c, E, d.s, nullptr, d.err, nullptr);
    if (e == cudaSuccess) e = cudaEventRecord(d.b, nullptr);
    if (e == cudaSuccess) e = cudaEventSynchronize(d.b);
    if (e != cudaSuccess) return fail(CHARM_GPU_ECUDA, cudaGetErrorString(e));
    float t = 0.f;
    cudaEventElapsedTime(&t, d.a, d.b);
    if (ms) *ms = (double) t / reps;
    unsigned herr = 0;
    if (cudaMemcpy(&herr, d.err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(sum, d.s, ss, cudaMemcpyDeviceToHost) != cudaSuccess ||
        (vals && cudaMemcpy(vals, d.v, sv, cudaMemcpyDeviceToHost) != cudaSuccess))
        return fail(CHARM_GPU_ECUDA, "charm_gpu_p2_interp: copy back failed");
    if (herr) return fail(CHARM_GPU_ETIMEDOUT, "charm_gpu_p2_interp: a bounded wait for the tensor cores ran out");
    return CHARM_GPU_OK;
}
