// kzg_mlp.cu - learned warm start for contact points that miss the manifold cache.
//
// The reference warm-starts a new contact point with the impulses of the nearest cached point
// within 0.1 m, else with zero (BuildContactConstraints, PhysicsWorld.cpp:518-529).  With a model
// loaded and enabled, the zero is replaced by the prediction of a small MLP: 24 features of the
// prepared contact row -> 64 -> 64 -> 3 (ReLU), BF16 weights and activations, FP32 accumulation on
// the tensor cores (tcgen05: UMMA 128 x N x 16 from shared-memory operands into tensor memory, for
// the in-step inference and for training).  The network predicts the impulses divided by the row
// effective masses (a velocity, m/s; learned through asinh, see kTargetScale); the impulse is the
// prediction times the effective mass, clamped into the friction cone.  The solver then runs
// unchanged, so the solution still converges to the same tolerance - the prediction only changes
// where it starts.
//
// The same translation unit holds the training path (all on the GPU): logging of features and
// converged impulses during a step, and one Adam step = forward + backward over a batch of logged
// samples (one CTA per 128 samples, per-CTA partial gradients summed in a fixed order, so training
// is deterministic).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "kzg_ctx.h"
#include "kzg_internal.h"

namespace kzg {

namespace {

constexpr int kF = KZG_MLP_FEATURES;  // 24
constexpr int kH = 64;
constexpr int kO = 3;
constexpr int kP = KZG_MLP_PARAMS;  // 5955
constexpr int kOffW1 = 0, kOffB1 = kH * kF, kOffW2 = kOffB1 + kH, kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH,
              kOffB3 = kOffW3 + kO * kH;
static_assert(kOffB3 + kO == kP, "parameter layout");
constexpr int kTile = 128;  // samples per CTA (4 warps x 32 rows)
constexpr int kMlpThreads = 128;
constexpr int kLogFloats = KZG_MLP_LOG_FLOATS;  // 24 features + 3 targets + 3 masks

typedef __nv_bfloat16 bf16;

// ---- forward pass on tcgen05 ----------------------------------------------------------------
// One CTA of 128 threads runs a 128-sample tile: three UMMAs of M = 128 (one sample per TMEM lane)
// issued by one thread, X (128 x 32) * W1^T -> 64 columns, H1 (128 x 64) * W2^T -> 64 columns,
// H2 * W3^T -> 16 columns (3 used), bf16 operands, f32 accumulators in 128 TMEM columns (D1 at 0,
// D2 at 64, D3 at 0 again once D1 is read).  Thread t reads TMEM lane t (warp w owns lanes
// 32w..32w+31), applies bias and ReLU and writes its row of the next operand.
//
// Operands sit in shared memory in the canonical K-major layout without swizzle: 8 x 8 bf16 core
// matrices of 128 contiguous bytes (8 rows of 16 bytes), the core matrices of one 8-row group
// adjacent along K (leading byte offset 128), the 8-row groups K / 8 x 128 bytes apart (stride byte
// offset).  One UMMA consumes K = 16, two core matrices; the next starts 256 bytes further.
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kMmaSpins = 1u << 20;  // mbarrier polls before a tile gives up (KZG_DEVERR_MMA)

struct MlpSmemTc {
    alignas(128) unsigned char X[kTile * 32 * 2];
    alignas(128) unsigned char H1[kTile * kH * 2];
    alignas(128) unsigned char H2[kTile * kH * 2];
    alignas(128) unsigned char W1[kH * 32 * 2];
    alignas(128) unsigned char W2[kH * kH * 2];
    alignas(128) unsigned char W3[16 * kH * 2];
    float b1[kH], b2[kH], b3[16];
    alignas(8) unsigned long long mbar;
    uint32_t tmem;
};

// Byte offset of element (r, k) of an operand with K columns in the layout above.
__device__ __forceinline__ uint32_t umma_off(int r, int k, int K) {
    return (uint32_t)(((((r >> 3) * (K >> 3)) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading byte offset >> 4
// (16-29), stride byte offset >> 4 (32-45), descriptor version 1 (46-47), base offset 0, no
// swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, int K) {
    const uint64_t lbo = 128u, sbo = (uint64_t)(K >> 3) * 128u;
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B bf16 (7-9 = 1, 10-12 = 1), both
// K-major (15, 16 = 0), N >> 3 (17-22), M >> 4 (24-28) with M = 128.
__host__ __device__ constexpr uint32_t umma_idesc(uint32_t n) { return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24); }
static_assert(umma_idesc(64) == 0x08100490u && umma_idesc(16) == 0x08040490u, "instruction descriptors");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc ? 1u : 0u) : "memory");
}

// Operand stores (generic proxy) made visible to the tensor core (async proxy), then a CTA barrier
// ordered with the tcgen05 operations before and after it.
__device__ __forceinline__ void tc_sync() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Thread 0: the UMMAs of one product D (128 x n, at d_tmem) = A (128 x K) * B^T (B: n rows of K),
// K / 16 of them, accumulated in order.
__device__ __forceinline__ void tc_chain(uint32_t d_tmem, const unsigned char* A, const unsigned char* B, int K,
                                         uint32_t n) {
    if (threadIdx.x == 0) {
        const uint32_t a0 = smem_u32(A), b0 = smem_u32(B);
        for (int j = 0; j < K / 16; ++j)
            umma(d_tmem, umma_desc(a0 + 256u * j, K), umma_desc(b0 + 256u * j, K), umma_idesc(n), j > 0);
    }
}

// Thread 0: the CTA's mbarrier completes once every UMMA it issued so far is done.
__device__ __forceinline__ void tc_commit(unsigned long long* mbar) {
    if (threadIdx.x == 0)
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void tc_layer(uint32_t d_tmem, const unsigned char* A, const unsigned char* W, int K,
                                         uint32_t n, unsigned long long* mbar) {
    tc_chain(d_tmem, A, W, K, n);
    tc_commit(mbar);
}

// Waits for the committed UMMAs (bounded); false when the wait gave up.
__device__ __forceinline__ bool tc_wait(unsigned long long* mbar, uint32_t& phase) {
    const uint32_t a = smem_u32(mbar);
    uint32_t done = 0;
    for (uint32_t n = 0; n < kMmaSpins && !done; ++n)
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(a), "r"(phase) : "memory");
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return __syncthreads_and(done != 0) != 0;
}

// After a wait that gave up (every thread of the CTA calls it): waits once more, bounded, for the
// committed UMMAs still in flight, so that the tensor memory they write is not freed under them.
__device__ __forceinline__ void tc_drain(unsigned long long* mbar, uint32_t phase) {
    uint32_t p = phase ^ 1u;  // the phase the failed wait polled (tc_wait flips it either way)
    tc_wait(mbar, p);
}

// 16 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Epilogue of a hidden layer: this thread's 64 accumulators + bias, ReLU, bf16, into row t of H
// (and, for the weight gradients, into column t of Ht: 64 rows of K = 128 samples).
__device__ __forceinline__ void tc_hidden(uint32_t taddr, const float* bias, unsigned char* H,
                                          unsigned char* Ht = nullptr) {
    const int t = threadIdx.x;
#pragma unroll
    for (int c0 = 0; c0 < kH; c0 += 16) {
        float v[16];
        tmem_ld16(taddr + (uint32_t)c0, v);
#pragma unroll
        for (int h = 0; h < 16; h += 8) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const __nv_bfloat162 p = __floats2bfloat162_rn(fmaxf(v[h + 2 * q] + bias[c0 + h + 2 * q], 0.0f),
                                                               fmaxf(v[h + 2 * q + 1] + bias[c0 + h + 2 * q + 1], 0.0f));
                w[q] = *reinterpret_cast<const uint32_t*>(&p);
                if (Ht) {
                    *reinterpret_cast<__nv_bfloat16*>(Ht + umma_off(c0 + h + 2 * q, t, kTile)) = p.x;
                    *reinterpret_cast<__nv_bfloat16*>(Ht + umma_off(c0 + h + 2 * q + 1, t, kTile)) = p.y;
                }
            }
            *reinterpret_cast<uint4*>(H + umma_off(t, c0 + h, kH)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// bf16 weights in the UMMA layout (W1 padded to K = 32, W3 to 16 rows) and the biases.
__device__ void stage_weights_tc(const float* __restrict__ th, MlpSmemTc& S, int tid) {
    for (int i = tid; i < kH * 32; i += kMlpThreads) {
        const int n = i >> 5, k = i & 31;
        *reinterpret_cast<bf16*>(S.W1 + umma_off(n, k, 32)) = __float2bfloat16_rn(k < kF ? th[kOffW1 + n * kF + k] : 0.0f);
    }
    for (int i = tid; i < kH * kH; i += kMlpThreads)
        *reinterpret_cast<bf16*>(S.W2 + umma_off(i >> 6, i & 63, kH)) = __float2bfloat16_rn(th[kOffW2 + i]);
    for (int i = tid; i < 16 * kH; i += kMlpThreads) {
        const int n = i >> 6, k = i & 63;
        *reinterpret_cast<bf16*>(S.W3 + umma_off(n, k, kH)) = __float2bfloat16_rn(n < kO ? th[kOffW3 + n * kH + k] : 0.0f);
    }
    for (int i = tid; i < kH; i += kMlpThreads) {
        S.b1[i] = th[kOffB1 + i];
        S.b2[i] = th[kOffB2 + i];
    }
    if (tid < 16) S.b3[tid] = tid < kO ? th[kOffB3 + tid] : 0.0f;
}

// This thread's row of X (24 normalised features, zero-padded to 32; f = nullptr: a zero row).
__device__ __forceinline__ void tc_stage_row(MlpSmemTc& S, const float* f, const float* __restrict__ norm) {
    const int t = threadIdx.x;
#pragma unroll
    for (int k0 = 0; k0 < 32; k0 += 8) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int k = k0 + 2 * q;
            const float x0 = (f && k < kF) ? (f[k] - norm[k]) * norm[kF + k] : 0.0f;
            const float x1 = (f && k + 1 < kF) ? (f[k + 1] - norm[k + 1]) * norm[kF + k + 1] : 0.0f;
            const __nv_bfloat162 p = __floats2bfloat162_rn(x0, x1);
            w[q] = *reinterpret_cast<const uint32_t*>(&p);
        }
        *reinterpret_cast<uint4*>(S.X + umma_off(t, k0, 32)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// TMEM allocation (warp 0; ncols a power of 2 >= 32) and the mbarrier, once per CTA; returns the
// TMEM base address.
__device__ uint32_t tc_begin(MlpSmemTc& S, uint32_t ncols = kTmemCols) {
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&S.tmem)), "r"(ncols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&S.mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return S.tmem;
}

__device__ void tc_end(MlpSmemTc& S, uint32_t tmem, uint32_t ncols = kTmemCols) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(ncols) : "memory");
}

// The forward pass of the tile staged in S.X; y: this thread's 3 outputs.  False (the CTA stops
// using the tensor core) when a wait gave up; the caller then raises KZG_DEVERR_MMA.
// H1t, H2t: transposed copies of the hidden layers for the weight gradients, or null.
__device__ bool forward_tc(MlpSmemTc& S, uint32_t tmem, uint32_t& phase, float (&y)[kO],
                           unsigned char* H1t = nullptr, unsigned char* H2t = nullptr) {
    const uint32_t lane_base = tmem + ((uint32_t)(threadIdx.x & ~31u) << 16);
    tc_sync();
    tc_layer(tmem, S.X, S.W1, 32, kH, &S.mbar);
    if (!tc_wait(&S.mbar, phase)) return false;
    tc_hidden(lane_base, S.b1, S.H1, H1t);
    tc_sync();
    tc_layer(tmem + 64u, S.H1, S.W2, kH, kH, &S.mbar);
    if (!tc_wait(&S.mbar, phase)) return false;
    tc_hidden(lane_base + 64u, S.b2, S.H2, H2t);
    tc_sync();
    tc_layer(tmem, S.H2, S.W3, kH, 16, &S.mbar);
    if (!tc_wait(&S.mbar, phase)) return false;
    float v[16];
    tmem_ld16(lane_base, v);
#pragma unroll
    for (int q = 0; q < kO; ++q) y[q] = v[q] + S.b3[q];
    return true;
}

// ---- features ------------------------------------------------------------------------------
// 24 features of a prepared contact row that missed the cache, in the contact frame (n, t1, t2):
//   0 normal velocity  1-2 tangential velocities  3 penetration depth
//   4-6 rA . (n, t1, t2)   7-9 rB . (n, t1, t2)
//   10-11 log inverse masses   12-13 log n.I^-1 n (A, B)
//   14-16 impulses of the pair's nearest cached point / effective masses (0 without one)
//   17 the pair's cached normal impulse per current point / normal effective mass (0 without)
//   18-20 log effective masses (n, t1, t2)   21 friction   22 restitution bias   23 dt (g . n)
// Mass-like quantities enter as log(x + 1e-6) so that bodies of any size share one scale.
__device__ void row_features(const DeviceBodies& b, const DeviceRows& r, uint32_t A, uint32_t B, uint32_t row,
                             float4 prior, float3 g, float dt, float* f) {
    const Vec3 n = V3(r.n[row]), t1 = V3(r.t1[row]), t2 = V3(r.t2[row]);
    const Vec3 rA = V3(r.rAr[row]), rB = V3(r.rBr[row]);
    const Vec3 rel = (V3(b.lv[A]) + V3(b.av[A]).cross(rA)) - (V3(b.lv[B]) + V3(b.av[B]).cross(rB));
    const float4 m = r.mass[row], bias = r.bias[row];
    const Mat3 IA = M3(&b.iiw[3 * A]), IB = M3(&b.iiw[3 * B]);
    const float eps = 1e-6f;
    f[0] = bias.z;
    f[1] = rel.dot(t1);
    f[2] = rel.dot(t2);
    f[3] = -r.pA[row].w;
    f[4] = rA.dot(n); f[5] = rA.dot(t1); f[6] = rA.dot(t2);
    f[7] = rB.dot(n); f[8] = rB.dot(t1); f[9] = rB.dot(t2);
    f[10] = logf(b.inv_mass[A] + eps);
    f[11] = logf(b.inv_mass[B] + eps);
    f[12] = logf(n.dot(IA * n) + eps);
    f[13] = logf(n.dot(IB * n) + eps);
    f[14] = m.x > 0.0f ? prior.x / m.x : 0.0f;
    f[15] = m.y > 0.0f ? prior.y / m.y : 0.0f;
    f[16] = m.z > 0.0f ? prior.z / m.z : 0.0f;
    f[17] = m.x > 0.0f ? prior.w / m.x : 0.0f;
    f[18] = logf(m.x + eps);
    f[19] = logf(m.y + eps);
    f[20] = logf(m.z + eps);
    f[21] = r.t1[row].w;
    f[22] = bias.x;
    f[23] = dt * ((g.x * n.x + g.y * n.y) + g.z * n.z);
}

// Targets are impulse / effective mass y (m/s), learned as asinh(y / kTargetScale) so that the
// heavy tail of deep-stack contacts does not swamp the loss; predictions map back with sinh,
// limited to |y| <= kTargetScale * sinh(kOutLimit).
constexpr float kTargetScale = 0.05f;
constexpr float kOutLimit = 6.0f;

struct StepView {
    DeviceBodies b;
    DeviceRows r;
    const uint32_t *con_a, *con_b, *miss_rows;
    const float4* miss_prior;
    const Counters* cnt;
    float3 g;
    float dt;
};

// ---- inference: warm start of the cache misses --------------------------------------------
__global__ void __launch_bounds__(kMlpThreads) k_mlp_infer(StepView v, const float* __restrict__ theta,
                                                        const float* __restrict__ norm, float blend_n, float blend_t,
                                                        uint32_t* err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    MlpSmemTc& S = *reinterpret_cast<MlpSmemTc*>(smem_raw);
    const int tid = threadIdx.x;
    const uint32_t nmiss = v.cnt->nmiss;
    if (blockIdx.x * kTile >= nmiss) return;  // the whole CTA: no tile, no tensor memory
    stage_weights_tc(theta, S, tid);
    const uint32_t tmem = tc_begin(S);
    uint32_t phase = 0;
    for (uint32_t base = blockIdx.x * kTile; base < nmiss; base += gridDim.x * kTile) {
        const uint32_t k = base + tid;
        uint32_t row = 0;
        if (k < nmiss) {
            row = v.miss_rows[k];
            const uint32_t c = row >> 2;
            float f[kF];
            row_features(v.b, v.r, v.con_a[c], v.con_b[c], row, v.miss_prior[k], v.g, v.dt, f);
            tc_stage_row(S, f, norm);
        } else {
            tc_stage_row(S, nullptr, norm);
        }
        float y[kO];
        if (!forward_tc(S, tmem, phase, y)) {
            if (tid == 0) atomicOr(err, KZG_DEVERR_MMA);
            tc_drain(&S.mbar, phase);
            break;
        }
        if (k < nmiss) {
            const float4 m = v.r.mass[row];
            const float fric = v.r.t1[row].w;
            for (int q = 0; q < 3; ++q)
                y[q] = (q == 0 ? blend_n : blend_t) * kTargetScale * sinhf(fminf(fmaxf(y[q], -kOutLimit), kOutLimit));
            const float ni = fmaxf(y[0] * m.x, 0.0f);
            const float mf = fric * ni;
            const float t1 = fminf(fmaxf(y[1] * m.y, -mf), mf);
            const float t2 = fminf(fmaxf(y[2] * m.z, -mf), mf);
            const float4 im = v.r.imp[row];
            v.r.imp[row] = make_float4(ni, t1, t2, im.w);
        }
    }
    tc_end(S, tmem);
}

// ---- logging: features before the solve, converged impulses after it ----------------------
__global__ void k_mlp_log_features(StepView v, float* log, const uint32_t* log_n, uint32_t cap) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.cnt->nmiss) return;
    const uint32_t slot = *log_n + k;
    if (slot >= cap) return;
    const uint32_t row = v.miss_rows[k], c = row >> 2;
    float f[kF];
    row_features(v.b, v.r, v.con_a[c], v.con_b[c], row, v.miss_prior[k], v.g, v.dt, f);
    float* o = log + (size_t)slot * kLogFloats;
    for (int i = 0; i < kF; ++i) o[i] = f[i];
}

__global__ void k_mlp_log_targets(StepView v, float* log, const uint32_t* log_n, uint32_t cap) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.cnt->nmiss) return;
    const uint32_t slot = *log_n + k;
    if (slot >= cap) return;
    const uint32_t row = v.miss_rows[k];
    const float4 m = v.r.mass[row], im = v.r.imp[row];
    float* o = log + (size_t)slot * kLogFloats + kF;
    const float ms[3] = {m.x, m.y, m.z}, ls[3] = {im.x, im.y, im.z};
    for (int q = 0; q < 3; ++q) {
        const bool ok = ms[q] > 0.0f;
        o[q] = ok ? ls[q] / ms[q] : 0.0f;
        o[3 + q] = ok ? 1.0f : 0.0f;
    }
}

__global__ void k_mlp_log_advance(const Counters* cnt, uint32_t* log_n, uint32_t cap) {
    *log_n = min(cap, *log_n + cnt->nmiss);
}

// ---- training ------------------------------------------------------------------------------
// ---- training: forward + backward of up to 128 samples per CTA, on tcgen05 -------------------
// After the forward pass (with transposed copies of X, H1, H2), five more products:
//   dH2 = dY W3          (128 x 64, K = 16)   -> dZ2 = dH2 * (H2 > 0)
//   dW3^T = H2^T dY      (64 x 16,  K = 128)
//   dH1 = dZ2 W2         (128 x 64, K = 64)   -> dZ1 = dH1 * (H1 > 0)
//   dW2 = dZ2^T H1       (64 x 64,  K = 128)
//   dW1 = dZ1^T X        (64 x 32,  K = 128)
// The weight gradients have 64 rows: they run as M = 128 products whose A rows 64-127 are read from
// the buffer placed after the A operand (their results land in TMEM lanes that are never read).
// TMEM (256 columns): forward 0-127; dW3^T 0-15, dW1 16-47, dW2 64-127, dH2 128-191, dH1 192-255.
// Bias gradients and the loss are summed over the samples in a fixed order (deterministic).
struct MlpSmemTrainTc {
    MlpSmemTc f;
    alignas(128) unsigned char dY[kTile * 16 * 2];   // A of dH2 (K = 16)
    alignas(128) unsigned char W3T[kH * 16 * 2];     // B of dH2: W3^T, 64 rows of K = 16
    alignas(128) unsigned char dZ2[kTile * kH * 2];  // A of dH1 (K = 64)
    alignas(128) unsigned char W2T[kH * kH * 2];     // B of dH1: W2^T
    alignas(128) unsigned char dZ2t[kH * kTile * 2]; // A of dW2 (rows 64-127: dZ1t)
    alignas(128) unsigned char dZ1t[kH * kTile * 2]; // A of dW1 (rows 64-127: H2t)
    alignas(128) unsigned char H2t[kH * kTile * 2];  // A of dW3^T (rows 64-127: H1t)
    alignas(128) unsigned char H1t[kH * kTile * 2];  // B of dW2
    alignas(128) unsigned char Xt[32 * kTile * 2];   // B of dW1
    alignas(128) unsigned char dYt[16 * kTile * 2];  // B of dW3^T
    float col[kTile * (kH + 1)];                     // per-sample values of the bias sums
    float lred[4], dred[4][kO];
};
constexpr uint32_t kTrainTmemCols = 256;

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
    *reinterpret_cast<bf16*>(base + off) = __float2bfloat16_rn(v);
}

// Epilogue of dH = this thread's 64 accumulators at taddr, masked by the layer's ReLU (H > 0):
// dZ into row t of dZ (when given), column t of dZt and the bias-sum staging.
__device__ __forceinline__ void tc_backprop(uint32_t taddr, const unsigned char* H, unsigned char* dZ,
                                            unsigned char* dZt, float* col) {
    const int t = threadIdx.x;
#pragma unroll
    for (int c0 = 0; c0 < kH; c0 += 16) {
        float v[16];
        tmem_ld16(taddr + (uint32_t)c0, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int c = c0 + i;
            const float h = __bfloat162float(*reinterpret_cast<const bf16*>(H + umma_off(t, c, kH)));
            const float d = h > 0.0f ? v[i] : 0.0f;
            if (dZ) st_bf16(dZ, umma_off(t, c, kH), d);
            st_bf16(dZt, umma_off(c, t, kTile), d);
            col[t * (kH + 1) + c] = d;
        }
    }
}

// Fixed-order sum over the 128 samples of column c of the staging (threads 0-63, one column each).
__device__ __forceinline__ float tc_colsum(const float* col, int c) {
    float s = 0.0f;
    for (int t = 0; t < kTile; ++t) s += col[t * (kH + 1) + c];
    return s;
}

// One CTA: forward + backward of up to 128 samples; writes its partial gradient (kP floats) and
// partial loss.  Loss over the valid outputs, times inv_nvalid: (y - target)^2 (tau = 0), or the
// pinball loss of quantile tau, tau (target - y) above the prediction and (1 - tau) (y - target)
// below it, which fits the tau-quantile of the target instead of its mean.
__global__ void __launch_bounds__(kMlpThreads) k_mlp_train(const float* __restrict__ theta, const float* __restrict__ norm,
                                                        const float* __restrict__ ds, uint32_t first, uint32_t count,
                                                        float inv_nvalid, float tau, float* __restrict__ part,
                                                        float* __restrict__ part_loss, uint32_t* err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    MlpSmemTrainTc& S = *reinterpret_cast<MlpSmemTrainTc*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    stage_weights_tc(theta, S.f, tid);
    for (int i = tid; i < kH * kH; i += kMlpThreads)  // W2T[n][k] = W2[k][n]
        st_bf16(S.W2T, umma_off(i & 63, i >> 6, kH), theta[kOffW2 + i]);
    for (int i = tid; i < kH * 16; i += kMlpThreads) {  // W3T[h][o] = W3[o][h], o padded to 16
        const int h = i >> 4, o = i & 15;
        st_bf16(S.W3T, umma_off(h, o, 16), o < kO ? theta[kOffW3 + o * kH + h] : 0.0f);
    }
    const uint32_t tmem = tc_begin(S.f, kTrainTmemCols);
    const uint32_t lane_base = tmem + ((uint32_t)(tid & ~31) << 16);
    uint32_t phase = 0;
    const uint32_t s = blockIdx.x * kTile + tid;
    const bool valid = s < count;
    const float* rec = ds + (size_t)(first + (valid ? s : 0)) * kLogFloats;
    float f[kF], tgt[3] = {0, 0, 0}, msk[3] = {0, 0, 0};
    for (int i = 0; i < kF; ++i) f[i] = rec[i];
    if (valid)
        for (int q = 0; q < 3; ++q) {
            tgt[q] = rec[kF + q];
            msk[q] = rec[kF + 3 + q];
        }
    tc_stage_row(S.f, valid ? f : nullptr, norm);
    for (int k = 0; k < 32; ++k)
        st_bf16(S.Xt, umma_off(k, tid, kTile), (valid && k < kF) ? (f[k] - norm[k]) * norm[kF + k] : 0.0f);
    float* P = part + (size_t)blockIdx.x * kP;
    bool ok = false;
    do {
        float y[kO];
        if (!forward_tc(S.f, tmem, phase, y, S.H1t, S.H2t)) break;
        // loss and dY (fp32 for the bias gradient, bf16 for the products)
        float loss = 0.0f, dy[3];
        for (int q = 0; q < 3; ++q) {
            const float e = y[q] - tgt[q];
            if (tau > 0.0f) {
                loss += msk[q] * (e > 0.0f ? (1.0f - tau) * e : -tau * e);
                dy[q] = msk[q] * (e > 0.0f ? (1.0f - tau) : -tau) * inv_nvalid;
            } else {
                loss += msk[q] * e * e;
                dy[q] = msk[q] * 2.0f * e * inv_nvalid;
            }
        }
        for (int o = 0; o < 16; ++o) {
            const float v = o < 3 ? dy[o] : 0.0f;
            st_bf16(S.dY, umma_off(tid, o, 16), v);
            st_bf16(S.dYt, umma_off(o, tid, kTile), v);
        }
        {  // loss and db3: warp sums (xor tree), then the four warps in order
            float l = loss * inv_nvalid, d0 = dy[0], d1 = dy[1], d2 = dy[2];
            for (int o = 16; o > 0; o >>= 1) {
                l += __shfl_xor_sync(0xffffffffu, l, o);
                d0 += __shfl_xor_sync(0xffffffffu, d0, o);
                d1 += __shfl_xor_sync(0xffffffffu, d1, o);
                d2 += __shfl_xor_sync(0xffffffffu, d2, o);
            }
            if (lane == 0) {
                S.lred[warp] = l;
                S.dred[warp][0] = d0;
                S.dred[warp][1] = d1;
                S.dred[warp][2] = d2;
            }
        }
        tc_sync();
        tc_chain(tmem + 128u, S.dY, S.W3T, 16, kH);   // dH2
        tc_chain(tmem, S.H2t, S.dYt, kTile, 16);      // dW3^T
        tc_commit(&S.f.mbar);
        if (!tc_wait(&S.f.mbar, phase)) break;
        tc_backprop(lane_base + 128u, S.f.H2, S.dZ2, S.dZ2t, S.col);
        if (warp < 2) {  // dW3^T: row h = TMEM lane h
            float v[16];
            tmem_ld16(lane_base, v);
            for (int o = 0; o < kO; ++o) P[kOffW3 + o * kH + tid] = v[o];
        }
        tc_sync();
        if (tid < kH) P[kOffB2 + tid] = tc_colsum(S.col, tid);
        tc_chain(tmem + 192u, S.dZ2, S.W2T, kH, kH);  // dH1
        tc_chain(tmem + 64u, S.dZ2t, S.H1t, kTile, kH);  // dW2
        tc_commit(&S.f.mbar);
        if (!tc_wait(&S.f.mbar, phase)) break;
        tc_backprop(lane_base + 192u, S.f.H1, nullptr, S.dZ1t, S.col);
        if (warp < 2) {  // dW2: row j = TMEM lane j
#pragma unroll
            for (int c0 = 0; c0 < kH; c0 += 16) {
                float v[16];
                tmem_ld16(lane_base + 64u + (uint32_t)c0, v);
                for (int i = 0; i < 16; ++i) P[kOffW2 + tid * kH + c0 + i] = v[i];
            }
        }
        tc_sync();
        if (tid < kH) P[kOffB1 + tid] = tc_colsum(S.col, tid);
        tc_chain(tmem + 16u, S.dZ1t, S.Xt, kTile, 32);  // dW1
        tc_commit(&S.f.mbar);
        if (!tc_wait(&S.f.mbar, phase)) break;
        if (warp < 2) {  // dW1: row i = TMEM lane i, 24 of its 32 columns
#pragma unroll
            for (int c0 = 0; c0 < 32; c0 += 16) {
                float v[16];
                tmem_ld16(lane_base + 16u + (uint32_t)c0, v);
                for (int i = 0; i < 16; ++i)
                    if (c0 + i < kF) P[kOffW1 + tid * kF + c0 + i] = v[i];
            }
        }
        if (tid < kO) P[kOffB3 + tid] = ((S.dred[0][tid] + S.dred[1][tid]) + S.dred[2][tid]) + S.dred[3][tid];
        if (tid == 0) part_loss[blockIdx.x] = ((S.lred[0] + S.lred[1]) + S.lred[2]) + S.lred[3];
        ok = true;
    } while (false);
    if (!ok) {
        if (tid == 0) atomicOr(err, KZG_DEVERR_MMA);
        tc_drain(&S.f.mbar, phase);
    }
    tc_end(S.f, tmem, kTrainTmemCols);
}

__global__ void k_mlp_reduce(const float* __restrict__ part, const float* __restrict__ part_loss, uint32_t nblk,
                             float* __restrict__ grad, float* __restrict__ loss) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (uint32_t)kP) {
        float s = 0.0f;
        for (uint32_t bidx = 0; bidx < nblk; ++bidx) s += part[(size_t)bidx * kP + i];
        grad[i] = s;
    }
    if (i == 0) {
        float s = 0.0f;
        for (uint32_t bidx = 0; bidx < nblk; ++bidx) s += part_loss[bidx];
        *loss = s;
    }
}

__global__ void k_mlp_adam(float* __restrict__ theta, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ grad, float lr, float bc1, float bc2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)kP) return;
    const float gi = grad[i];
    const float mi = 0.9f * m[i] + 0.1f * gi, vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    theta[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
}

// Forward only over dataset samples (predictions for tests), on the same tensor-core path.
__global__ void __launch_bounds__(kMlpThreads) k_mlp_predict(const float* __restrict__ theta, const float* __restrict__ norm,
                                                          const float* __restrict__ ds, uint32_t first, uint32_t count,
                                                          float* __restrict__ out, uint32_t* err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    MlpSmemTc& S = *reinterpret_cast<MlpSmemTc*>(smem_raw);
    const int tid = threadIdx.x;
    stage_weights_tc(theta, S, tid);
    const uint32_t tmem = tc_begin(S);
    uint32_t phase = 0;
    const uint32_t s = blockIdx.x * kTile + tid;
    const bool valid = s < count;
    float f[kF];
    const float* rec = ds + (size_t)(first + (valid ? s : 0)) * kLogFloats;
    for (int i = 0; i < kF; ++i) f[i] = rec[i];
    tc_stage_row(S, valid ? f : nullptr, norm);
    float y[kO];
    if (forward_tc(S, tmem, phase, y)) {
        if (valid)
            for (int q = 0; q < kO; ++q) out[(size_t)s * kO + q] = y[q];
    } else {
        if (tid == 0) atomicOr(err, KZG_DEVERR_MMA);
        tc_drain(&S.mbar, phase);
    }
    tc_end(S, tmem);
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
#define MLP_CK(x)                                                      \
    do {                                                               \
        cudaError_t e_ = (x);                                          \
        if (e_ != cudaSuccess) {                                       \
            ctx.err = std::string(#x) + ": " + cudaGetErrorString(e_); \
            return KZG_ERR_CUDA;                                       \
        }                                                              \
    } while (0)

cudaError_t mlp_configure_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(MlpSmemTrainTc));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpSmemTc));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpSmemTc));
}

static kzg_status mlp_alloc(Ctx& ctx) {
    MlpState& M = ctx.mlp;
    if (M.theta) return KZG_OK;
    MLP_CK(cudaMalloc(&M.theta, sizeof(float) * kP));
    MLP_CK(cudaMalloc(&M.adam_m, sizeof(float) * kP));
    MLP_CK(cudaMalloc(&M.adam_v, sizeof(float) * kP));
    MLP_CK(cudaMalloc(&M.grad, sizeof(float) * (kP + 1)));
    MLP_CK(cudaMalloc(&M.norm, sizeof(float) * 2 * kF));
    MLP_CK(cudaMalloc(&M.log_n, sizeof(uint32_t)));
    MLP_CK(cudaMemset(M.adam_m, 0, sizeof(float) * kP));
    MLP_CK(cudaMemset(M.adam_v, 0, sizeof(float) * kP));
    MLP_CK(cudaMemset(M.log_n, 0, sizeof(uint32_t)));
    return KZG_OK;
}

void mlp_free(Ctx& ctx) {
    MlpState& M = ctx.mlp;
    for (void* p : {(void*)M.theta, (void*)M.adam_m, (void*)M.adam_v, (void*)M.grad, (void*)M.norm, (void*)M.log_n,
                    (void*)M.log, (void*)M.ds, (void*)M.part, (void*)M.out})
        if (p) cudaFree(p);
    M = MlpState{};
}

kzg_status mlp_set_params(Ctx& ctx, const float* theta, const float* mean, const float* stdv) {
    kzg_status s = mlp_alloc(ctx);
    if (s != KZG_OK) return s;
    std::vector<float> norm(2 * kF);
    for (int i = 0; i < kF; ++i) {
        if (!(stdv[i] > 0.0f)) {
            ctx.err = "feature standard deviations must be > 0";
            return KZG_ERR_INVALID;
        }
        norm[i] = mean[i];
        norm[kF + i] = 1.0f / stdv[i];
    }
    MLP_CK(cudaMemcpy(ctx.mlp.theta, theta, sizeof(float) * kP, cudaMemcpyHostToDevice));
    MLP_CK(cudaMemcpy(ctx.mlp.norm, norm.data(), sizeof(float) * 2 * kF, cudaMemcpyHostToDevice));
    MLP_CK(cudaMemset(ctx.mlp.adam_m, 0, sizeof(float) * kP));
    MLP_CK(cudaMemset(ctx.mlp.adam_v, 0, sizeof(float) * kP));
    ctx.mlp.adam_t = 0;
    ctx.mlp.std.assign(stdv, stdv + kF);
    ctx.mlp.have = true;
    return KZG_OK;
}

kzg_status mlp_get_params(Ctx& ctx, float* theta, float* mean, float* stdv) {
    if (!ctx.mlp.have) {
        ctx.err = "no model parameters set";
        return KZG_ERR_INVALID;
    }
    std::vector<float> norm(2 * kF);
    MLP_CK(cudaMemcpy(theta, ctx.mlp.theta, sizeof(float) * kP, cudaMemcpyDeviceToHost));
    MLP_CK(cudaMemcpy(norm.data(), ctx.mlp.norm, sizeof(float) * 2 * kF, cudaMemcpyDeviceToHost));
    if (mean) std::memcpy(mean, norm.data(), sizeof(float) * kF);
    if (stdv) std::memcpy(stdv, ctx.mlp.std.data(), sizeof(float) * kF);
    return KZG_OK;
}

kzg_status mlp_log_begin(Ctx& ctx, uint32_t capacity) {
    kzg_status s = mlp_alloc(ctx);
    if (s != KZG_OK) return s;
    MlpState& M = ctx.mlp;
    if (M.log) cudaFree(M.log);
    M.log = nullptr;
    if (capacity) MLP_CK(cudaMalloc(&M.log, sizeof(float) * kLogFloats * (size_t)capacity));
    MLP_CK(cudaMemset(M.log_n, 0, sizeof(uint32_t)));
    M.log_cap = capacity;
    M.logging = capacity > 0;
    return KZG_OK;
}

kzg_status mlp_log_fetch(Ctx& ctx, float* out, uint32_t cap, uint32_t* n) {
    MlpState& M = ctx.mlp;
    uint32_t h = 0;
    if (M.log_n) MLP_CK(cudaMemcpy(&h, M.log_n, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    *n = h;
    if (out && h) MLP_CK(cudaMemcpy(out, M.log, sizeof(float) * kLogFloats * std::min(h, cap), cudaMemcpyDeviceToHost));
    return KZG_OK;
}

kzg_status mlp_set_dataset(Ctx& ctx, const float* samples, uint32_t n) {
    kzg_status s = mlp_alloc(ctx);
    if (s != KZG_OK) return s;
    MlpState& M = ctx.mlp;
    if (M.ds) cudaFree(M.ds);
    M.ds = nullptr;
    M.ds_n = n;
    M.ds_valid_prefix.assign(n + 1, 0.0);
    for (uint32_t i = 0; i < n; ++i) {
        const float* m = samples + (size_t)i * kLogFloats + kF + 3;
        M.ds_valid_prefix[i + 1] = M.ds_valid_prefix[i] + (double)(m[0] + m[1] + m[2]);
    }
    if (n) {
        MLP_CK(cudaMalloc(&M.ds, sizeof(float) * kLogFloats * (size_t)n));
        MLP_CK(cudaMemcpy(M.ds, samples, sizeof(float) * kLogFloats * (size_t)n, cudaMemcpyHostToDevice));
    }
    return KZG_OK;
}

// Reads the device error word after an MLP launch outside the step: a tensor-core wait that gave up
// is taken out of the word and returned as KZG_ERR_DEVICE.
static kzg_status take_mma_error(Ctx& ctx) {
    uint32_t e = 0;
    MLP_CK(cudaMemcpyAsync(&e, &ctx.dcnt->error, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream));
    MLP_CK(cudaStreamSynchronize(ctx.stream));
    if (e & KZG_DEVERR_MMA) {
        const uint32_t keep = e & ~KZG_DEVERR_MMA;
        MLP_CK(cudaMemcpy(&ctx.dcnt->error, &keep, sizeof(uint32_t), cudaMemcpyHostToDevice));
        ctx.err = "mlp: a tensor-core wait gave up (KZG_DEVERR_MMA)";
        return KZG_ERR_DEVICE;
    }
    return KZG_OK;
}

static kzg_status mlp_batch_grad(Ctx& ctx, uint32_t first, uint32_t count, float* loss_out) {
    MlpState& M = ctx.mlp;
    if (!M.have || !M.ds || count == 0 || first > M.ds_n || count > M.ds_n - first) {
        ctx.err = "mlp: parameters and a dataset covering [first, first + count) are required";
        return KZG_ERR_INVALID;
    }
    const uint32_t nblk = (count + kTile - 1) / kTile;
    if (nblk > M.part_blocks) {
        if (M.part) cudaFree(M.part);
        M.part = nullptr;
        MLP_CK(cudaMalloc(&M.part, sizeof(float) * ((size_t)nblk * kP + nblk)));
        M.part_blocks = nblk;
    }
    const double nvalid = M.ds_valid_prefix[first + count] - M.ds_valid_prefix[first];
    const float inv = nvalid > 0.0 ? (float)(1.0 / nvalid) : 0.0f;
    float* part_loss = M.part + (size_t)nblk * kP;
    k_mlp_train<<<nblk, kMlpThreads, sizeof(MlpSmemTrainTc), ctx.stream>>>(M.theta, M.norm, M.ds, first, count, inv,
                                                                          M.tau, M.part, part_loss, &ctx.dcnt->error);
    k_mlp_reduce<<<(kP + 255) / 256, 256, 0, ctx.stream>>>(M.part, part_loss, nblk, M.grad, M.grad + kP);
    MLP_CK(cudaGetLastError());
    const kzg_status s = take_mma_error(ctx);  // a tile without gradients: no update from this batch
    if (s != KZG_OK) return s;
    if (loss_out) {
        MLP_CK(cudaMemcpyAsync(loss_out, M.grad + kP, sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
        MLP_CK(cudaStreamSynchronize(ctx.stream));
    }
    return KZG_OK;
}

kzg_status mlp_gradient(Ctx& ctx, uint32_t first, uint32_t count, float* grad, float* loss) {
    kzg_status s = mlp_batch_grad(ctx, first, count, loss);
    if (s != KZG_OK) return s;
    MLP_CK(cudaMemcpyAsync(grad, ctx.mlp.grad, sizeof(float) * kP, cudaMemcpyDeviceToHost, ctx.stream));
    MLP_CK(cudaStreamSynchronize(ctx.stream));
    return KZG_OK;
}

kzg_status mlp_train_step(Ctx& ctx, uint32_t first, uint32_t count, float lr, float* loss) {
    kzg_status s = mlp_batch_grad(ctx, first, count, nullptr);
    if (s != KZG_OK) return s;
    MlpState& M = ctx.mlp;
    ++M.adam_t;
    const float bc1 = 1.0f - std::pow(0.9f, (float)M.adam_t), bc2 = 1.0f - std::pow(0.999f, (float)M.adam_t);
    k_mlp_adam<<<(kP + 255) / 256, 256, 0, ctx.stream>>>(M.theta, M.adam_m, M.adam_v, M.grad, lr, bc1, bc2);
    MLP_CK(cudaGetLastError());
    if (loss) {
        MLP_CK(cudaMemcpyAsync(loss, M.grad + kP, sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
        MLP_CK(cudaStreamSynchronize(ctx.stream));
    }
    return KZG_OK;
}

kzg_status mlp_predict(Ctx& ctx, uint32_t first, uint32_t count, float* out) {
    MlpState& M = ctx.mlp;
    if (!M.have || !M.ds || first > M.ds_n || count > M.ds_n - first) {
        ctx.err = "mlp: parameters and a dataset covering [first, first + count) are required";
        return KZG_ERR_INVALID;
    }
    if (count == 0) return KZG_OK;
    if (count > M.out_cap) {
        if (M.out) cudaFree(M.out);
        M.out = nullptr;
        MLP_CK(cudaMalloc(&M.out, sizeof(float) * kO * (size_t)count));
        M.out_cap = count;
    }
    const uint32_t nblk = (count + kTile - 1) / kTile;
    uint32_t* err = &ctx.dcnt->error;
    k_mlp_predict<<<nblk, kMlpThreads, sizeof(MlpSmemTc), ctx.stream>>>(M.theta, M.norm, M.ds, first, count, M.out, err);
    MLP_CK(cudaGetLastError());
    MLP_CK(cudaMemcpyAsync(out, M.out, sizeof(float) * kO * (size_t)count, cudaMemcpyDeviceToHost, ctx.stream));
    return take_mma_error(ctx);
}

// In-step hooks (kzg_step.cu).  launches: kernels issued.
static StepView step_view(Ctx& ctx, float dt) {
    return StepView{ctx.b, ctx.r, ctx.con_a, ctx.con_b, ctx.miss_rows, ctx.miss_prior, ctx.dcnt,
                    make_float3(ctx.ws.gravity[0], ctx.ws.gravity[1], ctx.ws.gravity[2]), dt};
}

uint32_t mlp_after_prepare(Ctx& ctx, float dt) {
    MlpState& M = ctx.mlp;
    uint32_t n = 0;
    const uint32_t rows = 4u * ctx.cfg.max_pairs;  // grids by capacity: kernels stop at the device count
    if (M.logging) {
        k_mlp_log_features<<<(rows + 255) / 256, 256, 0, ctx.stream>>>(step_view(ctx, dt), M.log, M.log_n, M.log_cap);
        ++n;
    }
    if (M.enabled && M.have) {
        const unsigned grid = std::max(1u, std::min((rows + kTile - 1) / kTile, 152u * 4u));
        k_mlp_infer<<<grid, kMlpThreads, sizeof(MlpSmemTc), ctx.stream>>>(step_view(ctx, dt), M.theta, M.norm,
                                                                         M.blend_n, M.blend_t, &ctx.dcnt->error);
        ++n;
    }
    return n;
}

uint32_t mlp_after_solve(Ctx& ctx, float dt) {
    MlpState& M = ctx.mlp;
    if (!M.logging) return 0;
    const uint32_t rows = 4u * ctx.cfg.max_pairs;
    k_mlp_log_targets<<<(rows + 255) / 256, 256, 0, ctx.stream>>>(step_view(ctx, dt), M.log, M.log_n, M.log_cap);
    k_mlp_log_advance<<<1, 1, 0, ctx.stream>>>(ctx.dcnt, M.log_n, M.log_cap);
    return 2;
}

}  // namespace kzg
