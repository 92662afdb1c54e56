// kzg_solver.cuh - island schedule and sequential-impulse solve (included by kzg_step.cu).
//
// The reference solves each island with (PhysicsWorld.cpp:666-743):
//   1. WarmStart of every constraint in island order                      (:673)
//   2. greedy first-fit batches of at most 4 contact points whose bodies are pairwise distinct
//      (static bodies included), velocity iterations over the batches      (:680-722)
//   3. split-impulse bias iterations over the constraints in island order (:736-742)
// A dynamic body's velocity is a chain of float updates whose order those sweeps fix.  k_schedule
// rebuilds exactly the reference's batches and turns each sweep into dependency levels - a point's
// level is one more than the last level of the same sweep on either of its dynamic bodies - so
// the level-synchronous solve applies every body's updates in the reference's order, bit for bit.
#pragma once

#include <cooperative_groups.h>

#include "kzg_schedule.cuh"
#include "kzg_joint.cuh"

namespace cg = cooperative_groups;

namespace kzg {

// ---------------------------------------------------------------------------------------------
// solve
// ---------------------------------------------------------------------------------------------
struct SolveBufs {
    const uint32_t *isl_start, *con_a, *con_b, *con_bits, *con_la, *con_lb, *meta, *isl_bodies;
    const uint32_t *wl_list, *vl_list, *bl_list, *wl_off, *vl_off, *bl_off;
    const uint32_t *small_list, *large_list;
    DeviceRows r;
    DeviceBodies b;
    uint32_t vel_iters, pos_iters;
    float ws_factor;
    int vel_bias;
    float res_tol;     // > 0: residual-terminated velocity iterations
    uint32_t res_cap;  // their cap
    uint4* vrec;       // big islands: per velocity item {row, A, B, dynamic A | dynamic B << 1} (reuses
                       // the batch-record buffer, free once the schedule is built)
    float4* pk;        // cluster islands: packed velocity items, kPackArrays x pk_cap per cluster
    uint32_t pk_cap;   // points per cluster island (0: no cluster solve)
    const uint32_t* isl_con;  // constraints of each island (sorted)
    uint32_t max_cons;        // constraint capacity
    uint32_t* cl_ids;  // cluster islands: per cluster 2 x kClusterBodies words (new local id of each
                       // local body; body of each new id), then the permuted local ids of A and B
                       // per constraint (2 x max_pairs)
    JointDev* joints;                  // null without joints
    const unsigned long long* jkeys;   // joints sorted by island root, then joint index
    const uint2* jisl;                 // per joint island: its range of jkeys
    const uint32_t* jisl_cisl;         // per joint island: its contact island, or kNone
    const uint32_t* order;   // largest-first island order taken from shared counters, or null (the lists)
    const uint32_t* jflag;   // per island: 1 when joints share it, or null
    uint32_t warp_bodies;    // islands with at most this many dynamic bodies: warp solve
};

// The solve kernel an island goes to (the lists the schedule appends to follow the same rule).
__device__ __forceinline__ bool warp_solved(const SolveBufs& S, uint32_t isl) {
    return !(S.jflag && S.jflag[isl]) && S.meta[4 * isl + 3] <= S.warp_bodies;
}
__device__ __forceinline__ bool cta_solved(const SolveBufs& S, uint32_t isl, uint32_t smem_bodies) {
    const uint32_t nloc = S.meta[4 * isl + 3];
    return !(S.jflag && S.jflag[isl]) && nloc > S.warp_bodies && nloc <= smem_bodies;
}

// Velocity storage of one island: staged in shared memory (local index) or read/written in place
// (global memory, body slot).  Bodies that are not dynamic are never written; their velocity is
// read from global memory (static: zero, kinematic: constant) and their pseudo velocity is zero.
struct VelView {
    float4* v;  // linear  (shared: by local index; global: by slot)
    float4* w;  // angular
    const float4* glv;
    const float4* gav;
    bool shared;
    __device__ __forceinline__ Vec3 lin(uint32_t loc, uint32_t body) const {
        if (loc == kNone) return V3(__ldg(&glv[body]));
        return V3(v[shared ? loc : body]);
    }
    __device__ __forceinline__ Vec3 ang(uint32_t loc, uint32_t body) const {
        if (loc == kNone) return V3(__ldg(&gav[body]));
        return V3(w[shared ? loc : body]);
    }
    __device__ __forceinline__ void put(uint32_t loc, uint32_t body, const Vec3& l, const Vec3& a) const {
        const uint32_t k = shared ? loc : body;
        v[k] = F4(l, 0.0f);
        w[k] = F4(a, 0.0f);
    }
    // pseudo velocities: zero for bodies that are not dynamic
    __device__ __forceinline__ Vec3 plin(uint32_t loc, uint32_t body) const {
        return loc == kNone ? Vec3() : V3(v[shared ? loc : body]);
    }
    __device__ __forceinline__ Vec3 pang(uint32_t loc, uint32_t body) const {
        return loc == kNone ? Vec3() : V3(w[shared ? loc : body]);
    }
};

// Velocity storage of a giant island spread over the shared memory of a thread-block cluster:
// local body l lives in CTA l % kClusterCtas, slot l / kClusterCtas, read and written through
// distributed shared memory.
constexpr uint32_t kClusterCtas = 16;
struct ClusterView {
    float4* v;  // this CTA's arrays; the same offsets in every CTA of the cluster
    float4* w;
    const float4* glv;
    const float4* gav;
    uint32_t rank;  // this CTA's rank: its own bodies are read and written without the cluster mapping
    __device__ __forceinline__ float4* rv(uint32_t loc) const {
        const uint32_t r = loc % kClusterCtas;
        return (r == rank ? v : cg::this_cluster().map_shared_rank(v, r)) + loc / kClusterCtas;
    }
    __device__ __forceinline__ float4* rw(uint32_t loc) const {
        const uint32_t r = loc % kClusterCtas;
        return (r == rank ? w : cg::this_cluster().map_shared_rank(w, r)) + loc / kClusterCtas;
    }
    // The same slots addressed in the cluster's shared window directly (mapa + ld/st.shared::cluster,
    // the own CTA included), without generic-address resolution: the hot path of the packed solve.
    __device__ __forceinline__ uint32_t caddr(const float4* base, uint32_t loc) const {
        const uint32_t a = (uint32_t)__cvta_generic_to_shared(base) + (loc / kClusterCtas) * 16u;
        uint32_t r;
        asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(loc % kClusterCtas));
        return r;
    }
    __device__ __forceinline__ float4 ldc(uint32_t addr) const {
        float4 x;
        asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                     : "=f"(x.x), "=f"(x.y), "=f"(x.z), "=f"(x.w) : "r"(addr));
        return x;
    }
    __device__ __forceinline__ void stc(uint32_t addr, const float4& x) const {
        asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};"
                     :: "r"(addr), "f"(x.x), "f"(x.y), "f"(x.z), "f"(x.w) : "memory");
    }
    __device__ __forceinline__ Vec3 lin(uint32_t loc, uint32_t body) const {
        return loc == kNone ? V3(__ldg(&glv[body])) : V3(*rv(loc));
    }
    __device__ __forceinline__ Vec3 ang(uint32_t loc, uint32_t body) const {
        return loc == kNone ? V3(__ldg(&gav[body])) : V3(*rw(loc));
    }
    __device__ __forceinline__ void put(uint32_t loc, uint32_t, const Vec3& l, const Vec3& a) const {
        *rv(loc) = F4(l, 0.0f);
        *rw(loc) = F4(a, 0.0f);
    }
    __device__ __forceinline__ Vec3 plin(uint32_t loc, uint32_t) const { return loc == kNone ? Vec3() : V3(*rv(loc)); }
    __device__ __forceinline__ Vec3 pang(uint32_t loc, uint32_t) const { return loc == kNone ? Vec3() : V3(*rw(loc)); }
};

// WarmStart for one point (ContactSolver.cpp:117-132 + ApplyImpulsePair :32-43).
template <typename View>
__device__ __forceinline__ void warm_point(const SolveBufs& S, const View& V, uint32_t row) {
    const uint32_t c = row >> 2;
    const uint32_t A = S.con_a[c], B = S.con_b[c], la = __ldcg(&S.con_la[c]), lb = __ldcg(&S.con_lb[c]);
    const float4 im = S.r.imp[row];
    const Vec3 n = V3(S.r.n[row]), t1 = V3(S.r.t1[row]), t2 = V3(S.r.t2[row]);
    const Vec3 imp = ((n * im.x + t1 * im.y) + t2 * im.z) * S.ws_factor;
    if (la != kNone) {
        const Vec3 rA = V3(S.r.rA[row]);
        V.put(la, A, V.lin(la, A) + imp * S.b.inv_mass[A], V.ang(la, A) + M3(&S.b.iiw[3 * A]) * rA.cross(imp));
    }
    if (lb != kNone) {
        const Vec3 rB = V3(S.r.rB[row]);
        V.put(lb, B, V.lin(lb, B) - imp * S.b.inv_mass[B], V.ang(lb, B) - M3(&S.b.iiw[3 * B]) * rB.cross(imp));
    }
}

// One lane of SolveVelocityBatchSIMD (ContactSolverSIMD.cpp:93-256): friction t1, t2 (relative
// velocity recomputed before each axis), then normal; _mm_{add,sub,mul,min,max}_ps semantics.
// Returns the point's share of the island residual: (sum over its rows of |dImpulse|,
// (|n| + |t1|) + |t2| of its accumulated impulses).
// Everything one velocity point reads besides the body velocities (loaded ahead of time by the
// prefetching sweep).
// The normal row's velocity bias: SolveVelocityBatchSIMD adds positionBias or zero to
// restitutionBias (ContactSolverSIMD.cpp), SolveContactVelocity adds positionBias only under
// useVelocityBias (ContactSolver.cpp:167-168).
__device__ __forceinline__ float normal_bias(bool scalar, int vel_bias, const float4 bias) {
    if (scalar) return vel_bias ? bias.x + bias.y : bias.x;
    return bias.x + (vel_bias ? bias.y : 0.0f);
}

struct VelItem {
    uint32_t row, A, B, la, lb;
    float4 rA, rB, n, t1, t2, m, im;  // t1.w = friction
    float nb, invA, invB;
    Mat3 IA, IB;
};

template <bool kScalar>
__device__ __forceinline__ void load_vel_item(const SolveBufs& S, uint32_t row, uint32_t A, uint32_t B, uint32_t la,
                                              uint32_t lb, VelItem& it) {
    it.row = row; it.A = A; it.B = B; it.la = la; it.lb = lb;
    it.rA = S.r.rAr[row];
    it.rB = S.r.rBr[row];
    it.n = S.r.n[row];
    it.t1 = S.r.t1[row];
    it.t2 = S.r.t2[row];
    it.m = S.r.mass[row];
    it.im = S.r.imp[row];
    const float4 bias = S.r.bias[row];  // one 16-byte load (a reference to it loads x and y apart, slower)
    it.nb = normal_bias(kScalar, S.vel_bias, bias);
    it.invA = S.b.inv_mass[A];
    it.invB = S.b.inv_mass[B];
    it.IA = M3(&S.b.iiw[3 * A]);
    it.IB = M3(&S.b.iiw[3 * B]);
}

// The three rows of one lane of SolveVelocityBatchSIMD on loaded data: updates the body
// velocities and the accumulated impulses im (normal, t1, t2) in place and returns the point's
// residual shares.
__device__ __forceinline__ float2 velocity_rows(const Vec3& rA, const Vec3& rB, const float4& n4, const float4& t14,
                                                const float4& t24, const float4& m4, float invA, float invB, float nb,
                                                const Mat3& IA, const Mat3& IB, Vec3& vA, Vec3& wA, Vec3& vB,
                                                Vec3& wB, float4& im) {
    const float fric = t14.w;
    float nacc = im.x, t1acc = im.y, t2acc = im.z;
    float dsum = 0.0f;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        const Vec3 dir = t == 0 ? V3(t14) : (t == 1 ? V3(t24) : V3(n4));
        const Vec3 wa = wA.cross(rA), wb = wB.cross(rB);
        const Vec3 rel((vA.x + wa.x) - (vB.x + wb.x), (vA.y + wa.y) - (vB.y + wb.y), (vA.z + wa.z) - (vB.z + wb.z));
        const float vd = rel.dot(dir);
        float dl;
        if (t < 2) {
            const float mass = t == 0 ? m4.y : m4.z;
            const float acc = t == 0 ? t1acc : t2acc;
            const float lambda = (0.0f - mass) * vd;
            const float maxf = fric * nacc;
            float na = acc + lambda;
            const float lo = 0.0f - maxf;
            na = na > lo ? na : lo;
            na = na < maxf ? na : maxf;
            dl = na - acc;
            if (t == 0) t1acc = na; else t2acc = na;
        } else {
            const float lambda = (0.0f - m4.x) * (vd - nb);
            float na = nacc + lambda;
            na = na > 0.0f ? na : 0.0f;
            dl = na - nacc;
            nacc = na;
        }
        dsum += fabsf(dl);
        const Vec3 imp(dir.x * dl, dir.y * dl, dir.z * dl);
        vA = Vec3(vA.x + imp.x * invA, vA.y + imp.y * invA, vA.z + imp.z * invA);
        wA = wA + IA * rA.cross(imp);
        vB = Vec3(vB.x - imp.x * invB, vB.y - imp.y * invB, vB.z - imp.z * invB);
        wB = wB - IB * rB.cross(imp);
    }
    im = make_float4(nacc, t1acc, t2acc, im.w);
    return make_float2(dsum, (fabsf(nacc) + fabsf(t1acc)) + fabsf(t2acc));
}

// SolveContactVelocity (ContactSolver.cpp:136-181) on loaded data, the scalar solver's point: both
// friction rows take the relative velocity measured before them, the normal row measures it again;
// -mass * v, math::Clamp / math::Max, and impulses reach dynamic bodies only (ApplyImpulsePair).
// Same in-place updates and residual shares as velocity_rows.
__device__ __forceinline__ float2 velocity_rows_scalar(const Vec3& rA, const Vec3& rB, const float4& n4,
                                                       const float4& t14, const float4& t24, const float4& m4,
                                                       float invA, float invB, float nb, const Mat3& IA,
                                                       const Mat3& IB, bool dynA, bool dynB, Vec3& vA, Vec3& wA,
                                                       Vec3& vB, Vec3& wB, float4& im) {
    const float fric = t14.w;
    float nacc = im.x, t1acc = im.y, t2acc = im.z;
    float dsum = 0.0f;
    auto rel = [&]() {
        const Vec3 wa = wA.cross(rA), wb = wB.cross(rB);
        return Vec3((vA.x + wa.x) - (vB.x + wb.x), (vA.y + wa.y) - (vB.y + wb.y), (vA.z + wa.z) - (vB.z + wb.z));
    };
    auto apply = [&](const Vec3& dir, float dl) {
        const Vec3 imp(dir.x * dl, dir.y * dl, dir.z * dl);
        if (dynA) {
            vA = Vec3(vA.x + imp.x * invA, vA.y + imp.y * invA, vA.z + imp.z * invA);
            wA = wA + IA * rA.cross(imp);
        }
        if (dynB) {
            vB = Vec3(vB.x - imp.x * invB, vB.y - imp.y * invB, vB.z - imp.z * invB);
            wB = wB - IB * rB.cross(imp);
        }
    };
    const Vec3 vt = rel();
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const Vec3 dir = t == 0 ? V3(t14) : V3(t24);
        const float mass = t == 0 ? m4.y : m4.z;
        const float acc = t == 0 ? t1acc : t2acc;
        const float lambda = -mass * vt.dot(dir);
        const float maxf = fric * nacc;
        float na = acc + lambda;
        na = na < -maxf ? -maxf : (na > maxf ? maxf : na);
        const float dl = na - acc;
        if (t == 0) t1acc = na; else t2acc = na;
        dsum += fabsf(dl);
        apply(dir, dl);
    }
    const Vec3 n = V3(n4);
    const float lambda = -m4.x * (rel().dot(n) - nb);
    float na = nacc + lambda;
    na = na > 0.0f ? na : 0.0f;
    const float dl = na - nacc;
    nacc = na;
    dsum += fabsf(dl);
    apply(n, dl);
    im = make_float4(nacc, t1acc, t2acc, im.w);
    return make_float2(dsum, (fabsf(nacc) + fabsf(t1acc)) + fabsf(t2acc));
}

// One point of the velocity sweep on a loaded item: a lane of SolveVelocityBatchSIMD, or
// SolveContactVelocity under the scalar solver (kScalar: SolverSettings::useSIMDSolver = false,
// fixed at compile time so that the batch solver's kernels carry no second row routine).
template <bool kScalar, typename View>
__device__ __forceinline__ float2 velocity_item(const SolveBufs& S, const View& V, const VelItem& it) {
    const uint32_t A = it.A, B = it.B, la = it.la, lb = it.lb;
    Vec3 vA = V.lin(la, A), wA = V.ang(la, A), vB = V.lin(lb, B), wB = V.ang(lb, B);
    float4 im = it.im;
    float2 q;
    if constexpr (kScalar)
        q = velocity_rows_scalar(V3(it.rA), V3(it.rB), it.n, it.t1, it.t2, it.m, it.invA, it.invB, it.nb, it.IA, it.IB,
                                 la != kNone, lb != kNone, vA, wA, vB, wB, im);
    else
        q = velocity_rows(V3(it.rA), V3(it.rB), it.n, it.t1, it.t2, it.m, it.invA, it.invB, it.nb, it.IA, it.IB, vA, wA,
                          vB, wB, im);
    if (la != kNone) V.put(la, A, vA, wA);
    if (lb != kNone) V.put(lb, B, vB, wB);
    S.r.imp[it.row] = im;
    return q;
}

template <bool kScalar, typename View>
__device__ __forceinline__ float2 velocity_point_ab(const SolveBufs& S, const View& V, uint32_t row, uint32_t A,
                                                   uint32_t B, uint32_t la, uint32_t lb) {
    VelItem it;
    load_vel_item<kScalar>(S, row, A, B, la, lb, it);
    return velocity_item<kScalar>(S, V, it);
}

template <bool kScalar, typename View>
__device__ __forceinline__ float2 velocity_point(const SolveBufs& S, const View& V, uint32_t row) {
    const uint32_t c = row >> 2;
    return velocity_point_ab<kScalar>(S, V, row, S.con_a[c], S.con_b[c], __ldcg(&S.con_la[c]), __ldcg(&S.con_lb[c]));
}

// Fixed-point (2^-20 N s) magnitude for the residual sums: integer sums are exact and independent
// of the order of the additions, so the stopping iteration does not depend on the thread count.
__device__ __forceinline__ unsigned long long res_fixed(float x) {
    return (unsigned long long)(fminf(x, 1e12f) * 1048576.0f);
}

// SolveBiasConstraint for one point (ContactSolver.cpp:265-289); V holds pseudo velocities.
template <typename View>
__device__ __forceinline__ void bias_point(const SolveBufs& S, const View& V, uint32_t row) {
    const uint32_t c = row >> 2;
    const uint32_t A = S.con_a[c], B = S.con_b[c], la = __ldcg(&S.con_la[c]), lb = __ldcg(&S.con_lb[c]);
    const Vec3 rA = V3(S.r.rAr[row]), rB = V3(S.r.rBr[row]);
    const Vec3 n = V3(S.r.n[row]);
    const float nm = S.r.mass[row].x, pbias = S.r.bias[row].y;
    float4 im = S.r.imp[row];
    const Vec3 pvA = V.plin(la, A), pwA = V.pang(la, A);
    const Vec3 pvB = V.plin(lb, B), pwB = V.pang(lb, B);
    const Vec3 vr = (pvA + pwA.cross(rA)) - (pvB + pwB.cross(rB));
    float lambda = -nm * (vr.dot(n) - pbias);
    const float ni = rmax(im.w + lambda, 0.0f);
    lambda = ni - im.w;
    im.w = ni;
    S.r.imp[row] = im;
    const Vec3 imp = n * lambda;
    if (la != kNone) V.put(la, A, pvA + imp * S.b.inv_mass[A], pwA + M3(&S.b.iiw[3 * A]) * rA.cross(imp));
    if (lb != kNone) V.put(lb, B, pvB - imp * S.b.inv_mass[B], pwB - M3(&S.b.iiw[3 * B]) * rB.cross(imp));
}

// Warm start + velocity sweeps of one island; sync() separates levels.  Velocity iterations run
// the fixed count, or - with a residual tolerance - until the island's residual, the relative
// impulse change sum|dImpulse| / sum|impulse| of an iteration (reduced by sync.sum2), is within
// it, at most res_cap times.
template <bool kScalar, typename Sync, typename View>
__device__ __forceinline__ void solve_velocity(const SolveBufs& S, uint32_t isl, const View& V, uint32_t tid,
                                               uint32_t nthreads, Sync sync, Counters* cnt) {
    const uint32_t base = 4u * S.isl_start[isl];
    const uint32_t loff = base + isl;
    const uint32_t nw = S.meta[4 * isl], nv = S.meta[4 * isl + 1];
    sync.reset(tid);
    for (uint32_t l = 0; l < nw; ++l) {
        const uint32_t e = S.wl_off[loff + l + 1];
        for (uint32_t k = S.wl_off[loff + l] + tid; k < e; k += nthreads) warm_point(S, V, S.wl_list[base + k]);
        sync();
    }
    const bool residual = S.res_tol > 0.0f;
    const uint32_t iters = residual ? S.res_cap : S.vel_iters;
    uint32_t used = 0;
    float res = 0.0f;
    for (uint32_t it = 0; it < iters; ++it) {
        unsigned long long sd = 0, sl = 0;
        for (uint32_t l = 0; l < nv; ++l) {
            const uint32_t e = S.vl_off[loff + l + 1];
            for (uint32_t k = S.vl_off[loff + l] + tid; k < e; k += nthreads) {
                const float2 q = velocity_point<kScalar>(S, V, S.vl_list[base + k]);
                sd += res_fixed(q.x);
                sl += res_fixed(q.y);
            }
            sync();
        }
        used = it + 1;
        if (residual || used == iters) {
            sync.sum2(sd, sl, it);
            res = sl ? (float)((double)sd / (double)sl) : (sd ? 1.0f : 0.0f);
            if (residual && (double)sd <= (double)S.res_tol * (double)sl) break;
        }
    }
    if (tid == 0) {
        atomicMax(&cnt->max_iters, used);
        atomicAdd(&cnt->pt_iters, S.vl_off[loff + nv] * used);
        atomicMax(&cnt->res_bits, __float_as_uint(res));
    }
}

template <typename Sync, typename View>
__device__ __forceinline__ void solve_bias(const SolveBufs& S, uint32_t isl, const View& P, uint32_t tid,
                                           uint32_t nthreads, Sync sync) {
    if (S.vel_bias) return;
    const uint32_t base = 4u * S.isl_start[isl];
    const uint32_t loff = base + isl;
    const uint32_t nbl = S.meta[4 * isl + 2];
    for (uint32_t it = 0; it < S.pos_iters; ++it)
        for (uint32_t l = 0; l < nbl; ++l) {
            const uint32_t e = S.bl_off[loff + l + 1];
            for (uint32_t k = S.bl_off[loff + l] + tid; k < e; k += nthreads) bias_point(S, P, S.bl_list[base + k]);
            sync();
        }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct WarpSync {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
    __device__ __forceinline__ void reset(uint32_t) const {}
    // group-wide sums of the two residual accumulators (every lane gets them)
    __device__ __forceinline__ void sum2(unsigned long long& a, unsigned long long& b, uint32_t) const {
        a = warp_sum(a);
        b = warp_sum(b);
    }
};
// Residual sums go through three rotating pairs of shared words: iteration it accumulates into
// red[it % 3] and clears red[(it + 1) % 3], which was last read two barriers earlier.
struct CtaSync {
    unsigned long long* red;  // 3 x 2 words
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
    __device__ __forceinline__ void reset(uint32_t tid) const {
        if (tid < 6) red[tid] = 0ull;
        __syncthreads();
    }
    __device__ __forceinline__ void sum2(unsigned long long& a, unsigned long long& b, uint32_t it) const {
        a = warp_sum(a);
        b = warp_sum(b);
        unsigned long long* r = red + 2 * (it % 3);
        if ((threadIdx.x & 31u) == 0) {
            atomicAdd(&r[0], a);
            atomicAdd(&r[1], b);
        }
        if (threadIdx.x == 0) {
            unsigned long long* nx = red + 2 * ((it + 1) % 3);
            nx[0] = 0ull;
            nx[1] = 0ull;
        }
        __syncthreads();
        a = r[0];
        b = r[1];
    }
};

// Stage an island's velocities in shared memory, run the warm-start and velocity sweeps, write
// them back; then reuse the same buffers for the split-impulse pseudo velocities and the bias
// sweeps.  Pseudo velocities are loaded, not assumed zero: the position pass clears them only for
// active bodies (PhysicsWorld.cpp:276-290), so a sleeping body solved in an island keeps
// accumulating them until it wakes.
template <bool kScalar, typename Sync>
__device__ __forceinline__ void solve_island_shared(const SolveBufs& S, uint32_t isl, float4* sv, float4* sw,
                                                    uint32_t tid, uint32_t nthreads, Sync sync, Counters* cnt) {
    const uint32_t nloc = S.meta[4 * isl + 3];
    const uint32_t* bodies = S.isl_bodies + 2u * S.isl_start[isl];
    for (uint32_t k = tid; k < nloc; k += nthreads) {
        sv[k] = S.b.lv[bodies[k]];
        sw[k] = S.b.av[bodies[k]];
    }
    sync();
    const VelView V{sv, sw, S.b.lv, S.b.av, true};
    solve_velocity<kScalar>(S, isl, V, tid, nthreads, sync, cnt);
    for (uint32_t k = tid; k < nloc; k += nthreads) {
        S.b.lv[bodies[k]] = sv[k];
        S.b.av[bodies[k]] = sw[k];
        sv[k] = S.b.plv[bodies[k]];
        sw[k] = S.b.pav[bodies[k]];
    }
    sync();
    solve_bias(S, isl, V, tid, nthreads, sync);
    if (!S.vel_bias)
        for (uint32_t k = tid; k < nloc; k += nthreads) {
            S.b.plv[bodies[k]] = sv[k];
            S.b.pav[bodies[k]] = sw[k];
        }
    sync();
}

// Small islands: one warp each.
template <bool kScalar>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_solve_warp(SolveBufs S, Counters* cnt) {
    extern __shared__ float4 smem[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    float4* sv = smem + warp * 2u * kWarpBodies;
    float4* sw = sv + kWarpBodies;
    if (S.order) {  // largest first, from a shared counter
        const uint32_t n = cnt->nislands;
        for (;;) {
            uint32_t k = 0;
            if (lane == 0) k = atomicAdd(&cnt->nx_solve_w, 1u);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= n) break;
            const uint32_t isl = S.order[k];
            if (warp_solved(S, isl)) solve_island_shared<kScalar>(S, isl, sv, sw, lane, 32u, WarpSync{}, cnt);
        }
        return;
    }
    const uint32_t n = cnt->nsmall;
    for (uint32_t idx = blockIdx.x * kWarpsPerBlock + warp; idx < n; idx += gridDim.x * kWarpsPerBlock)
        solve_island_shared<kScalar>(S, S.small_list[idx], sv, sw, lane, 32u, WarpSync{}, cnt);
}

// Large islands whose velocities fit shared memory: one CTA each.
template <bool kScalar>
__global__ void __launch_bounds__(kCtaThreads) k_solve_cta(SolveBufs S, Counters* cnt, uint32_t smem_bodies) {
    extern __shared__ float4 smem[];
    __shared__ unsigned long long red[6];
    __shared__ uint32_t next;
    if (S.order) {  // largest first, from a shared counter
        const uint32_t n = cnt->nislands;
        for (;;) {
            if (threadIdx.x == 0) next = atomicAdd(&cnt->nx_solve_c, 1u);
            __syncthreads();
            const uint32_t k = next;
            __syncthreads();
            if (k >= n) break;
            const uint32_t isl = S.order[k];
            if (cta_solved(S, isl, smem_bodies))
                solve_island_shared<kScalar>(S, isl, smem, smem + smem_bodies, threadIdx.x, blockDim.x, CtaSync{red},
                                             cnt);
        }
        return;
    }
    const uint32_t n = cnt->nlarge;
    for (uint32_t idx = blockIdx.x; idx < n; idx += gridDim.x) {
        const uint32_t isl = S.large_list[idx];
        if (S.meta[4 * isl + 3] > smem_bodies) continue;
        solve_island_shared<kScalar>(S, isl, smem, smem + smem_bodies, threadIdx.x, blockDim.x, CtaSync{red}, cnt);
    }
}

// Islands too large for shared memory: one 1024-thread CTA each, velocities updated in place
// (L2-resident).  A level of a settled pile holds ~1,000 points, one per thread.
constexpr uint32_t kBigThreads = 768;
constexpr uint32_t kBigOffs = 8192;  // velocity level offsets staged in shared memory

// Warm start + velocity sweeps of a big island.  Each velocity item is one 16-byte record
// {row, A, B, dynamic flags}, and every thread loads its record of the next level before it solves
// the current one, so after a barrier only the row and body loads stand between it and its math.
struct NoHook {
    __device__ void operator()() const {}
};
// after_warm runs on every thread between the warm-start sweep and the velocity sweeps.
template <bool kScalar, typename AfterWarm = NoHook>
__device__ void solve_velocity_big(const SolveBufs& S, uint32_t isl, uint32_t* soff, unsigned long long* red,
                                   Counters* cnt, AfterWarm after_warm = AfterWarm{}) {
    const uint32_t tid = threadIdx.x, nthreads = blockDim.x;
    const uint32_t base = 4u * S.isl_start[isl], loff = base + isl;
    const uint32_t nw = S.meta[4 * isl], nv = S.meta[4 * isl + 1];
    const VelView V{S.b.lv, S.b.av, S.b.lv, S.b.av, false};
    const CtaSync sync{red};
    const uint32_t total = S.vl_off[loff + nv];
    for (uint32_t k = tid; k < total; k += nthreads) {
        const uint32_t row = S.vl_list[base + k], c = row >> 2;
        S.vrec[base + k] = make_uint4(row, S.con_a[c], S.con_b[c],
                                      (S.con_la[c] != kNone ? 1u : 0u) | (S.con_lb[c] != kNone ? 2u : 0u));
    }
    const bool staged = nv <= kBigOffs;
    if (staged)
        for (uint32_t l = tid; l <= nv; l += nthreads) soff[l] = S.vl_off[loff + l];
    sync.reset(tid);
    for (uint32_t l = 0; l < nw; ++l) {
        const uint32_t e = S.wl_off[loff + l + 1];
        for (uint32_t k = S.wl_off[loff + l] + tid; k < e; k += nthreads) warm_point(S, V, S.wl_list[base + k]);
        sync();
    }
    after_warm();
    auto off = [&](uint32_t l) -> uint32_t { return staged ? soff[l] : S.vl_off[loff + l]; };
    auto item = [&](const uint4& r) -> float2 {
        return velocity_point_ab<kScalar>(S, V, r.x, r.y, r.z, (r.w & 1u) ? 0u : kNone, (r.w & 2u) ? 0u : kNone);
    };
    const bool residual = S.res_tol > 0.0f;
    const uint32_t iters = residual ? S.res_cap : S.vel_iters;
    uint32_t used = 0;
    float res = 0.0f;
    uint4 cur = make_uint4(kNone, 0u, 0u, 0u);
    if (iters && nv && off(0) + tid < off(1)) cur = S.vrec[base + off(0) + tid];
    for (uint32_t it = 0; it < iters; ++it) {
        unsigned long long sd = 0, sl = 0;
        for (uint32_t l = 0; l < nv; ++l) {
            const uint32_t lo = off(l), hi = off(l + 1);
            const uint32_t ln = l + 1 < nv ? l + 1 : 0u;  // after the last level: the next iteration's first
            const uint32_t nlo = off(ln), nhi = off(ln + 1);
            uint4 nxt = make_uint4(kNone, 0u, 0u, 0u);
            if (nlo + tid < nhi) nxt = S.vrec[base + nlo + tid];
            if (cur.x != kNone) {
                const float2 q = item(cur);
                sd += res_fixed(q.x);
                sl += res_fixed(q.y);
            }
            for (uint32_t k = lo + tid + nthreads; k < hi; k += nthreads) {
                const float2 q = item(S.vrec[base + k]);
                sd += res_fixed(q.x);
                sl += res_fixed(q.y);
            }
            sync();
            cur = nxt;
        }
        used = it + 1;
        if (residual || used == iters) {
            sync.sum2(sd, sl, it);
            res = sl ? (float)((double)sd / (double)sl) : (sd ? 1.0f : 0.0f);
            if (residual && (double)sd <= (double)S.res_tol * (double)sl) break;
        }
    }
    if (tid == 0) {
        atomicMax(&cnt->max_iters, used);
        atomicAdd(&cnt->pt_iters, total * used);
        atomicMax(&cnt->res_bits, __float_as_uint(res));
    }
}

__device__ __forceinline__ bool cluster_island(const SolveBufs& S, uint32_t isl, uint32_t smem_bodies);

// An island holding joints, in the reference's order (PhysicsWorld.cpp:666-743): contact warm start,
// joint warm starts, contact velocity sweeps, the joints' velocity iterations (the configured count;
// the residual rule stops the contact sweeps only), contact bias sweeps.  The contact parts run
// level-parallel on the CTA (as in k_solve_big), the joint parts on thread 0 in joint order.
// Called functions, so that the register allocation of k_solve_big's own contact sweeps stays as
// it is without joints.
static __device__ __noinline__ void joints_warm(const DeviceBodies b, JointDev* J, const unsigned long long* jk,
                                                uint2 r) {
    const JBodies B{b};
    for (uint32_t s = r.x; s < r.y; ++s) joint_warm(B, J[(uint32_t)jk[s]]);
}
static __device__ __noinline__ void joints_velocity(const DeviceBodies b, JointDev* J, const unsigned long long* jk,
                                                    uint2 r, uint32_t iters) {
    const JBodies B{b};
    for (uint32_t it = 0; it < iters; ++it)
        for (uint32_t s = r.x; s < r.y; ++s) joint_velocity(B, J[(uint32_t)jk[s]]);
}

template <bool kScalar>
__device__ __forceinline__ void solve_joint_island(const SolveBufs& S, uint32_t k, uint32_t* soff,
                                                   unsigned long long* red, Counters* cnt) {
    const uint2 r = S.jisl[k];
    const uint32_t cisl = S.jisl_cisl[k];
    auto warm = [&]() {
        if (threadIdx.x == 0) joints_warm(S.b, S.joints, S.jkeys, r);
        __syncthreads();
    };
    if (cisl != kNone) solve_velocity_big<kScalar>(S, cisl, soff, red, cnt, warm);
    else warm();
    if (threadIdx.x == 0) joints_velocity(S.b, S.joints, S.jkeys, r, S.vel_iters);
    __syncthreads();
    if (cisl != kNone) {
        const VelView P{S.b.plv, S.b.pav, S.b.lv, S.b.av, false};
        solve_bias(S, cisl, P, threadIdx.x, blockDim.x, CtaSync{red});
    }
    __syncthreads();
}

// Large islands that neither one CTA's shared memory nor (when S.pk_cap > 0) a cluster takes.
template <bool kScalar>
__global__ void __launch_bounds__(kBigThreads, 1) k_solve_big(SolveBufs S, Counters* cnt, uint32_t smem_bodies) {
    __shared__ unsigned long long red[6];
    __shared__ uint32_t soff[kBigOffs + 1];
    const uint32_t n = cnt->nlarge;
    for (uint32_t idx = blockIdx.x; idx < n; idx += gridDim.x) {
        const uint32_t isl = S.large_list[idx];
        if (S.meta[4 * isl + 3] <= smem_bodies || (S.pk_cap && cluster_island(S, isl, smem_bodies))) continue;
        const VelView P{S.b.plv, S.b.pav, S.b.lv, S.b.av, false};
        solve_velocity_big<kScalar>(S, isl, soff, red, cnt);
        solve_bias(S, isl, P, threadIdx.x, blockDim.x, CtaSync{red});
        __syncthreads();
    }
}

// Islands that hold joints (launched only when the world has joints): one CTA each.  Joint islands
// are usually small (a chain, a ragdoll), so the CTAs are small and several share an SM.
constexpr uint32_t kJointThreads = 128;
template <bool kScalar>
__global__ void __launch_bounds__(kJointThreads) k_solve_joint(SolveBufs S, Counters* cnt) {
    __shared__ unsigned long long red[6];
    __shared__ uint32_t soff[kBigOffs + 1];
    const uint32_t nj = cnt->njisl;
    for (uint32_t idx = blockIdx.x; idx < nj; idx += gridDim.x) solve_joint_island<kScalar>(S, idx, soff, red, cnt);
}

// ---------------------------------------------------------------------------------------------
// Giant islands on a thread-block cluster
// ---------------------------------------------------------------------------------------------
// A settled pile is one island of ~20k bodies whose dependency levels hold ~1,000 points each.
// One CTA is bound by its own L2 bandwidth and latency on every level; here kClusterCtas CTAs on
// as many SMs share each level, the island's velocities live in their distributed shared memory
// (ClusterView) and a hardware cluster barrier separates the levels.
constexpr uint32_t kClusterThreads = 256;
constexpr uint32_t kClusterSlots = 6144;  // bodies per CTA: 2 x 16 B x 6144 = 192 KB
constexpr uint32_t kClusterBodies = kClusterCtas * kClusterSlots;

// The two halves of a cluster barrier (every thread of every CTA of the cluster, in order, once each
// per phase): arrive with release semantics for the shared-memory stores before it, wait with
// acquire semantics for the loads after it.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Level barrier and residual sums over the whole cluster: every CTA sums its warps into its own
// rotating words (as CtaSync does), and after the barrier every thread adds the kClusterCtas partial
// sums it reads through distributed shared memory.
struct ClusterSync {
    unsigned long long* red;  // 3 x 2 words per CTA
    __device__ __forceinline__ void operator()() const { cg::this_cluster().sync(); }
    __device__ __forceinline__ void reset(uint32_t) const {
        if (threadIdx.x < 6) red[threadIdx.x] = 0ull;
        cg::this_cluster().sync();
    }
    __device__ __forceinline__ void sum2(unsigned long long& a, unsigned long long& b, uint32_t it) const {
        cg::cluster_group cl = cg::this_cluster();
        a = warp_sum(a);
        b = warp_sum(b);
        unsigned long long* r = red + 2 * (it % 3);
        if ((threadIdx.x & 31u) == 0) {
            atomicAdd(&r[0], a);
            atomicAdd(&r[1], b);
        }
        if (threadIdx.x == 0) {
            unsigned long long* nx = red + 2 * ((it + 1) % 3);
            nx[0] = 0ull;
            nx[1] = 0ull;
        }
        cl.sync();
        a = 0ull;
        b = 0ull;
        for (uint32_t k = 0; k < kClusterCtas; ++k) {
            const unsigned long long* rk = cl.map_shared_rank(r, k);
            a += rk[0];
            b += rk[1];
        }
    }
};

// Packed velocity items of a cluster island: kPackArrays float4 arrays of pk_cap entries per cluster
// (structure of arrays).  Every point belongs to the CTA that holds its first dynamic body (so that
// body's velocity is local shared memory); each CTA's points form one region, in velocity-level
// order.  The points a warp solves in one level are consecutive, so every field is one coalesced
// 16-byte load with no index to chase.
//   0 rA, inverse mass A     1 rB, inverse mass B      2 normal, velocity bias   3 t1, friction
//   4 t2, local A            5 masses, local B         6-10 inverse inertias of A and B (9 + 9
//   floats), 10.z = row      11 accumulated impulses   12, 13 linear and angular velocity of the
//   body that is not dynamic (constant during the solve; zero when both are dynamic)
constexpr uint32_t kPackArrays = 14;
constexpr uint32_t kPackCapMax = 1u << 19;
constexpr uint32_t kClusterGrid = 2;     // clusters launched; more giant islands queue on them
constexpr uint32_t kClusterOffs = 4096;  // velocity levels staged in shared memory

struct PackItem {
    float4 q[kPackArrays];
};

// The fields of a point's packed item, gathered from its row and bodies.
template <bool kScalar>
__device__ __forceinline__ void gather_item(const SolveBufs& S, uint32_t row, PackItem& it) {
    const uint32_t c = row >> 2;
    const uint32_t A = S.con_a[c], B = S.con_b[c], la = __ldcg(&S.con_la[c]), lb = __ldcg(&S.con_lb[c]);
    const float4 rA = S.r.rAr[row], rB = S.r.rBr[row], bias = S.r.bias[row];
    const float4 n = S.r.n[row], t2 = S.r.t2[row], m = S.r.mass[row];
    const Mat3 IA = M3(&S.b.iiw[3 * A]), IB = M3(&S.b.iiw[3 * B]);
    const uint32_t st = la == kNone ? A : (lb == kNone ? B : kNone);
    it.q[0] = make_float4(rA.x, rA.y, rA.z, S.b.inv_mass[A]);
    it.q[1] = make_float4(rB.x, rB.y, rB.z, S.b.inv_mass[B]);
    it.q[2] = make_float4(n.x, n.y, n.z, normal_bias(kScalar, S.vel_bias, bias));
    it.q[3] = S.r.t1[row];
    it.q[4] = make_float4(t2.x, t2.y, t2.z, __uint_as_float(la));
    it.q[5] = make_float4(m.x, m.y, m.z, __uint_as_float(lb));
    it.q[6] = make_float4(IA.c0.x, IA.c0.y, IA.c0.z, IA.c1.x);
    it.q[7] = make_float4(IA.c1.y, IA.c1.z, IA.c2.x, IA.c2.y);
    it.q[8] = make_float4(IA.c2.z, IB.c0.x, IB.c0.y, IB.c0.z);
    it.q[9] = make_float4(IB.c1.x, IB.c1.y, IB.c1.z, IB.c2.x);
    it.q[10] = make_float4(IB.c2.y, IB.c2.z, __uint_as_float(row), 0.0f);
    it.q[11] = S.r.imp[row];
    it.q[12] = st == kNone ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : S.b.lv[st];
    it.q[13] = st == kNone ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : S.b.av[st];
}

__device__ __forceinline__ void store_pack(float4* pk, uint32_t cap, uint32_t k, const PackItem& it) {
#pragma unroll
    for (uint32_t j = 0; j < kPackArrays; ++j) pk[j * cap + k] = it.q[j];
}

__device__ __forceinline__ void load_pack(const float4* pk, uint32_t cap, uint32_t k, PackItem& it) {
#pragma unroll
    for (uint32_t j = 0; j < kPackArrays; ++j) it.q[j] = __ldcg(&pk[j * cap + k]);
}

// The CTA of the cluster that holds a point's first dynamic body.
__device__ __forceinline__ uint32_t point_owner(const SolveBufs& S, uint32_t row) {
    const uint32_t c = row >> 2, la = __ldcg(&S.con_la[c]);
    return (la != kNone ? la : __ldcg(&S.con_lb[c])) % kClusterCtas;
}

// Velocity loads of a packed item: the dynamic bodies' from distributed shared memory, the other
// body's from the item.
struct PackVel {
    Vec3 vA, wA, vB, wB;
};
__device__ __forceinline__ PackVel pack_velocities(const ClusterView& V, const PackItem& it) {
    const uint32_t la = __float_as_uint(it.q[4].w), lb = __float_as_uint(it.q[5].w);
    PackVel p;
    p.vA = la != kNone ? V3(V.ldc(V.caddr(V.v, la))) : V3(it.q[12]);
    p.wA = la != kNone ? V3(V.ldc(V.caddr(V.w, la))) : V3(it.q[13]);
    p.vB = lb != kNone ? V3(V.ldc(V.caddr(V.v, lb))) : V3(it.q[12]);
    p.wB = lb != kNone ? V3(V.ldc(V.caddr(V.w, lb))) : V3(it.q[13]);
    return p;
}

// Solves a packed item whose velocities are loaded; stores the velocities and returns the
// accumulated impulses in `im_out` (stored by the caller: the same thread reads them back next
// iteration, so they need not be ordered before the level barrier).
__device__ __forceinline__ float2 pack_solve(const ClusterView& V, uint32_t k, const PackItem& it, PackVel& p,
                                             float4& im_out, bool scalar) {
    const float4* q = it.q;
    const Mat3 IA{V3(q[6]), Vec3(q[6].w, q[7].x, q[7].y), Vec3(q[7].z, q[7].w, q[8].x)};
    const Mat3 IB{Vec3(q[8].y, q[8].z, q[8].w), V3(q[9]), Vec3(q[9].w, q[10].x, q[10].y)};
    float4 im = q[11];
    const uint32_t la = __float_as_uint(q[4].w), lb = __float_as_uint(q[5].w);
    const float2 r = scalar ? velocity_rows_scalar(V3(q[0]), V3(q[1]), q[2], q[3], q[4], q[5], q[0].w, q[1].w, q[2].w,
                                                   IA, IB, la != kNone, lb != kNone, p.vA, p.wA, p.vB, p.wB, im)
                            : velocity_rows(V3(q[0]), V3(q[1]), q[2], q[3], q[4], q[5], q[0].w, q[1].w, q[2].w, IA,
                                            IB, p.vA, p.wA, p.vB, p.wB, im);
    if (la != kNone) {
        V.stc(V.caddr(V.v, la), F4(p.vA, 0.0f));
        V.stc(V.caddr(V.w, la), F4(p.wA, 0.0f));
    }
    if (lb != kNone) {
        V.stc(V.caddr(V.v, lb), F4(p.vB, 0.0f));
        V.stc(V.caddr(V.w, lb), F4(p.wB, 0.0f));
    }
    im_out = im;
    return r;
}

// Warm-start and bias points of a cluster island, loaded ahead: each thread loads its point of the
// next level while it applies the current one (nothing a level writes is read by these loads but
// the velocities, which are not part of them).
struct WarmItem {
    uint32_t A, B, la, lb;
    float4 im, n, t1, t2, rA, rB;
    float iA, iB;
    Mat3 IA, IB;
};
__device__ __forceinline__ void load_warm(const SolveBufs& S, uint32_t row, WarmItem& w) {
    const uint32_t c = row >> 2;
    w.A = S.con_a[c];
    w.B = S.con_b[c];
    w.la = __ldcg(&S.con_la[c]);
    w.lb = __ldcg(&S.con_lb[c]);
    w.im = S.r.imp[row];
    w.n = S.r.n[row];
    w.t1 = S.r.t1[row];
    w.t2 = S.r.t2[row];
    w.rA = S.r.rA[row];
    w.rB = S.r.rB[row];
    w.iA = S.b.inv_mass[w.A];
    w.iB = S.b.inv_mass[w.B];
    w.IA = M3(&S.b.iiw[3 * w.A]);
    w.IB = M3(&S.b.iiw[3 * w.B]);
}
// WarmStart for one loaded point (the arithmetic of warm_point).
template <typename View>
__device__ __forceinline__ void apply_warm(const SolveBufs& S, const View& V, const WarmItem& w) {
    const Vec3 imp = ((V3(w.n) * w.im.x + V3(w.t1) * w.im.y) + V3(w.t2) * w.im.z) * S.ws_factor;
    if (w.la != kNone) V.put(w.la, w.A, V.lin(w.la, w.A) + imp * w.iA, V.ang(w.la, w.A) + w.IA * V3(w.rA).cross(imp));
    if (w.lb != kNone) V.put(w.lb, w.B, V.lin(w.lb, w.B) - imp * w.iB, V.ang(w.lb, w.B) - w.IB * V3(w.rB).cross(imp));
}

// Bias points load only their indices ahead (registers are short); their row and body data are
// independent loads issued together at the level.
struct BiasIdx {
    uint32_t row, A, B, la, lb;
};
__device__ __forceinline__ void load_bias_idx(const SolveBufs& S, uint32_t row, BiasIdx& b) {
    const uint32_t c = row >> 2;
    b.row = row;
    b.A = S.con_a[c];
    b.B = S.con_b[c];
    b.la = __ldcg(&S.con_la[c]);
    b.lb = __ldcg(&S.con_lb[c]);
}
// SolveBiasConstraint for one point (the arithmetic of bias_point).
template <typename View>
__device__ __forceinline__ void apply_bias(const SolveBufs& S, const View& V, const BiasIdx& b) {
    const uint32_t row = b.row, A = b.A, B = b.B, la = b.la, lb = b.lb;
    const Vec3 rA = V3(S.r.rAr[row]), rB = V3(S.r.rBr[row]);
    const Vec3 n = V3(S.r.n[row]);
    const float nm = S.r.mass[row].x, pbias = S.r.bias[row].y;
    float4 im = S.r.imp[row];
    const float iA = S.b.inv_mass[A], iB = S.b.inv_mass[B];
    const Mat3 IA = M3(&S.b.iiw[3 * A]), IB = M3(&S.b.iiw[3 * B]);
    const Vec3 pvA = V.plin(la, A), pwA = V.pang(la, A);
    const Vec3 pvB = V.plin(lb, B), pwB = V.pang(lb, B);
    const Vec3 vr = (pvA + pwA.cross(rA)) - (pvB + pwB.cross(rB));
    float lambda = -nm * (vr.dot(n) - pbias);
    const float ni = rmax(im.w + lambda, 0.0f);
    lambda = ni - im.w;
    im.w = ni;
    S.r.imp[row] = im;
    const Vec3 imp = n * lambda;
    if (la != kNone) V.put(la, A, pvA + imp * iA, pwA + IA * rA.cross(imp));
    if (lb != kNone) V.put(lb, B, pvB - imp * iB, pwB - IB * rB.cross(imp));
}

// One pass over a sweep's levels (list/off at the island's regions), each thread taking the points
// gtid, gtid + gthreads, ... of a level, its first point of the next level loaded ahead.
template <typename Item, typename Sync, typename Load, typename Apply>
__device__ __forceinline__ void sweep_prefetched(const uint32_t* list, const uint32_t* off, uint32_t base,
                                                 uint32_t loff, uint32_t nl, uint32_t gtid, uint32_t gthreads,
                                                 Sync sync, Load load, Apply apply) {
    Item cur, nxt;
    bool has_cur = nl && off[loff] + gtid < off[loff + 1];
    if (has_cur) load(list[base + off[loff] + gtid], cur);
    for (uint32_t l = 0; l < nl; ++l) {
        const uint32_t lo = off[loff + l], hi = off[loff + l + 1];
        bool has_nxt = false;
        if (l + 1 < nl) {
            const uint32_t kn = hi + gtid;
            has_nxt = kn < off[loff + l + 2];
            if (has_nxt) load(list[base + kn], nxt);
        }
        if (has_cur) apply(cur);
        for (uint32_t k = lo + gtid + gthreads; k < hi; k += gthreads) {  // wide levels
            Item x;
            load(list[base + k], x);
            apply(x);
        }
        sync();
        cur = nxt;
        has_cur = has_nxt;
    }
}

// Warm start + velocity sweeps of a cluster island on packed items.  The points are first
// partitioned: each level's points go to the CTAs holding their first dynamic bodies (counted into
// every CTA's level table soff, scanned there, then packed at region start + level offset + rank).
// Before a thread solves its point of a level it loads its packed point of the next one - nothing
// the current level writes - so after each barrier only the velocity loads stand between it and its
// math.  Needs at least two velocity levels (the prefetched point must differ from the current one).
template <bool kScalar, typename Sync>
__device__ void solve_velocity_packed(const SolveBufs& S, uint32_t isl, const ClusterView& V, float4* pk,
                                      uint32_t* soff, uint32_t* lofs, uint32_t* rall, uint32_t* tmp, uint32_t rank,
                                      uint32_t gtid, uint32_t gthreads, Sync sync, Counters* cnt) {
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t cap = S.pk_cap, tid = threadIdx.x, nthr = blockDim.x;
    const uint32_t base = 4u * S.isl_start[isl], loff = base + isl;
    const uint32_t nw = S.meta[4 * isl], nv = S.meta[4 * isl + 1];
    const uint32_t total = S.vl_off[loff + nv];
    // ---- partition: counts per (level, owner); a point's rank inside its group goes to vrec.x.
    // Both passes walk the island's points flat, kB per thread at once so that their loads overlap;
    // a point's level comes from the level offsets staged in lofs.
    for (uint32_t l = tid; l <= nv; l += nthr) {
        soff[l] = 0;
        lofs[l] = S.vl_off[loff + l];
    }
    cl.sync();
    auto level_of = [&](uint32_t k) -> uint32_t {  // the level l with lofs[l] <= k < lofs[l + 1]
        uint32_t lo = 0, hi = nv;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (lofs[mid] <= k) lo = mid; else hi = mid;
        }
        return lo;
    };
    constexpr uint32_t kB = 4;
    for (uint32_t k0 = gtid; k0 < total; k0 += kB * gthreads) {
        uint32_t rw[kB], lv[kB], ow[kB];
#pragma unroll
        for (uint32_t j = 0; j < kB; ++j) {
            const uint32_t k = k0 + j * gthreads;
            rw[j] = k < total ? S.vl_list[base + k] : 0u;
            lv[j] = k < total ? level_of(k) : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < kB; ++j) ow[j] = k0 + j * gthreads < total ? point_owner(S, rw[j]) : 0u;
#pragma unroll
        for (uint32_t j = 0; j < kB; ++j)
            if (k0 + j * gthreads < total)
                S.vrec[base + k0 + j * gthreads].x = atomicAdd(cl.map_shared_rank(soff, ow[j]) + lv[j], 1u);
    }
    cl.sync();
    {  // exclusive scan of this CTA's level counts; soff[nv] = its points
        const uint32_t chunk = (nv + nthr - 1) / nthr;
        const uint32_t lo = min(nv, tid * chunk), hi = min(nv, lo + chunk);
        uint32_t part = 0;
        for (uint32_t l = lo; l < hi; ++l) part += soff[l];
        uint32_t run = group_scan(part, tid, nthr, tmp, &soff[nv + 1], CtaSync{nullptr});
        for (uint32_t l = lo; l < hi; ++l) {
            const uint32_t c = soff[l];
            soff[l] = run;
            run += c;
        }
        __syncthreads();
        if (tid == 0) soff[nv] = soff[nv + 1];
    }
    cl.sync();
    if (tid < kClusterCtas) rall[tid] = cl.map_shared_rank(soff, tid)[nv];
    __syncthreads();
    if (tid == 0)
        for (uint32_t r = 0, run = 0; r < kClusterCtas; ++r) {
            const uint32_t c = rall[r];
            rall[r] = run;
            run += c;
        }
    __syncthreads();
    for (uint32_t k = gtid; k < total; k += gthreads) {
        const uint32_t row = S.vl_list[base + k], o = point_owner(S, row);
        const uint32_t pos = rall[o] + cl.map_shared_rank(soff, o)[level_of(k)] + S.vrec[base + k].x;
        PackItem x;
        gather_item<kScalar>(S, row, x);
        store_pack(pk, cap, pos, x);
    }
    const uint32_t R = rall[rank];
    sync.reset(gtid);  // a cluster barrier: every packed point is visible
    sweep_prefetched<WarmItem>(S.wl_list, S.wl_off, base, loff, nw, gtid, gthreads, sync,
                               [&](uint32_t row, WarmItem& w) { load_warm(S, row, w); },
                               [&](const WarmItem& w) { apply_warm(S, V, w); });
    const bool residual = S.res_tol > 0.0f;
    const uint32_t iters = residual ? S.res_cap : S.vel_iters;
    uint32_t used = 0;
    float res = 0.0f;
    PackItem cur;
    uint32_t kc = R + soff[0] + tid;
    bool has_cur = iters && kc < R + soff[1];
    if (has_cur) load_pack(pk, cap, kc, cur);
    for (uint32_t it = 0; it < iters; ++it) {
        unsigned long long sd = 0, sl = 0;
        // Levels are separated by a split cluster barrier: a thread arrives (release) once its
        // level's velocities are stored and waits (acquire) only before it reads velocities again,
        // with its bookkeeping for the next level in between.
        for (uint32_t l = 0; l < nv; ++l) {
            const uint32_t ln = l + 1 < nv ? l + 1 : 0u;  // after the last level: the next iteration's first
            const uint32_t kn = R + soff[ln] + tid;
            const bool has_nxt = kn < R + soff[ln + 1];
            if (l > 0) cluster_wait();
            PackVel pv;
            if (has_cur) pv = pack_velocities(V, cur);  // issued first: the level's critical path
            PackItem nxt;
            if (has_nxt) load_pack(pk, cap, kn, nxt);
            float4 imc;
            if (has_cur) {
                const float2 q = pack_solve(V, kc, cur, pv, imc, kScalar);
                sd += res_fixed(q.x);
                sl += res_fixed(q.y);
            }
            for (uint32_t k = R + soff[l] + tid + nthr; k < R + soff[l + 1]; k += nthr) {  // wide levels
                PackItem x;
                load_pack(pk, cap, k, x);
                PackVel px = pack_velocities(V, x);
                float4 imx;
                const float2 q = pack_solve(V, k, x, px, imx, kScalar);
                pk[11 * cap + k] = imx;
                sd += res_fixed(q.x);
                sl += res_fixed(q.y);
            }
            cluster_arrive();
            if (has_cur) pk[11 * cap + kc] = imc;  // after the arrive: only this thread reads it again
            cur = nxt;
            kc = kn;
            has_cur = has_nxt;
        }
        if (nv > 0) cluster_wait();
        used = it + 1;
        if (residual || used == iters) {
            sync.sum2(sd, sl, it);
            res = sl ? (float)((double)sd / (double)sl) : (sd ? 1.0f : 0.0f);
            if (residual && (double)sd <= (double)S.res_tol * (double)sl) break;
        }
    }
    for (uint32_t k = R + tid; k < R + soff[nv]; k += nthr)  // the accumulated impulses back to their rows
        S.r.imp[__float_as_uint(pk[10 * cap + k].z)] = pk[11 * cap + k];
    if (gtid == 0) {
        atomicMax(&cnt->max_iters, used);
        atomicAdd(&cnt->pt_iters, total * used);
        atomicMax(&cnt->res_bits, __float_as_uint(res));
    }
}

// Whether k_solve_cluster solves a large island (k_solve_big takes the rest of those that do not fit
// one CTA's shared memory).
__device__ __forceinline__ bool cluster_island(const SolveBufs& S, uint32_t isl, uint32_t smem_bodies) {
    const uint32_t nloc = S.meta[4 * isl + 3], nv = S.meta[4 * isl + 1];
    if (nloc <= smem_bodies || nloc > kClusterCtas * kClusterSlots || nv > kClusterOffs) return false;
    const uint32_t base = 4u * S.isl_start[isl];
    return S.vl_off[base + isl + nv] <= S.pk_cap;
}

// Spatial ownership of a cluster island's bodies: CTA t holds the bodies whose x-z position falls in
// tile t of a kTilesX x kTilesZ grid over the island - contacts join near bodies, so most points
// find both velocities in one CTA's shared memory (8-CTA clusters of 4 x 2 tiles solved the settled
// pile in 15.1 ms against 11.2 ms for 16 CTAs of 4 x 4).  The tiles hold equal shares of the
// bodies: kTilesX strips at the quantiles of x, each cut at the quantiles of its bodies' z
// (kHistBins-bin histograms over the island's extent, gathered in CTA 0's `hist`).  Equal-area
// tiles gave the centre of a pile 4.8 times the points of a corner per level, and every level
// waited for the centre CTAs.  New local ids are slot * kClusterCtas + tile (the
// ClusterView mapping); if a tile overflows its kClusterSlots slots the island keeps its ids.
// Writes the new ids of the island's constraints (SC.con_la / SC.con_lb) and its bodies by new id;
// returns how many bodies this CTA holds.  Every read of what it writes goes through L2.
constexpr uint32_t kTilesX = 4, kTilesZ = kClusterCtas / kTilesX;
static_assert(kTilesX * kTilesZ == kClusterCtas, "cluster_layout tiles the island kTilesX x kTilesZ");
constexpr uint32_t kHistBins = 256;
constexpr uint32_t kHistWords = kHistBins * (1 + kTilesX) + (kTilesX - 1) + kTilesX * (kTilesZ - 1);
__device__ __forceinline__ uint32_t hist_bin(float v, float v0, float s) {
    return min(kHistBins - 1u, (uint32_t)fmaxf(0.0f, (v - v0) * s));
}
// The kCuts bins at which the running count of h[0..kHistBins) first reaches q / (kCuts + 1) of n.
template <uint32_t kCuts>
__device__ __forceinline__ void hist_cuts(const uint32_t* h, uint32_t n, uint32_t* cut) {
    uint32_t run = 0, q = 0;
    for (uint32_t b = 0; b < kHistBins && q < kCuts; ++b) {
        run += h[b];
        while (q < kCuts && (uint64_t)run * (kCuts + 1) >= (uint64_t)(q + 1) * n) cut[q++] = b;
    }
    while (q < kCuts) cut[q++] = kHistBins - 1u;
}
// The piece a bin falls in: how many cuts lie below it.
template <uint32_t kCuts>
__device__ __forceinline__ uint32_t hist_piece(const uint32_t* cut, uint32_t b) {
    uint32_t t = 0;
#pragma unroll
    for (uint32_t q = 0; q < kCuts; ++q) t += b > cut[q] ? 1u : 0u;
    return t;
}

__device__ uint32_t cluster_layout(const SolveBufs& S, const SolveBufs& SC, uint32_t isl, uint32_t* ids,
                                   uint32_t* sc, float* sbb, uint32_t* hist, uint32_t rank, uint32_t gtid,
                                   uint32_t gthreads) {
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const uint32_t nloc = S.meta[4 * isl + 3], s0 = S.isl_start[isl], s1 = S.isl_start[isl + 1];
    const uint32_t* bodies = S.isl_bodies + 2u * s0;
    uint32_t* newid = ids;                     // by old local id
    uint32_t* body_of = ids + kClusterBodies;  // by new local id
    // island extent in x and z: warp partials in sbb[4 * warp ..], the CTA's in sbb[0..3]
    float mnx = 3.0e38f, mxx = -3.0e38f, mnz = 3.0e38f, mxz = -3.0e38f;
    for (uint32_t l = gtid; l < nloc; l += gthreads) {
        const float4 p = S.b.pos[bodies[l]];
        mnx = fminf(mnx, p.x);
        mxx = fmaxf(mxx, p.x);
        mnz = fminf(mnz, p.z);
        mxz = fmaxf(mxz, p.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, o));
        mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
    }
    if (lane == 0) {
        sbb[4 + 4 * warp + 0] = mnx;
        sbb[4 + 4 * warp + 1] = mxx;
        sbb[4 + 4 * warp + 2] = mnz;
        sbb[4 + 4 * warp + 3] = mxz;
    }
    __syncthreads();
    if (tid == 0) {
        for (uint32_t w = 1; w < nwarps; ++w) {
            mnx = fminf(mnx, sbb[4 + 4 * w + 0]);
            mxx = fmaxf(mxx, sbb[4 + 4 * w + 1]);
            mnz = fminf(mnz, sbb[4 + 4 * w + 2]);
            mxz = fmaxf(mxz, sbb[4 + 4 * w + 3]);
        }
        sbb[0] = mnx;
        sbb[1] = mxx;
        sbb[2] = mnz;
        sbb[3] = mxz;
        sc[0] = 0;  // bodies this CTA holds
    }
    cl.sync();
    if (tid == 0) {
        for (uint32_t r = 0; r < kClusterCtas; ++r) {
            const float* o = cl.map_shared_rank(sbb, r);
            mnx = fminf(mnx, o[0]);
            mxx = fmaxf(mxx, o[1]);
            mnz = fminf(mnz, o[2]);
            mxz = fmaxf(mxz, o[3]);
        }
        sbb[36] = mnx;
        sbb[37] = (float)kHistBins / fmaxf(mxx - mnx, 1.0e-6f);
        sbb[38] = mnz;
        sbb[39] = (float)kHistBins / fmaxf(mxz - mnz, 1.0e-6f);
    }
    if (rank == 0)
        for (uint32_t k = tid; k < kHistWords; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    cl.sync();
    const float x0 = sbb[36], sx = sbb[37], z0 = sbb[38], sz = sbb[39];
    uint32_t* h0 = cl.map_shared_rank(hist, 0);  // x histogram, then one z histogram per strip, then the cuts
    uint32_t* xcut = h0 + kHistBins * (1 + kTilesX);
    uint32_t* zcut = xcut + (kTilesX - 1);
    for (uint32_t l = gtid; l < nloc; l += gthreads) atomicAdd(&h0[hist_bin(S.b.pos[bodies[l]].x, x0, sx)], 1u);
    cl.sync();
    if (rank == 0 && tid == 0) hist_cuts<kTilesX - 1>(hist, nloc, hist + kHistBins * (1 + kTilesX));
    cl.sync();
    uint32_t xc[kTilesX - 1];
#pragma unroll
    for (uint32_t q = 0; q < kTilesX - 1; ++q) xc[q] = xcut[q];
    for (uint32_t l = gtid; l < nloc; l += gthreads) {
        const float4 p = S.b.pos[bodies[l]];
        const uint32_t ix = hist_piece<kTilesX - 1>(xc, hist_bin(p.x, x0, sx));
        atomicAdd(&h0[kHistBins * (1 + ix) + hist_bin(p.z, z0, sz)], 1u);
    }
    cl.sync();
    if (rank == 0 && tid < kTilesX) {
        const uint32_t* hz = hist + kHistBins * (1 + tid);
        uint32_t n = 0;
        for (uint32_t b = 0; b < kHistBins; ++b) n += hz[b];
        hist_cuts<kTilesZ - 1>(hz, n, hist + kHistBins * (1 + kTilesX) + (kTilesX - 1) + tid * (kTilesZ - 1));
    }
    cl.sync();
    uint32_t zc[kTilesX][kTilesZ - 1];
#pragma unroll
    for (uint32_t i = 0; i < kTilesX; ++i)
#pragma unroll
        for (uint32_t q = 0; q < kTilesZ - 1; ++q) zc[i][q] = zcut[i * (kTilesZ - 1) + q];
    for (uint32_t l = gtid; l < nloc; l += gthreads) {
        const float4 p = S.b.pos[bodies[l]];
        const uint32_t ix = hist_piece<kTilesX - 1>(xc, hist_bin(p.x, x0, sx));
        uint32_t iz = 0;
        const uint32_t bz = hist_bin(p.z, z0, sz);
#pragma unroll
        for (uint32_t i = 0; i < kTilesX; ++i)
            if (i == ix) iz = hist_piece<kTilesZ - 1>(zc[i], bz);
        const uint32_t t = ix * kTilesZ + iz;
        const uint32_t slot = atomicAdd(cl.map_shared_rank(sc, t), 1u);
        newid[l] = slot * kClusterCtas + t;
    }
    cl.sync();
    if (tid == 0) {  // a full tile: keep the plain ids
        uint32_t over = 0;
        for (uint32_t r = 0; r < kClusterCtas; ++r) over |= cl.map_shared_rank(sc, r)[0] > kClusterSlots ? 1u : 0u;
        sc[1] = over;
    }
    __syncthreads();
    const bool plain = sc[1] != 0u;
    for (uint32_t l = gtid; l < nloc; l += gthreads) {  // the same thread wrote newid[l]
        const uint32_t n = plain ? l : newid[l];
        if (plain) newid[l] = l;
        body_of[n] = bodies[l];
    }
    cl.sync();
    uint32_t* la = const_cast<uint32_t*>(SC.con_la);
    uint32_t* lb = const_cast<uint32_t*>(SC.con_lb);
    for (uint32_t k = s0 + gtid; k < s1; k += gthreads) {
        const uint32_t c = S.isl_con[k], a = S.con_la[c], b = S.con_lb[c];
        la[c] = a == kNone ? kNone : __ldcg(&newid[a]);
        lb[c] = b == kNone ? kNone : __ldcg(&newid[b]);
    }
    cl.sync();
    return plain ? (nloc + kClusterCtas - 1 - rank) / kClusterCtas : sc[0];
}

// Islands with more than smem_bodies and at most kClusterCtas * kClusterSlots dynamic bodies.
// kScalar: SolverSettings::useSIMDSolver = false, fixed at compile time so that the batch
// solver's level loop carries no second row routine.
template <bool kScalar>
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterThreads, 1)
    k_solve_cluster(SolveBufs S, Counters* cnt, uint32_t smem_bodies) {
    extern __shared__ float4 smem[];
    __shared__ unsigned long long red[6];
    __shared__ uint32_t soff[kClusterOffs + 2], lofs[kClusterOffs + 1];  // soff: cluster_layout's histograms first
    static_assert(kHistWords <= kClusterOffs + 2, "the layout histograms live in soff");
    __shared__ uint32_t rall[kClusterCtas], tmp[33], sc[2];
    __shared__ float sbb[40];
    cg::cluster_group cl = cg::this_cluster();
    float4* sv = smem;
    float4* sw = smem + kClusterSlots;
    const uint32_t rank = cl.block_rank(), tid = threadIdx.x;
    const uint32_t gtid = rank * blockDim.x + tid, gthreads = kClusterCtas * blockDim.x;
    const uint32_t ncl = gridDim.x / kClusterCtas, cid = blockIdx.x / kClusterCtas;
    const uint32_t n = cnt->nlarge;
    const ClusterView V{sv, sw, S.b.lv, S.b.av, rank};
    const ClusterSync sync{red};
    SolveBufs SC = S;  // the island's constraints with permuted local ids
    SC.con_la = S.cl_ids + 2u * kClusterGrid * kClusterBodies;
    SC.con_lb = SC.con_la + S.max_cons;
    uint32_t* ids = S.cl_ids + 2u * kClusterBodies * cid;
    const uint32_t* body_of = ids + kClusterBodies;
    for (uint32_t idx = cid; idx < n; idx += ncl) {  // the same islands in every CTA of a cluster
        const uint32_t isl = S.large_list[idx];
        if (!cluster_island(S, isl, smem_bodies)) continue;
        const uint32_t nown = cluster_layout(S, SC, isl, ids, sc, sbb, soff, rank, gtid, gthreads);
        for (uint32_t k = tid; k < nown; k += blockDim.x) {
            const uint32_t b = __ldcg(&body_of[k * kClusterCtas + rank]);
            sv[k] = S.b.lv[b];
            sw[k] = S.b.av[b];
        }
        cl.sync();
        if (S.meta[4 * isl + 1] >= 2)  // prefetching needs two distinct levels
            solve_velocity_packed<kScalar>(SC, isl, V, S.pk + (size_t)cid * kPackArrays * S.pk_cap, soff, lofs, rall, tmp, rank,
                                  gtid, gthreads, sync, cnt);
        else
            solve_velocity<kScalar>(SC, isl, V, gtid, gthreads, sync, cnt);
        for (uint32_t k = tid; k < nown; k += blockDim.x) {
            const uint32_t b = __ldcg(&body_of[k * kClusterCtas + rank]);
            S.b.lv[b] = sv[k];
            S.b.av[b] = sw[k];
            sv[k] = S.b.plv[b];  // pseudo velocities (non-zero only for sleeping bodies)
            sw[k] = S.b.pav[b];
        }
        cl.sync();
        if (!S.vel_bias) {
            const uint32_t base = 4u * S.isl_start[isl], loff = base + isl, nbl = S.meta[4 * isl + 2];
            for (uint32_t it = 0; it < S.pos_iters; ++it)
                sweep_prefetched<BiasIdx>(S.bl_list, S.bl_off, base, loff, nbl, gtid, gthreads, sync,
                                          [&](uint32_t row, BiasIdx& b) { load_bias_idx(SC, row, b); },
                                          [&](const BiasIdx& b) { apply_bias(SC, V, b); });
        }
        if (!S.vel_bias)
            for (uint32_t k = tid; k < nown; k += blockDim.x) {
                const uint32_t b = __ldcg(&body_of[k * kClusterCtas + rank]);
                S.b.plv[b] = sv[k];
                S.b.pav[b] = sw[k];
            }
        cl.sync();
    }
}

}  // namespace kzg
