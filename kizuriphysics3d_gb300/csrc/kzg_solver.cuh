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

namespace kzg {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kHubMin = 24;        // points on one body in one island that make it a hub
constexpr uint32_t kWarpBodies = 384;   // island velocities staged per warp (warp-per-island solve)
constexpr uint32_t kWarpsPerBlock = 4;
constexpr uint32_t kCtaThreads = 256;
constexpr uint32_t kCtaBodiesMax = 6400;  // island velocities staged per CTA (2 x 16 B x 6400 = 200 KB)

struct SchedBufs {
    const uint32_t *isl_start, *isl_con, *con_a, *con_b, *con_np, *con_bits;
    const float4* bias;
    const float* inv_mass;
    uint32_t frame;
    uint32_t *bcnt, *bbody, *bmem;      // batch count, 8 bodies, 4 point rows per batch
    uint32_t *onx, *hnx0, *hnx1;        // skip structures (next usable batch), region base + 2*isl
    uint32_t *body_stamp, *body_loc, *body_cnt;
    uint32_t *isl_bodies, *last_local;  // per island dynamic bodies / level scratch, region 2*s0
    uint32_t *con_la, *con_lb;          // per constraint: local index of A / B (kNone if not dynamic)
    uint32_t *lvl_tmp, *ids_tmp, *lvl_count;
    uint32_t *wl_list, *vl_list, *bl_list, *wl_off, *vl_off, *bl_off, *meta;
    uint32_t *small_list, *large_list;
};

// smallest usable batch index >= i (path halving; every link points forward)
__device__ __forceinline__ uint32_t nx_find(uint32_t* nx, uint32_t i) {
    for (;;) {
        uint32_t p = nx[i];
        if (p == i) return i;
        uint32_t gp = nx[p];
        nx[i] = gp;
        i = gp;
    }
}

__device__ __forceinline__ bool batch_has(const uint32_t* bbody, uint32_t cntb, uint32_t x) {
    for (uint32_t k = 0; k < 2 * cntb; ++k)
        if (bbody[k] == x) return true;
    return false;
}

__device__ void sched_sort(uint32_t base, uint32_t loff, uint32_t npts, uint32_t nlev, const uint32_t* pts_level,
                           const uint32_t* pts_id, uint32_t* count, uint32_t* list, uint32_t* off) {
    // counting sort of npts points by level (levels 1..nlev) into list[base..], offsets off[loff..]
    for (uint32_t l = 0; l <= nlev; ++l) count[loff + l] = 0;
    for (uint32_t k = 0; k < npts; ++k) count[loff + pts_level[base + k] - 1]++;
    uint32_t run = 0;
    for (uint32_t l = 0; l < nlev; ++l) {
        uint32_t c = count[loff + l];
        off[loff + l] = run;
        count[loff + l] = run;
        run += c;
    }
    off[loff + nlev] = run;
    for (uint32_t k = 0; k < npts; ++k) list[base + count[loff + pts_level[base + k] - 1]++] = pts_id[base + k];
}

__global__ void k_schedule(SchedBufs S, Counters* cnt) {
    uint32_t isl = blockIdx.x * blockDim.x + threadIdx.x;
    if (isl >= cnt->nislands) return;
    const uint32_t s0 = S.isl_start[isl], s1 = S.isl_start[isl + 1];
    const uint32_t base = 4u * s0;      // point region of this island
    const uint32_t loff = base + isl;   // level-offset region (one extra entry per island)
    const uint32_t xoff = base + 2u * isl;  // skip-structure region (two extra entries)
    const uint32_t boff = 2u * s0;      // body region
    uint32_t* lvl = S.lvl_tmp;
    uint32_t* ids = S.ids_tmp;

    // ---- local indices of the island's dynamic bodies; points per body (hub detection)
    uint32_t nloc = 0;
    for (uint32_t s = s0; s < s1; ++s) {
        const uint32_t c = S.isl_con[s];
        const uint32_t bits = S.con_bits[c], a = S.con_a[c], b = S.con_b[c], np = S.con_np[c];
        uint32_t la = kNone, lb = kNone;
        if (bits & 2u) {
            if (S.body_stamp[a] != S.frame) {
                S.body_stamp[a] = S.frame;
                S.body_loc[a] = nloc;
                S.isl_bodies[boff + nloc++] = a;
            }
            la = S.body_loc[a];
        }
        if (bits & 4u) {
            if (S.body_stamp[b] != S.frame) {
                S.body_stamp[b] = S.frame;
                S.body_loc[b] = nloc;
                S.isl_bodies[boff + nloc++] = b;
            }
            lb = S.body_loc[b];
        }
        S.con_la[c] = la;
        S.con_lb[c] = lb;
        if (!(bits & 1u)) {
            S.body_cnt[a] += np;
            S.body_cnt[b] += np;
        }
    }
    uint32_t hub0 = kNone, hub1 = kNone, c0 = kHubMin - 1, c1 = kHubMin - 1;
    for (uint32_t s = s0; s < s1; ++s) {
        const uint32_t c = S.isl_con[s];
        const uint32_t xs[2] = {S.con_a[c], S.con_b[c]};
        for (int q = 0; q < 2; ++q) {
            const uint32_t x = xs[q];
            const uint32_t k = S.body_cnt[x];
            if (x == hub0 || x == hub1 || k <= c1) continue;
            if (k > c0) { hub1 = hub0; c1 = c0; hub0 = x; c0 = k; }
            else { hub1 = x; c1 = k; }
        }
    }
    for (uint32_t s = s0; s < s1; ++s) {
        const uint32_t c = S.isl_con[s];
        S.body_cnt[S.con_a[c]] = 0;
        S.body_cnt[S.con_b[c]] = 0;
    }

    // ---- greedy first-fit batching (constraint order, then point index).  onx finds the first
    // batch that is not full; hnxK the first that is not full and does not hold hub K.
    uint32_t* onx = S.onx + xoff;
    uint32_t* hx0 = S.hnx0 + xoff;
    uint32_t* hx1 = S.hnx1 + xoff;
    onx[0] = 0; hx0[0] = 0; hx1[0] = 0;
    uint32_t nbt = 0;
    for (uint32_t s = s0; s < s1; ++s) {
        const uint32_t c = S.isl_con[s];
        if (S.con_bits[c] & 1u) continue;  // sensors are never batched (:690)
        const uint32_t a = S.con_a[c], b = S.con_b[c];
        const int ha = a == hub0 ? 0 : (a == hub1 ? 1 : -1);
        const int hb = b == hub0 ? 0 : (b == hub1 ? 1 : -1);
        for (uint32_t p = 0; p < S.con_np[c]; ++p) {
            uint32_t j;
            if (ha >= 0 || hb >= 0) {
                const int h = ha >= 0 ? ha : hb;
                const uint32_t other = ha >= 0 ? b : a;
                uint32_t* hx = h == 0 ? hx0 : hx1;
                j = nx_find(hx, 0);
                while (j < nbt && batch_has(&S.bbody[8u * (base + j)], S.bcnt[base + j], other)) j = nx_find(hx, j + 1);
            } else {
                j = nx_find(onx, 0);
                while (j < nbt && (batch_has(&S.bbody[8u * (base + j)], S.bcnt[base + j], a) ||
                                   batch_has(&S.bbody[8u * (base + j)], S.bcnt[base + j], b)))
                    j = nx_find(onx, j + 1);
            }
            if (j == nbt) {  // new batch
                S.bcnt[base + j] = 0;
                ++nbt;
                onx[nbt] = nbt; hx0[nbt] = nbt; hx1[nbt] = nbt;
            }
            const uint32_t k = S.bcnt[base + j];
            S.bbody[8u * (base + j) + 2 * k] = a;
            S.bbody[8u * (base + j) + 2 * k + 1] = b;
            S.bmem[4u * (base + j) + k] = 4u * c + p;
            S.bcnt[base + j] = k + 1;
            if (k + 1 == 4u) { onx[j] = j + 1; hx0[j] = j + 1; hx1[j] = j + 1; }
            if (ha == 0 || hb == 0) hx0[j] = j + 1;
            if (ha == 1 || hb == 1) hx1[j] = j + 1;
        }
    }

    uint32_t* last = S.last_local + boff;
    // ---- velocity levels in batch order
    for (uint32_t k = 0; k < nloc; ++k) last[k] = 0;
    uint32_t nv = 0, nvpts = 0;
    for (uint32_t bi = 0; bi < nbt; ++bi) {
        const uint32_t cntb = S.bcnt[base + bi];
        for (uint32_t k = 0; k < cntb; ++k) {
            const uint32_t pt = S.bmem[4u * (base + bi) + k];
            const uint32_t c = pt >> 2, la = S.con_la[c], lb = S.con_lb[c];
            uint32_t l = 0;
            if (la != kNone) l = max(l, last[la]);
            if (lb != kNone) l = max(l, last[lb]);
            ++l;
            if (la != kNone) last[la] = l;
            if (lb != kNone) last[lb] = l;
            nv = max(nv, l);
            lvl[base + nvpts] = l;
            ids[base + nvpts] = pt;
            ++nvpts;
        }
    }
    sched_sort(base, loff, nvpts, nv, lvl, ids, S.lvl_count, S.vl_list, S.vl_off);

    // ---- warm-start levels: every point, constraint order
    for (uint32_t k = 0; k < nloc; ++k) last[k] = 0;
    uint32_t nw = 0, nwpts = 0;
    for (uint32_t s = s0; s < s1; ++s) {
        const uint32_t c = S.isl_con[s], la = S.con_la[c], lb = S.con_lb[c];
        for (uint32_t p = 0; p < S.con_np[c]; ++p) {
            uint32_t l = 0;
            if (la != kNone) l = max(l, last[la]);
            if (lb != kNone) l = max(l, last[lb]);
            ++l;
            if (la != kNone) last[la] = l;
            if (lb != kNone) last[lb] = l;
            nw = max(nw, l);
            lvl[base + nwpts] = l;
            ids[base + nwpts] = 4u * c + p;
            ++nwpts;
        }
    }
    sched_sort(base, loff, nwpts, nw, lvl, ids, S.lvl_count, S.wl_list, S.wl_off);

    // ---- bias levels: points with positionBias > 0 of constraints with a massive body
    for (uint32_t k = 0; k < nloc; ++k) last[k] = 0;
    uint32_t nbl = 0, nbpts = 0;
    for (uint32_t s = s0; s < s1; ++s) {
        const uint32_t c = S.isl_con[s];
        if (S.inv_mass[S.con_a[c]] <= 0.0f && S.inv_mass[S.con_b[c]] <= 0.0f) continue;
        const uint32_t la = S.con_la[c], lb = S.con_lb[c];
        for (uint32_t p = 0; p < S.con_np[c]; ++p) {
            if (S.bias[4u * c + p].y <= 0.0f) continue;
            uint32_t l = 0;
            if (la != kNone) l = max(l, last[la]);
            if (lb != kNone) l = max(l, last[lb]);
            ++l;
            if (la != kNone) last[la] = l;
            if (lb != kNone) last[lb] = l;
            nbl = max(nbl, l);
            lvl[base + nbpts] = l;
            ids[base + nbpts] = 4u * c + p;
            ++nbpts;
        }
    }
    sched_sort(base, loff, nbpts, nbl, lvl, ids, S.lvl_count, S.bl_list, S.bl_off);

    S.meta[4 * isl + 0] = nw;
    S.meta[4 * isl + 1] = nv;
    S.meta[4 * isl + 2] = nbl;
    S.meta[4 * isl + 3] = nloc;
    if (nloc <= kWarpBodies) S.small_list[atomicAdd(&cnt->nsmall, 1u)] = isl;
    else S.large_list[atomicAdd(&cnt->nlarge, 1u)] = isl;
    atomicAdd(&cnt->batches, nbt);
    atomicMax(&cnt->max_vlev, nv);
    atomicMax(&cnt->max_blev, nbl);
}

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
};

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
};

// WarmStart for one point (ContactSolver.cpp:117-132 + ApplyImpulsePair :32-43).
__device__ __forceinline__ void warm_point(const SolveBufs& S, const VelView& V, uint32_t row) {
    const uint32_t c = row >> 2;
    const uint32_t A = S.con_a[c], B = S.con_b[c], la = S.con_la[c], lb = S.con_lb[c];
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
__device__ __forceinline__ void velocity_point(const SolveBufs& S, const VelView& V, uint32_t row) {
    const uint32_t c = row >> 2;
    const uint32_t A = S.con_a[c], B = S.con_b[c], la = S.con_la[c], lb = S.con_lb[c];
    const Vec3 rA = V3(S.r.rAr[row]), rB = V3(S.r.rBr[row]);
    const float4 n4 = S.r.n[row], t14 = S.r.t1[row], t24 = S.r.t2[row], m4 = S.r.mass[row];
    const float4 im = S.r.imp[row];
    const float4 bias = S.r.bias[row];
    const float invA = S.b.inv_mass[A], invB = S.b.inv_mass[B];
    const Mat3 IA = M3(&S.b.iiw[3 * A]), IB = M3(&S.b.iiw[3 * B]);
    Vec3 vA = V.lin(la, A), wA = V.ang(la, A), vB = V.lin(lb, B), wB = V.ang(lb, B);
    const float nb = bias.x + (S.vel_bias ? bias.y : 0.0f);
    const float fric = t14.w;
    float nacc = im.x, t1acc = im.y, t2acc = im.z;
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
        const Vec3 imp(dir.x * dl, dir.y * dl, dir.z * dl);
        vA = Vec3(vA.x + imp.x * invA, vA.y + imp.y * invA, vA.z + imp.z * invA);
        wA = wA + IA * rA.cross(imp);
        vB = Vec3(vB.x - imp.x * invB, vB.y - imp.y * invB, vB.z - imp.z * invB);
        wB = wB - IB * rB.cross(imp);
    }
    if (la != kNone) V.put(la, A, vA, wA);
    if (lb != kNone) V.put(lb, B, vB, wB);
    S.r.imp[row] = make_float4(nacc, t1acc, t2acc, im.w);
}

// SolveBiasConstraint for one point (ContactSolver.cpp:265-289); V holds pseudo velocities.
__device__ __forceinline__ void bias_point(const SolveBufs& S, const VelView& V, uint32_t row) {
    const uint32_t c = row >> 2;
    const uint32_t A = S.con_a[c], B = S.con_b[c], la = S.con_la[c], lb = S.con_lb[c];
    const Vec3 rA = V3(S.r.rAr[row]), rB = V3(S.r.rBr[row]);
    const Vec3 n = V3(S.r.n[row]);
    const float nm = S.r.mass[row].x, pbias = S.r.bias[row].y;
    float4 im = S.r.imp[row];
    const Vec3 pvA = la != kNone ? V3(V.v[V.shared ? la : A]) : Vec3();
    const Vec3 pwA = la != kNone ? V3(V.w[V.shared ? la : A]) : Vec3();
    const Vec3 pvB = lb != kNone ? V3(V.v[V.shared ? lb : B]) : Vec3();
    const Vec3 pwB = lb != kNone ? V3(V.w[V.shared ? lb : B]) : Vec3();
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

// Warm start + velocity sweeps, then the bias sweeps, of one island; sync() separates levels.
template <typename Sync>
__device__ __forceinline__ void solve_velocity(const SolveBufs& S, uint32_t isl, const VelView& V, uint32_t tid,
                                               uint32_t nthreads, Sync sync) {
    const uint32_t base = 4u * S.isl_start[isl];
    const uint32_t loff = base + isl;
    const uint32_t nw = S.meta[4 * isl], nv = S.meta[4 * isl + 1];
    for (uint32_t l = 0; l < nw; ++l) {
        const uint32_t e = S.wl_off[loff + l + 1];
        for (uint32_t k = S.wl_off[loff + l] + tid; k < e; k += nthreads) warm_point(S, V, S.wl_list[base + k]);
        sync();
    }
    for (uint32_t it = 0; it < S.vel_iters; ++it)
        for (uint32_t l = 0; l < nv; ++l) {
            const uint32_t e = S.vl_off[loff + l + 1];
            for (uint32_t k = S.vl_off[loff + l] + tid; k < e; k += nthreads) velocity_point(S, V, S.vl_list[base + k]);
            sync();
        }
}

template <typename Sync>
__device__ __forceinline__ void solve_bias(const SolveBufs& S, uint32_t isl, const VelView& P, uint32_t tid,
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

struct WarpSync {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct CtaSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// Stage an island's velocities in shared memory, run the warm-start and velocity sweeps, write
// them back; then reuse the same buffers for the split-impulse pseudo velocities (zero at the
// start of every step, PhysicsWorld.cpp:286-287) and the bias sweeps.
template <typename Sync>
__device__ __forceinline__ void solve_island_shared(const SolveBufs& S, uint32_t isl, float4* sv, float4* sw,
                                                    uint32_t tid, uint32_t nthreads, Sync sync) {
    const uint32_t nloc = S.meta[4 * isl + 3];
    const uint32_t* bodies = S.isl_bodies + 2u * S.isl_start[isl];
    for (uint32_t k = tid; k < nloc; k += nthreads) {
        sv[k] = S.b.lv[bodies[k]];
        sw[k] = S.b.av[bodies[k]];
    }
    sync();
    const VelView V{sv, sw, S.b.lv, S.b.av, true};
    solve_velocity(S, isl, V, tid, nthreads, sync);
    for (uint32_t k = tid; k < nloc; k += nthreads) {
        S.b.lv[bodies[k]] = sv[k];
        S.b.av[bodies[k]] = sw[k];
        sv[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        sw[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
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
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_solve_warp(SolveBufs S, const Counters* cnt) {
    extern __shared__ float4 smem[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    float4* sv = smem + warp * 2u * kWarpBodies;
    float4* sw = sv + kWarpBodies;
    const uint32_t n = cnt->nsmall;
    for (uint32_t idx = blockIdx.x * kWarpsPerBlock + warp; idx < n; idx += gridDim.x * kWarpsPerBlock)
        solve_island_shared(S, S.small_list[idx], sv, sw, lane, 32u, WarpSync{});
}

// Large islands: one CTA each; velocities in shared memory when they fit, else in place.
__global__ void __launch_bounds__(kCtaThreads) k_solve_cta(SolveBufs S, const Counters* cnt, uint32_t smem_bodies) {
    extern __shared__ float4 smem[];
    const uint32_t n = cnt->nlarge;
    for (uint32_t idx = blockIdx.x; idx < n; idx += gridDim.x) {
        const uint32_t isl = S.large_list[idx];
        if (S.meta[4 * isl + 3] <= smem_bodies) {
            solve_island_shared(S, isl, smem, smem + smem_bodies, threadIdx.x, blockDim.x, CtaSync{});
        } else {
            const VelView V{S.b.lv, S.b.av, S.b.lv, S.b.av, false};
            const VelView P{S.b.plv, S.b.pav, S.b.lv, S.b.av, false};
            solve_velocity(S, isl, V, threadIdx.x, blockDim.x, CtaSync{});
            solve_bias(S, isl, P, threadIdx.x, blockDim.x, CtaSync{});
            __syncthreads();
        }
    }
}

}  // namespace kzg
