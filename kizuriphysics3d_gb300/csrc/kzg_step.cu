// kzg_step.cu - the per-step contact pipeline on the GPU (PhysicsWorld::StepFixed,
// reference src/World/PhysicsWorld.cpp:245-329), kernel by kernel:
//
//   broad phase      k_aabb, cell sort, k_find_pairs, pair-key sort   (canonical MakePairKey order)
//   narrow phase     k_narrow: one thread per pair; pairs that need EPA go to k_narrow_epa,
//                    one warp per pair                               (Collide, :350-400)
//   constraints      k_con_flags, scan, k_build_constraints           (BuildContactConstraints, :454-535)
//   velocities       k_integrate_vel                                  (IntegrateVelocities, :757-783)
//   prepare          k_prepare: one thread per contact point row      (ContactSolver::PrepareConstraint)
//   islands          union-find k_uf_*, stable sort by island         (BuildIslands, :587-664)
//   schedule         k_schedule_warp / k_schedule_cta: one warp per small island, one CTA per
//                    large one, build the reference's greedy 4-wide batches (:680-717) and the
//                    dependency levels of the warm-start, velocity and bias sweeps
//   solve            k_solve_warp / k_solve_cta / k_solve_big: one warp, CTA or 1024-thread CTA
//                    per island sweeps level by level (SolveIsland, :666-743)
//   cache store      k_cache_store                                    (:568-581)
//   positions        k_integrate_pos: positions, pseudo velocities, world inertia, force clear
//
// Floating point follows the reference op for op (kzg_math.cuh), so with the same pair order the
// result is bit-identical to the reference; levels only reorder work between bodies that share
// no dynamic body, which cannot change any value.
#include <cub/cub.cuh>
#include <cstring>

#include "kzg_ctx.h"
#include "kzg_internal.h"

namespace kzg {

// ---------------------------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long pair_key(uint32_t pa, uint32_t pb) {
    if (pa > pb) { uint32_t t = pa; pa = pb; pb = t; }
    return ((unsigned long long)pa << 32) | (unsigned long long)pb;
}
__device__ __forceinline__ uint32_t hash_key(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k;
}

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kThreads = 256;
inline unsigned blocks_for(uint32_t n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------------------------
// broad phase
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cell_coord(float c, float inv_cell) {
    float f = floorf(c * inv_cell);
    f = fminf(fmaxf(f, -32000.0f), 32000.0f);
    return (uint32_t)((int)f + 32768);
}
__device__ __forceinline__ unsigned long long cell_key(uint32_t world, uint32_t ix, uint32_t iy, uint32_t iz) {
    return ((unsigned long long)(world & 0xFFFFu) << 48) | ((unsigned long long)ix << 32) |
           ((unsigned long long)iy << 16) | (unsigned long long)iz;
}

__device__ __forceinline__ AABB body_bounds(const DeviceBodies& b, const ShapeDev* __restrict__ shapes, uint32_t i) {
    const ShapeDev& s = shapes[b.shape[i]];
    AABB local{Vec3(s.lmn[0], s.lmn[1], s.lmn[2]), Vec3(s.lmx[0], s.lmx[1], s.lmx[2])};
    return aabb_transformed(local, Q4(b.rot[i]), V3(b.pos[i]));
}

// Fat bounds of a moving body, kept like the tree's leaves (DynamicAABBTree::MoveProxy,
// BroadPhase.cpp:58-75): unchanged while they contain the tight bounds, else the tight bounds
// grown by the 0.1 margin and by |velocity x fixed timestep|.  Continuous collision tests them.
__device__ __forceinline__ void update_fat(const DeviceBodies& b, uint32_t i, const AABB& w, float fixed_dt) {
    if (b.motion[i] == KZG_MOTION_STATIC || !b.act[i]) return;  // UpdateBroadPhase walks the active list
    const Vec3 fmn = V3(b.fat_mn[i]), fmx = V3(b.fat_mx[i]);
    if (fmn.x <= w.mn.x && fmx.x >= w.mx.x && fmn.y <= w.mn.y && fmx.y >= w.mx.y && fmn.z <= w.mn.z &&
        fmx.z >= w.mx.z)
        return;
    const Vec3 d = (V3(b.lv[i]) * fixed_dt).abs(), margin(0.1f, 0.1f, 0.1f);
    b.fat_mn[i] = F4((w.mn - margin) - d, 0.0f);
    b.fat_mx[i] = F4((w.mx + margin) + d, 0.0f);
}

// New bodies (BodyManager::CreateBody, BodyManager.cpp:15-61): fat bounds, active, appended to the
// active list in creation order, no island index yet.
__global__ void k_init_bodies(DeviceBodies b, const ShapeDev* __restrict__ shapes, uint32_t first, uint32_t n,
                              uint32_t* alist, const Counters* cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t at = cnt->nact + i;
    i += first;
    const AABB w = body_bounds(b, shapes, i);
    const Vec3 margin(0.1f, 0.1f, 0.1f);  // CreateProxy: tight bounds + margin
    b.fat_mn[i] = F4(w.mn - margin, 0.0f);
    b.fat_mx[i] = F4(w.mx + margin, 0.0f);
    b.act[i] = 1u;
    b.sleep_t[i] = 0.0f;
    b.isl_idx[i] = 0xFFFFFFFFu;
    b.apos[i] = at;
    alist[at] = i;
}
__global__ void k_grow_active(Counters* cnt, uint32_t n) { cnt->nact += n; }

__global__ void k_fat(DeviceBodies b, const ShapeDev* __restrict__ shapes, uint32_t n, float fixed_dt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    update_fat(b, i, body_bounds(b, shapes, i), fixed_dt);
}

// Tight world AABB of every body (Shape::GetWorldBounds = local bounds transformed, Math.cpp:176)
// and its grid cell key; bodies that bypass the grid get key ~0.  Fat bounds follow.
__global__ void k_aabb(DeviceBodies b, const ShapeDev* __restrict__ shapes, uint32_t n, float inv_cell,
                       const uint8_t* __restrict__ is_large, unsigned long long* keys, uint32_t* vals,
                       float fixed_dt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    AABB w = body_bounds(b, shapes, i);
    b.aabb_mn[i] = F4(w.mn, 0.0f);
    b.aabb_mx[i] = F4(w.mx, 0.0f);
    update_fat(b, i, w, fixed_dt);
    unsigned long long key = ~0ull;
    if (!is_large[i]) {
        Vec3 c = (w.mn + w.mx) * 0.5f;
        key = cell_key(b.world[i], cell_coord(c.x, inv_cell), cell_coord(c.y, inv_cell), cell_coord(c.z, inv_cell));
    }
    keys[i] = key;
    vals[i] = i;
}

__device__ __forceinline__ bool pair_ok(const DeviceBodies& b, uint32_t i, uint32_t j) {
    if ((b.layer[i] & b.mask[j]) == 0u || (b.layer[j] & b.mask[i]) == 0u) return false;
    AABB A{V3(b.aabb_mn[i]), V3(b.aabb_mx[i])}, B{V3(b.aabb_mn[j]), V3(b.aabb_mx[j])};
    return aabb_overlaps(A, B);
}

// The pair's sort key: lower packed id << kb | higher, kb bits each (packed ids < 2^kb), so that
// the radix sort only passes over 2 kb bits and orders pairs as MakePairKey's 64-bit keys do.
__device__ __forceinline__ unsigned long long pair_sort_key(uint32_t pa, uint32_t pb, uint32_t kb) {
    if (pa > pb) { uint32_t t = pa; pa = pb; pb = t; }
    return ((unsigned long long)pa << kb) | (unsigned long long)pb;
}

__device__ __forceinline__ void emit_pair(unsigned long long* out, Counters* cnt, uint32_t cap, uint32_t kb,
                                          uint32_t pi, uint32_t pj) {
    uint32_t slot = atomicAdd(&cnt->npairs, 1u);
    if (slot < cap) out[slot] = pair_sort_key(pi, pj, kb);
    else atomicOr(&cnt->error, KZG_DEVERR_PAIRS);
}

// Every overlapping pair exactly once (BroadPhase::UpdatePairs semantics: layer filter both ways,
// tight AABB overlap with <=).  Grid bodies query the 27 neighbouring cells for partners with a
// larger packed id; large bodies (planes) are tested against every body of their world.
__global__ void k_find_pairs(DeviceBodies b, uint32_t n, const unsigned long long* __restrict__ skeys,
                             const uint32_t* __restrict__ svals, uint32_t nsmall, float inv_cell,
                             const uint8_t* __restrict__ is_large, const uint32_t* __restrict__ large_list,
                             const uint32_t* __restrict__ large_off, uint32_t nworld_large, unsigned long long* out,
                             Counters* cnt, uint32_t cap, uint32_t kb) {
    // Threads take the bodies in cell order, so that a warp's neighbours, its cell searches and the
    // bounds it reads are shared (the emitted pairs are sorted afterwards; their order here is free).
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t i = svals[t];
    const uint32_t pi = b.packed[i];
    const uint32_t wi = b.world[i];
    // large bodies of this world
    if (wi < nworld_large) {
        for (uint32_t k = large_off[wi]; k < large_off[wi + 1]; ++k) {
            uint32_t j = large_list[k];
            if (j == i) continue;
            if (is_large[i] && b.packed[j] <= pi) continue;  // large-large: owned by the lower id
            if (pair_ok(b, i, j)) emit_pair(out, cnt, cap, kb, pi, b.packed[j]);
        }
    }
    if (is_large[i]) return;
    Vec3 c = (V3(b.aabb_mn[i]) + V3(b.aabb_mx[i])) * 0.5f;
    int ix = (int)cell_coord(c.x, inv_cell), iy = (int)cell_coord(c.y, inv_cell), iz = (int)cell_coord(c.z, inv_cell);
    // The three cells along z of a column are consecutive keys (cell coordinates stay far from the
    // 16-bit field's ends), so each of the 9 columns is one lower_bound and a forward scan.
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
            const unsigned long long key = cell_key(wi, (uint32_t)(ix + dx), (uint32_t)(iy + dy), (uint32_t)(iz - 1));
            const unsigned long long key_hi = key + 2;
            uint32_t lo = 0, hi = nsmall;  // lower_bound
            while (lo < hi) {
                uint32_t mid = (lo + hi) >> 1;
                if (skeys[mid] < key) lo = mid + 1; else hi = mid;
            }
            for (uint32_t s = lo; s < nsmall && skeys[s] <= key_hi; ++s) {
                uint32_t j = svals[s];
                if (b.packed[j] <= pi) continue;
                if (pair_ok(b, i, j)) emit_pair(out, cnt, cap, kb, pi, b.packed[j]);
            }
        }
}

// Per-step counters to zero, the step counter advanced (the first kernel of every step).
__global__ void k_begin_step(Counters* cnt) {
    const uint32_t nz = (uint32_t)(offsetof(Counters, cache_entries) / sizeof(uint32_t));
    uint32_t* w = reinterpret_cast<uint32_t*>(cnt);
    for (uint32_t i = threadIdx.x; i < nz; i += blockDim.x) w[i] = 0u;
    if (threadIdx.x == 0) ++cnt->frame;
}

// A pair count past the capacity (flagged KZG_DEVERR_PAIRS by emit_pair) is clamped, so the rest of
// the step runs on the pairs that were stored and the overflow is reported after the step.
__global__ void k_clamp_pairs(Counters* cnt, uint32_t cap) {
    if (cnt->npairs > cap) cnt->npairs = cap;
}

// Pair keys past the pair count (up to cap) sort last.
__global__ void k_pad_keys(unsigned long long* keys, const Counters* cnt, uint32_t cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt->npairs && i < cap) keys[i] = ~0ull;
}

__global__ void k_unpack_pairs(const unsigned long long* __restrict__ keys, const Counters* cnt, uint2* pairs,
                               uint32_t kb) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt->npairs) return;
    unsigned long long k = keys[i];
    pairs[i] = make_uint2((uint32_t)(k >> kb) & 0x00FFFFFFu, (uint32_t)(k & ((1ull << kb) - 1ull)) & 0x00FFFFFFu);
}

// Caller-supplied pairs (packed BodyIDs, broad-phase order) -> slots; stale ids become invalid.
__global__ void k_pairs_from_packed(const uint32_t* __restrict__ packed_pairs, uint32_t np, DeviceBodies b, uint32_t nb,
                                    uint2* pairs) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    uint32_t pa = packed_pairs[2 * i], pb = packed_pairs[2 * i + 1];
    uint32_t sa = pa & 0x00FFFFFFu, sb = pb & 0x00FFFFFFu;
    bool ok = sa < nb && sb < nb && b.packed[sa] == pa && b.packed[sb] == pb;
    pairs[i] = ok ? make_uint2(sa, sb) : make_uint2(kInvalid, kInvalid);
}

// ---------------------------------------------------------------------------------------------
// narrow phase (PhysicsWorld::Collide, :366-393)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void store_manifold(const Manifold& m, uint32_t i, unsigned long long key, uint32_t* m_count,
                                               float4* m_data, unsigned long long* m_key) {
    m_key[i] = key;
    m_count[i] = m.n;
    float4* o = m_data + 12ull * i;
    for (uint32_t k = 0; k < m.n; ++k) {
        o[3 * k + 0] = F4(m.pts[k].pA, m.pts[k].sep);
        o[3 * k + 1] = F4(m.pts[k].pB, __uint_as_float(m.pts[k].feature));
        o[3 * k + 2] = F4(m.pts[k].n, 0.0f);
    }
}

// One thread per pair.  Pairs whose routine needs EPA are deferred to the warp pass below.
__global__ void __launch_bounds__(128) k_narrow(ShapeTables T, DeviceBodies b, const uint2* __restrict__ pairs,
                                                Counters* cnt, uint32_t* m_count, float4* m_data,
                                                unsigned long long* m_key, uint32_t* epa_list, GjkOut* epa_gjk,
                                                uint32_t gjk_cap) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt->npairs) return;
    uint2 pr = pairs[i];
    m_count[i] = 0;
    m_key[i] = 0;
    if (pr.x == kInvalid) return;
    const uint32_t A = pr.x, B = pr.y;
    if (b.motion[A] != KZG_MOTION_DYNAMIC && b.motion[B] != KZG_MOTION_DYNAMIC) return;
    const uint32_t pa = b.packed[A], pb = b.packed[B];
    const bool swapped = pa > pb;
    const uint32_t f = swapped ? B : A, s = swapped ? A : B;
    Body BA{&T.shapes[b.shape[f]], Q4(b.rot[f]), V3(b.pos[f])};
    Body BB{&T.shapes[b.shape[s]], Q4(b.rot[s]), V3(b.pos[s])};
    Manifold m;
    EpaDefer ed{&cnt->nepa, epa_list, epa_gjk, gjk_cap, i};
    collide(T, BA, BB, 0.02f, 1.0e-4f, m, ed);
    if (ed.deferred) return;  // queued for the warp pass
    if (swapped) swap_manifold(m);
    store_manifold(m, i, pair_key(pa, pb), m_count, m_data, m_key);
}

// One warp per deferred pair: the same routine with the warp-cooperative EPA.
constexpr uint32_t kEpaWarps = 5;
__global__ void __launch_bounds__(kEpaWarps * 32) k_narrow_epa(ShapeTables T, DeviceBodies b, const uint2* __restrict__ pairs,
                                                               Counters* cnt, const uint32_t* __restrict__ epa_list,
                                                               const GjkOut* __restrict__ epa_gjk, uint32_t gjk_cap,
                                                               uint32_t* m_count, float4* m_data, unsigned long long* m_key,
                                                               uint32_t* err) {
    extern __shared__ EpaWarpSmem epa_smem[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t n = cnt->nepa;
    // pairs are taken from a shared counter: their EPA costs vary by orders of magnitude
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(&cnt->epa_next, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= n) break;
        const uint32_t i = epa_list[idx];
        const uint2 pr = pairs[i];
        const uint32_t A = pr.x, B = pr.y;
        const uint32_t pa = b.packed[A], pb = b.packed[B];
        const bool swapped = pa > pb;
        const uint32_t f = swapped ? B : A, s = swapped ? A : B;
        Body BA{&T.shapes[b.shape[f]], Q4(b.rot[f]), V3(b.pos[f])};
        Body BB{&T.shapes[b.shape[s]], Q4(b.rot[s]), V3(b.pos[s])};
        Manifold m;
        EpaCoop ec{&epa_smem[warp], lane, err, idx < gjk_cap ? &epa_gjk[idx] : nullptr};
        collide(T, BA, BB, 0.02f, 1.0e-4f, m, ec);
        if (swapped) swap_manifold(m);
        if (lane == 0) store_manifold(m, i, pair_key(pa, pb), m_count, m_data, m_key);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------------
// constraints + warm start from the cache (BuildContactConstraints, :454-535)
// ---------------------------------------------------------------------------------------------
__global__ void k_con_flags(const uint32_t* __restrict__ m_count, const unsigned long long* __restrict__ m_key,
                            const Counters* cnt, uint32_t* flag) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt->npairs) return;
    flag[i] = (m_count[i] != 0u && m_key[i] != 0ull) ? 1u : 0u;
}

__device__ inline int cache_find(const unsigned long long* __restrict__ keys, uint32_t cap, unsigned long long key) {
    uint32_t mask = cap - 1u;
    uint32_t slot = hash_key(key) & mask;
    for (uint32_t p = 0; p < cap; ++p) {
        unsigned long long k = keys[slot];
        if (k == key) return (int)slot;
        if (k == 0ull) return -1;
        slot = (slot + 1u) & mask;
    }
    return -1;
}

__global__ void k_build_constraints(const uint2* __restrict__ pairs, const uint32_t* __restrict__ flag,
                                    const uint32_t* __restrict__ cidx, const uint32_t* __restrict__ m_count,
                                    const float4* __restrict__ m_data, const unsigned long long* __restrict__ m_key,
                                    DeviceBodies b, Counters* cnt, uint32_t* con_pair, uint32_t* con_a, uint32_t* con_b,
                                    uint32_t* con_np, uint32_t* con_bits, float2* con_fr,
                                    unsigned long long* con_key, DeviceRows r, const unsigned long long* __restrict__ c_key,
                                    const uint32_t* __restrict__ c_np, const float4* __restrict__ c_pos,
                                    const float4* __restrict__ c_imp, uint32_t c_cap, int warm, uint32_t* miss_rows,
                                    float4* miss_prior) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t np = cnt->npairs;
    if (i >= np) return;
    if (i == np - 1) cnt->ncons = cidx[i] + flag[i];
    if (!flag[i]) return;
    uint32_t c = cidx[i];
    uint32_t A = pairs[i].x, B = pairs[i].y;
    if (b.packed[A] > b.packed[B]) { uint32_t t = A; A = B; B = t; }
    con_pair[c] = i;
    con_a[c] = A;
    con_b[c] = B;
    uint32_t n = m_count[i];
    con_np[c] = n;
    atomicAdd(&cnt->npoints, n);
    unsigned long long key = m_key[i];
    con_key[c] = key;
    const bool sensor = ((b.flags[A] | b.flags[B]) & KZG_BODY_SENSOR) != 0u;
    const float fr = rsqrt_ieee(b.prm1[A].y * b.prm1[B].y);
    const float rs = rmax(b.prm1[A].z, b.prm1[B].z);
    con_fr[c] = make_float2(fr, rs);
    con_bits[c] = (sensor ? 1u : 0u) | (b.motion[A] == KZG_MOTION_DYNAMIC ? 2u : 0u) |
                  (b.motion[B] == KZG_MOTION_DYNAMIC ? 4u : 0u);
    int slot = warm ? cache_find(c_key, c_cap, key) : -1;
    const float4* md = m_data + 12ull * i;
    for (uint32_t p = 0; p < n; ++p) {
        uint32_t row = 4u * c + p;
        float4 pA = md[3 * p], pB = md[3 * p + 1], nn = md[3 * p + 2];
        r.pA[row] = pA;
        r.pB[row] = pB;
        r.n[row] = make_float4(nn.x, nn.y, nn.z, rs);
        r.t1[row] = make_float4(0.0f, 0.0f, 0.0f, fr);
        float ni = 0.0f, t1 = 0.0f, t2 = 0.0f;
        if (slot >= 0) {
            float best = 0.10f * 0.10f;
            uint32_t bi = kInvalid;
            uint32_t cn = c_np[slot];
            Vec3 pa = V3(pA);
            for (uint32_t k = 0; k < cn; ++k) {
                float d = (V3(c_pos[4u * slot + k]) - pa).len2();
                if (d < best) { best = d; bi = k; }
            }
            if (bi != kInvalid) {
                float4 im = c_imp[4u * slot + bi];
                ni = im.x; t1 = im.y; t2 = im.z;
            } else if (miss_rows) {
                // cache miss: remember the pair's nearest cached point at any distance and the
                // pair's cached normal impulse per current point (features of the learned warm
                // start), then the reference's zero start stands
                uint32_t nk = kInvalid;
                float nd = 0.0f, sum_n = 0.0f;
                for (uint32_t k = 0; k < cn; ++k) {
                    float d = (V3(c_pos[4u * slot + k]) - pa).len2();
                    if (nk == kInvalid || d < nd) { nd = d; nk = k; }
                    sum_n += c_imp[4u * slot + k].x;
                }
                const uint32_t m = atomicAdd(&cnt->nmiss, 1u);
                miss_rows[m] = row;
                float4 pr = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (nk != kInvalid) {
                    const float4 im = c_imp[4u * slot + nk];
                    pr = make_float4(im.x, im.y, im.z, sum_n / (float)n);
                }
                miss_prior[m] = pr;
            }
        } else if (warm && miss_rows) {
            const uint32_t m = atomicAdd(&cnt->nmiss, 1u);
            miss_rows[m] = row;
            miss_prior[m] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        r.imp[row] = make_float4(ni, t1, t2, 0.0f);
    }
}

// ---------------------------------------------------------------------------------------------
// IntegrateVelocities (:757-783)
// ---------------------------------------------------------------------------------------------
__global__ void k_integrate_vel(DeviceBodies b, uint32_t n, float3 g, float dt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || b.motion[i] != KZG_MOTION_DYNAMIC || !b.act[i]) return;  // the active list's bodies
    float4 p0 = b.prm0[i], p1 = b.prm1[i];
    float im = b.inv_mass[i];
    Vec3 lv = V3(b.lv[i]), av = V3(b.av[i]);
    Vec3 acc = Vec3(g.x, g.y, g.z) * p0.z + V3(b.force[i]) * im;
    lv = lv + acc * dt;
    av = av + (M3(&b.iiw[3 * i]) * V3(b.torque[i])) * dt;
    lv = lv * rdiv(1.0f, 1.0f + p0.x * dt);
    av = av * rdiv(1.0f, 1.0f + p0.y * dt);
    lv = clamp_length(lv, p0.w);
    av = clamp_length(av, p1.x);
    if (!lv.finite() || !av.finite()) { lv = Vec3(); av = Vec3(); }
    b.lv[i] = F4(lv, 0.0f);
    b.av[i] = F4(av, 0.0f);
}

// ---------------------------------------------------------------------------------------------
// PrepareConstraint (ContactSolver.cpp:56-112), one thread per point row
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float eff_mass(float imA, float imB, const Mat3& IA, const Mat3& IB, const Vec3& rA,
                                          const Vec3& rB, const Vec3& d) {
    Vec3 ra = rA.cross(d), rb = rB.cross(d);
    float k = imA + imB;
    k += ra.dot(IA * ra);
    k += rb.dot(IB * rb);
    return k > kEps ? rdiv(1.0f, k) : 0.0f;
}

struct PrepParams {
    float dt, baumgarte, slop, rest_thresh, max_bias;
};

__global__ void k_prepare(DeviceBodies b, const Counters* cnt, const uint32_t* __restrict__ con_a,
                          const uint32_t* __restrict__ con_b, const uint32_t* __restrict__ con_np, DeviceRows r,
                          PrepParams pp) {
    uint32_t row = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c = row >> 2, p = row & 3u;
    if (c >= cnt->ncons || p >= con_np[c]) return;
    const uint32_t A = con_a[c], B = con_b[c];
    const Vec3 posA = V3(b.pos[A]), posB = V3(b.pos[B]);
    const Quat qA = Q4(b.rot[A]), qB = Q4(b.rot[B]);
    float4 pA4 = r.pA[row], pB4 = r.pB[row], n4 = r.n[row], t14 = r.t1[row], imp = r.imp[row];
    const Vec3 pA = V3(pA4), pB = V3(pB4);
    const float sep = pA4.w, rest = n4.w, fric = t14.w;
    Vec3 rA = pA - posA, rB = pB - posB;
    Vec3 laA = qA.inv_rotate(rA), laB = qB.inv_rotate(rB);
    Vec3 n = V3(n4).normalized_or(Vec3(0.0f, 1.0f, 0.0f));
    Vec3 t1 = n.perp_normalized();
    Vec3 t2 = n.cross(t1);
    const float imA = b.inv_mass[A], imB = b.inv_mass[B];
    const Mat3 IA = M3(&b.iiw[3 * A]), IB = M3(&b.iiw[3 * B]);
    float nm = eff_mass(imA, imB, IA, IB, rA, rB, n);
    float tm1 = eff_mass(imA, imB, IA, IB, rA, rB, t1);
    float tm2 = eff_mass(imA, imB, IA, IB, rA, rB, t2);
    Vec3 vA = V3(b.lv[A]) + V3(b.av[A]).cross(pA - posA);
    Vec3 vB = V3(b.lv[B]) + V3(b.av[B]).cross(pB - posB);
    float nvel = (vA - vB).dot(n);
    float rbias = 0.0f;
    if (nvel < -pp.rest_thresh) rbias = -rest * nvel;
    float pbias = 0.0f;
    if (sep < -pp.slop) {
        pbias = rdiv(pp.baumgarte, pp.dt) * (-sep - pp.slop);
        pbias = rmin(pbias, pp.max_bias);
    }
    float mf = fric * imp.x;
    float ti1 = rclamp(imp.y, -mf, mf), ti2 = rclamp(imp.z, -mf, mf);
    float ni = rmax(imp.x, 0.0f);
    r.n[row] = F4(n, rest);
    r.t1[row] = F4(t1, fric);
    r.t2[row] = F4(t2, 0.0f);
    r.rA[row] = F4(rA, 0.0f);
    r.rB[row] = F4(rB, 0.0f);
    r.laA[row] = F4(laA, 0.0f);
    r.laB[row] = F4(laB, 0.0f);
    r.rAr[row] = F4(qA.rotate(laA), 0.0f);
    r.rBr[row] = F4(qB.rotate(laB), 0.0f);
    r.mass[row] = make_float4(nm, tm1, tm2, 0.0f);
    r.imp[row] = make_float4(ni, ti1, ti2, 0.0f);
    r.bias[row] = make_float4(rbias, pbias, nvel, 0.0f);
}

// ---------------------------------------------------------------------------------------------
// islands (BuildIslands, :587-664): union-find over dynamic-dynamic contacts
// ---------------------------------------------------------------------------------------------
__global__ void k_uf_init(uint32_t* uf, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) uf[i] = i;
}
__device__ __forceinline__ uint32_t uf_find(uint32_t* uf, uint32_t x) {
    for (;;) {
        uint32_t p = __ldcg(&uf[x]);
        if (p == x) return x;
        uint32_t gp = __ldcg(&uf[p]);
        if (gp != p) atomicCAS(&uf[x], p, gp);  // path halving
        x = p;
    }
}
__device__ __forceinline__ void uf_link(uint32_t* uf, uint32_t a, uint32_t bb) {
    for (;;) {
        a = uf_find(uf, a);
        bb = uf_find(uf, bb);
        if (a == bb) return;
        if (a > bb) { uint32_t t = a; a = bb; bb = t; }
        uint32_t old = atomicCAS(&uf[bb], bb, a);  // hook the larger root under the smaller
        if (old == bb) return;
        bb = old;
    }
}

// The union-find element a dynamic body joins islands through.  Sleeping off (node == null): the
// body itself.  Sleeping on: an active body itself; a sleeping body the active dynamic body that now
// holds its stale island index (BuildIslands' compact index, PhysicsWorld.cpp:593-605, 616-623), or
// none when that index is past the active dynamic count.
__device__ __forceinline__ uint32_t island_node(const uint32_t* __restrict__ node, uint32_t x) {
    return node ? node[x] : x;
}

// Joins two dynamic bodies' islands (BuildIslands' contact and joint unions).  With sleeping on, a
// sleeping body without a node still links the islands it touches (its own slot as the link):
// the reference puts each of its contacts in the other body's island and then solves those islands
// concurrently, a race on the sleeping body; joined, they are solved as one, deterministically.
__device__ __forceinline__ void island_union(uint32_t* uf, const uint32_t* __restrict__ node, uint32_t a, uint32_t bb) {
    const uint32_t na = island_node(node, a), nb = island_node(node, bb);
    if (na != kInvalid && nb != kInvalid) uf_link(uf, na, nb);
    else if (na != kInvalid) uf_link(uf, na, bb);
    else if (nb != kInvalid) uf_link(uf, a, nb);
}

__global__ void k_uf_union(const Counters* cnt, const uint32_t* __restrict__ con_a, const uint32_t* __restrict__ con_b,
                           const uint32_t* __restrict__ con_bits, const uint32_t* __restrict__ node, uint32_t* uf) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cnt->ncons || (con_bits[c] & 6u) != 6u) return;
    island_union(uf, node, con_a[c], con_b[c]);
}
// WorldStats::numIslands (PhysicsWorld.cpp:636-642): one island per union-find root among the
// dynamic bodies, bodies without a contact included.
__global__ void k_count_roots(const DeviceBodies b, uint32_t n, const uint32_t* __restrict__ uf, Counters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool root = i < n && b.motion[i] == KZG_MOTION_DYNAMIC && __ldcg(&uf[i]) == i;
    const unsigned m = __ballot_sync(0xffffffffu, root);
    if ((threadIdx.x & 31u) == 0 && m) atomicAdd(&cnt->nroots, (uint32_t)__popc(m));
}

// Island of every constraint; slots past the constraint count (up to cap) get a key above every
// body index so that a capacity-sized sort leaves them at the end.
// islandOf(A), else islandOf(B) (PhysicsWorld.cpp:645-650): the root of the first dynamic body with
// an island node; a constraint with neither (two sleeping bodies, both indices stale) is in no
// island and is not solved.  Such constraints, and slots past the constraint count (up to cap), get
// a key above every body index so that a capacity-sized sort leaves them at the end.
__global__ void k_island_keys(const Counters* cnt, const uint32_t* __restrict__ con_a, const uint32_t* __restrict__ con_b,
                              const uint32_t* __restrict__ con_bits, const uint32_t* __restrict__ node, uint32_t* uf,
                              uint32_t* key, uint32_t* val, uint32_t cap, uint32_t pad) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cnt->ncons) {
        if (c < cap) {
            key[c] = pad;
            val[c] = c;
        }
        return;
    }
    const uint32_t bits = con_bits[c];
    const uint32_t na = (bits & 2u) ? island_node(node, con_a[c]) : kInvalid;
    const uint32_t d = na != kInvalid ? na : ((bits & 4u) ? island_node(node, con_b[c]) : kInvalid);
    key[c] = d != kInvalid ? uf_find(uf, d) : pad;
    val[c] = c;
}
__global__ void k_island_heads(const Counters* cnt, const uint32_t* __restrict__ skey, uint32_t* head, uint32_t pad) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cnt->ncons) return;
    head[s] = (skey[s] != pad && (s == 0 || skey[s] != skey[s - 1])) ? 1u : 0u;
}
// Island ranges of the sorted constraints; the constraints keyed `pad` (in no island) sort last and
// end the last island.
__global__ void k_island_starts(Counters* cnt, const uint32_t* __restrict__ skey, const uint32_t* __restrict__ head,
                                const uint32_t* __restrict__ hscan, uint32_t* start, uint32_t pad) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = cnt->ncons;
    if (s >= n) return;
    if (head[s]) start[hscan[s]] = s;
    if (skey[s] != pad && (s == n - 1 || skey[s + 1] == pad)) {
        uint32_t ni = hscan[s] + head[s];
        start[ni] = s + 1;
        cnt->nislands = ni;
    }
}


// ---------------------------------------------------------------------------------------------
// sleeping (WorldSettings::allowSleeping): the wake rule of BuildContactConstraints
// (PhysicsWorld.cpp:473-490), BuildIslands' compact indices over the active list (:593-605) and
// UpdateSleeping (:866-951) with the active list of BodyManager (BodyManager.cpp:133-160)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ bool body_moving(const DeviceBodies& b, uint32_t i) {
    const uint32_t m = b.motion[i];
    if (m == KZG_MOTION_DYNAMIC) return __ldcg(&b.act[i]) != 0u;
    if (m == KZG_MOTION_KINEMATIC) return V3(b.lv[i]).len2() > 0.0f || V3(b.av[i]).len2() > 0.0f;
    return false;
}

// One warp walks the constraints in order, 32 at a time, and wakes a sleeping dynamic body touched
// by a moving one exactly as the sequential loop does: lanes before the first lane that wakes a body
// are final; that lane's wakes (A, then B, which then sees A moving) are applied - appended to the
// active list - and the lanes after it are decided again on the new state.
__global__ void __launch_bounds__(32) k_wake(DeviceBodies b, Counters* cnt, const uint32_t* __restrict__ con_a,
                                             const uint32_t* __restrict__ con_b, uint32_t* alist) {
    const uint32_t lane = threadIdx.x;
    const uint32_t nc = cnt->ncons;
    for (uint32_t w0 = 0; w0 < nc; w0 += 32) {
        const uint32_t c = w0 + lane;
        const bool v = c < nc;
        const uint32_t A = v ? con_a[c] : 0u, B = v ? con_b[c] : 0u;
        const bool dA = v && b.motion[A] == KZG_MOTION_DYNAMIC, dB = v && b.motion[B] == KZG_MOTION_DYNAMIC;
        uint32_t from = 0;
        for (;;) {
            bool wa = false, wb = false;
            if (v && lane >= from) {
                wa = dA && __ldcg(&b.act[A]) == 0u && body_moving(b, B);
                wb = dB && __ldcg(&b.act[B]) == 0u && (wa || body_moving(b, A));
            }
            const unsigned m = __ballot_sync(0xffffffffu, wa || wb);
            if (!m) break;
            const uint32_t f = (uint32_t)(__ffs(m) - 1);
            if (lane == f) {
                uint32_t n = cnt->nact;
                if (wa) { b.act[A] = 1u; b.sleep_t[A] = 0.0f; b.apos[A] = n; alist[n++] = A; }
                if (wb) { b.act[B] = 1u; b.sleep_t[B] = 0.0f; b.apos[B] = n; alist[n++] = B; }
                cnt->nact = n;
                __threadfence_block();
            }
            __syncwarp();
            from = f + 1;
        }
    }
}

// BuildIslands' compact index: active dynamic bodies numbered in active-list order.
__global__ void k_act_flags(const DeviceBodies b, const Counters* cnt, const uint32_t* __restrict__ alist, uint32_t cap,
                            uint32_t* flag) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cap) return;
    flag[p] = (p < cnt->nact && b.motion[alist[p]] == KZG_MOTION_DYNAMIC) ? 1u : 0u;
}
__global__ void k_act_index(DeviceBodies b, Counters* cnt, const uint32_t* __restrict__ alist,
                            const uint32_t* __restrict__ flag, const uint32_t* __restrict__ scan, uint32_t* dyn2slot) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = cnt->nact;
    if (p >= n) return;
    const uint32_t x = alist[p];
    b.isl_idx[x] = flag[p] ? scan[p] : 0xFFFFFFFFu;
    if (flag[p]) dyn2slot[scan[p]] = x;
    if (p == n - 1) cnt->ndyn = scan[p] + flag[p];
}
// Island node of every body (see island_node) and the union-find start.
__global__ void k_nodes(const DeviceBodies b, const Counters* cnt, uint32_t nb, const uint32_t* __restrict__ dyn2slot,
                        uint32_t* node, uint32_t* uf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    uint32_t nd = kInvalid;
    if (b.motion[i] == KZG_MOTION_DYNAMIC) {
        if (b.act[i]) nd = i;
        else if (b.isl_idx[i] < cnt->ndyn) nd = dyn2slot[b.isl_idx[i]];
    }
    node[i] = nd;
    uf[i] = i;
}
// WorldStats::numIslands of BuildIslands with sleeping on: the sets holding an active dynamic body.
__global__ void k_mark_roots(const DeviceBodies b, uint32_t nb, uint32_t* uf, uint32_t* mark) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb && b.motion[i] == KZG_MOTION_DYNAMIC && b.act[i]) mark[uf_find(uf, i)] = 1u;
}
__global__ void k_count_marks(const uint32_t* __restrict__ mark, uint32_t nb, Counters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned m = __ballot_sync(0xffffffffu, i < nb && mark[i] != 0u);
    if ((threadIdx.x & 31u) == 0 && m) atomicAdd(&cnt->nroots, (uint32_t)__popc(m));
}

// UpdateSleeping, pass 1: sleep timers of the active bodies; island index = active-list position;
// union-find over positions and the islands' smallest timer start.
__global__ void k_sleep_begin(DeviceBodies b, Counters* cnt, const uint32_t* __restrict__ alist, uint32_t cap,
                              float lin2, float ang2, float dt, uint32_t* suf, uint32_t* smin) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = cnt->nact;
    if (p == 0) cnt->nsleep_n = n;
    if (p >= cap) return;
    suf[p] = p;
    smin[p] = __float_as_uint(1.0e18f);  // math::kBigNumber (Types.h:44)
    if (p >= n) return;
    const uint32_t x = alist[p];
    b.isl_idx[x] = p;
    if (b.motion[x] != KZG_MOTION_DYNAMIC || !(b.flags[x] & KZG_BODY_ALLOW_SLEEPING)) {
        b.sleep_t[x] = 0.0f;
        return;
    }
    if (V3(b.lv[x]).len2() < lin2 && V3(b.av[x]).len2() < ang2) b.sleep_t[x] = b.sleep_t[x] + dt;
    else b.sleep_t[x] = 0.0f;
}
// pass 2: contacts between dynamic bodies whose island indices are both below n join.
__global__ void k_sleep_union(const DeviceBodies b, const Counters* cnt, const uint32_t* __restrict__ con_a,
                              const uint32_t* __restrict__ con_b, const uint32_t* __restrict__ con_bits, uint32_t* suf) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cnt->ncons || (con_bits[c] & 6u) != 6u) return;
    const uint32_t n = cnt->nsleep_n, ia = b.isl_idx[con_a[c]], ib = b.isl_idx[con_b[c]];
    if (ia < n && ib < n) uf_link(suf, ia, ib);
}
// pass 3: each island's smallest timer (timers are >= 0, so their bits order like the floats).
__global__ void k_sleep_min(const DeviceBodies b, const Counters* cnt, const uint32_t* __restrict__ alist, uint32_t* suf,
                            uint32_t* smin) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cnt->nsleep_n) return;
    const uint32_t x = alist[p];
    if (b.motion[x] != KZG_MOTION_DYNAMIC || !(b.flags[x] & KZG_BODY_ALLOW_SLEEPING)) return;
    atomicMin(&smin[uf_find(suf, p)], __float_as_uint(b.sleep_t[x]));
}
// pass 4: bodies of islands quiet for the threshold are deactivated, velocities zeroed (their
// removal from the active list follows in order).
__global__ void k_sleep_mark(DeviceBodies b, const Counters* cnt, const uint32_t* __restrict__ alist, uint32_t* suf,
                             const uint32_t* __restrict__ smin, float threshold, uint32_t* mark) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= cnt->nsleep_n) return;
    const uint32_t x = alist[p];
    uint32_t m = kInvalid;
    if (b.motion[x] == KZG_MOTION_DYNAMIC && (b.flags[x] & KZG_BODY_ALLOW_SLEEPING) &&
        __uint_as_float(smin[uf_find(suf, p)]) >= threshold) {
        b.lv[x] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.av[x] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        b.act[x] = 0u;
        m = x;
    }
    mark[p] = m;
}
// pass 5 (one warp): BodyManager::DeactivateBody's swap-removal, body by body in active-list order:
// the last entry moves into the removed one's place; the buffer keeps the old last value.
__global__ void __launch_bounds__(32) k_sleep_remove(DeviceBodies b, Counters* cnt, uint32_t* alist,
                                                     const uint32_t* __restrict__ mark) {
    const uint32_t lane = threadIdx.x;
    const uint32_t n = cnt->nsleep_n;
    uint32_t size = n;
    for (uint32_t p0 = 0; p0 < n; p0 += 32) {
        const uint32_t p = p0 + lane;
        const uint32_t x = p < n ? mark[p] : kInvalid;
        unsigned m = __ballot_sync(0xffffffffu, x != kInvalid);
        while (m) {
            const uint32_t l = (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            const uint32_t xb = __shfl_sync(0xffffffffu, x, l);
            if (lane == 0) {
                const uint32_t at = b.apos[xb], last = size - 1u;
                if (at != last) {
                    const uint32_t moved = alist[last];
                    alist[at] = moved;
                    b.apos[moved] = at;
                }
                b.apos[xb] = kInvalid;
                --size;
            }
            size = __shfl_sync(0xffffffffu, size, 0);
        }
    }
    if (lane == 0) cnt->nact = size;
}
// pass 6: the island count UpdateSleeping leaves in WorldStats, read over the list's buffer after
// the removals (positions past the new end hold leftover values).
__global__ void k_sleep_count(const DeviceBodies b, Counters* cnt, const uint32_t* __restrict__ alist, uint32_t* suf) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool c = p < cnt->nsleep_n && b.motion[alist[p]] == KZG_MOTION_DYNAMIC && uf_find(suf, p) == p;
    const unsigned m = __ballot_sync(0xffffffffu, c);
    if ((threadIdx.x & 31u) == 0 && m) atomicAdd(&cnt->sleep_islands, (uint32_t)__popc(m));
}

// Largest-first island order (KZG_ISLANDS_LARGEST_FIRST): islands binned by the power of two of
// their constraint count and listed bin by bin from the largest down; inside a bin the order is
// whatever the atomics give (islands share no dynamic body, so any order gives the same bits).
__global__ void k_island_bin_count(const Counters* cnt, const uint32_t* __restrict__ start, uint32_t* bins) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt->nislands) return;
    atomicAdd(&bins[31 - __clz(start[i + 1] - start[i])], 1u);  // every island has a constraint
}
__global__ void k_island_bin_offsets(uint32_t* bins) {  // one warp; cursors in bins[32..64)
    const uint32_t lane = threadIdx.x;
    const uint32_t c = bins[31 - lane];  // lane 0: the largest bin
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    bins[32 + 31 - lane] = x - c;
}
__global__ void k_island_bin_scatter(const Counters* cnt, const uint32_t* __restrict__ start, uint32_t* bins,
                                     uint32_t* order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt->nislands) return;
    order[atomicAdd(&bins[32 + 31 - __clz(start[i + 1] - start[i])], 1u)] = i;
}

}  // namespace kzg

#include "kzg_solver.cuh"


namespace kzg {

// ---------------------------------------------------------------------------------------------
// Joints: creation, Prepare, island membership and position correction (the velocity part runs in
// k_solve_big, kzg_solver.cuh)
// ---------------------------------------------------------------------------------------------
__global__ void k_joint_create(DeviceBodies b, JointDev* J, const kzg_joint_desc* __restrict__ d, uint32_t first,
                               uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) joint_create(JBodies{b}, J[first + i], d[i]);
}

// Constraint::Prepare of every enabled joint (PhysicsWorld.cpp:547-548), after the contacts'.
__global__ void k_joint_prepare(DeviceBodies b, JointDev* J, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !(J[i].flags & kJointDisabled)) joint_prepare(JBodies{b}, J[i]);
}

// Joints between two dynamic bodies join their islands (PhysicsWorld.cpp:625-633).
__global__ void k_joint_union(DeviceBodies b, const JointDev* __restrict__ J, uint32_t n,
                              const uint32_t* __restrict__ node, uint32_t* uf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (J[i].flags & kJointDisabled)) return;
    const uint32_t a = J[i].a, bb = J[i].b;
    if (b.motion[a] != KZG_MOTION_DYNAMIC || b.motion[bb] != KZG_MOTION_DYNAMIC) return;
    island_union(uf, node, a, bb);
}

// Island of each joint: islandOf(A), else islandOf(B) (PhysicsWorld.cpp:656-661), as the root of its
// dynamic body, keyed root << 32 | joint index so that a sort groups islands in joint order; a
// joint with no dynamic body or disabled gets ~0 (sorted last, never solved).
__global__ void k_joint_keys(DeviceBodies b, const JointDev* __restrict__ J, uint32_t n,
                             const uint32_t* __restrict__ node, uint32_t* uf, unsigned long long* keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long key = ~0ull;
    if (!(J[i].flags & kJointDisabled)) {
        const uint32_t a = J[i].a, bb = J[i].b;
        const uint32_t na = b.motion[a] == KZG_MOTION_DYNAMIC ? island_node(node, a) : kNone;
        const uint32_t d = na != kNone ? na : (b.motion[bb] == KZG_MOTION_DYNAMIC ? island_node(node, bb) : kNone);
        if (d != kNone) key = ((unsigned long long)uf_find(uf, d) << 32) | i;
    }
    keys[i] = key;
}

// One joint island per run of equal roots; its contact island (contact islands are sorted by root)
// is flagged so that the schedule hands it to k_solve_big's joint pass instead of the other solvers.
__global__ void k_joint_islands(const unsigned long long* __restrict__ sk, uint32_t n, Counters* cnt,
                                const uint32_t* __restrict__ isl_key, const uint32_t* __restrict__ isl_start,
                                uint2* jisl, uint32_t* jisl_cisl, uint32_t* jflag) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || sk[s] == ~0ull) return;
    const uint32_t root = (uint32_t)(sk[s] >> 32);
    if (s > 0 && (uint32_t)(sk[s - 1] >> 32) == root) return;
    uint32_t e = s + 1;
    while (e < n && sk[e] != ~0ull && (uint32_t)(sk[e] >> 32) == root) ++e;
    const uint32_t k = atomicAdd(&cnt->njisl, 1u);
    jisl[k] = make_uint2(s, e);
    const uint32_t ni = cnt->nislands;
    uint32_t lo = 0, hi = ni;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (isl_key[isl_start[mid]] < root) lo = mid + 1;
        else hi = mid;
    }
    const uint32_t c = (lo < ni && isl_key[isl_start[lo]] == root) ? lo : kNone;
    jisl_cisl[k] = c;
    if (c != kNone) jflag[c] = 1u;
}

// SolveIslandPositions (PhysicsWorld.cpp:745-752): each island's joints, position_iterations times.
__global__ void k_joint_positions(DeviceBodies b, JointDev* J, const unsigned long long* __restrict__ sk,
                                  const uint2* __restrict__ jisl, const Counters* cnt, uint32_t iters) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cnt->njisl) return;
    const uint2 r = jisl[k];
    const JBodies B{b};
    for (uint32_t it = 0; it < iters; ++it)
        for (uint32_t s = r.x; s < r.y; ++s) joint_position(B, J[(uint32_t)sk[s]]);
}

// UpdateSleeping's joint unions (PhysicsWorld.cpp:907-915), beside k_sleep_union.
__global__ void k_sleep_union_joints(const DeviceBodies b, const Counters* cnt, const JointDev* __restrict__ J,
                                     uint32_t nj, uint32_t* suf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nj || (J[i].flags & kJointDisabled)) return;
    const uint32_t a = J[i].a, bb = J[i].b;
    if (b.motion[a] != KZG_MOTION_DYNAMIC || b.motion[bb] != KZG_MOTION_DYNAMIC) return;
    const uint32_t n = cnt->nsleep_n, ia = b.isl_idx[a], ib = b.isl_idx[bb];
    if (ia < n && ib < n) uf_link(suf, ia, ib);
}
// WorldStats::numIslands as UpdateSleeping leaves it (PhysicsWorld.cpp:893-949).  The count reads
// the active list's buffer after the removals position by position and counts the positions that
// are their set's root, so it depends on which position the reference's union-by-rank
// (PhysicsWorld.cpp:38-57; contacts, then joints, in order) makes each root.  One thread replays
// those unions; parent and rank live in shared memory when they fit, else in global scratch.
// Run on demand (kzg_get_stats), on the buffers the last step left.
constexpr uint32_t kSleepCountSmem = 40000;  // positions held in shared memory (5 bytes each)
__global__ void __launch_bounds__(256) k_sleep_count_ref(const DeviceBodies b, Counters* cnt, const uint32_t* __restrict__ alist,
                                                        const uint32_t* __restrict__ con_a, const uint32_t* __restrict__ con_b,
                                                        const uint32_t* __restrict__ con_bits, const JointDev* __restrict__ J,
                                                        uint32_t nj, uint32_t* gpar, uint8_t* grank) {
    extern __shared__ uint32_t sm_uf[];
    __shared__ uint32_t count;
    const uint32_t n = cnt->nsleep_n;
    const bool shared = n <= kSleepCountSmem;
    uint32_t* par = shared ? sm_uf : gpar;
    uint8_t* rk = shared ? reinterpret_cast<uint8_t*>(sm_uf + kSleepCountSmem) : grank;
    for (uint32_t p = threadIdx.x; p < n; p += blockDim.x) {
        par[p] = p;
        rk[p] = 0;
    }
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        auto find = [&](uint32_t x) {
            while (par[x] != x) {
                par[x] = par[par[x]];
                x = par[x];
            }
            return x;
        };
        auto unite = [&](uint32_t a, uint32_t c) {
            a = find(a);
            c = find(c);
            if (a == c) return;
            if (rk[a] < rk[c]) { const uint32_t t = a; a = c; c = t; }
            par[c] = a;
            if (rk[a] == rk[c]) ++rk[a];
        };
        const uint32_t nc = cnt->ncons;
        for (uint32_t k = 0; k < nc; ++k) {
            if ((con_bits[k] & 6u) != 6u) continue;
            const uint32_t ia = b.isl_idx[con_a[k]], ib = b.isl_idx[con_b[k]];
            if (ia < n && ib < n) unite(ia, ib);
        }
        for (uint32_t k = 0; k < nj; ++k) {
            if (J[k].flags & kJointDisabled) continue;
            const uint32_t a = J[k].a, c = J[k].b;
            if (b.motion[a] != KZG_MOTION_DYNAMIC || b.motion[c] != KZG_MOTION_DYNAMIC) continue;
            const uint32_t ia = b.isl_idx[a], ib = b.isl_idx[c];
            if (ia < n && ib < n) unite(ia, ib);
        }
    }
    __syncthreads();
    uint32_t mine = 0;
    for (uint32_t p = threadIdx.x; p < n; p += blockDim.x)
        mine += (b.motion[alist[p]] == KZG_MOTION_DYNAMIC && par[p] == p) ? 1u : 0u;
    atomicAdd(&count, mine);
    __syncthreads();
    if (threadIdx.x == 0) cnt->sleep_islands = count;
}

cudaError_t create_joints(Ctx& ctx, uint32_t first, uint32_t n) {
    k_joint_create<<<blocks_for(n), kThreads, 0, ctx.stream>>>(ctx.b, ctx.joints, ctx.joint_stage, first, n);
    cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : cudaStreamSynchronize(ctx.stream);
}
size_t joint_record_bytes() { return sizeof(JointDev); }
size_t gjk_record_bytes() { return sizeof(GjkOut); }

// ---------------------------------------------------------------------------------------------
// cache store (:568-581) and position integration (:276-290, 785-802, 854-861)
// ---------------------------------------------------------------------------------------------
__global__ void k_cache_store(Counters* cnt, const unsigned long long* __restrict__ con_key,
                              const uint32_t* __restrict__ con_np, DeviceRows r, unsigned long long* c_key,
                              uint32_t* c_np, float4* c_pos, float4* c_imp, uint32_t cap) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cnt->ncons) return;
    unsigned long long key = con_key[c];
    uint32_t mask = cap - 1u;
    uint32_t slot = hash_key(key) & mask;
    uint32_t probes = 0;
    for (;;) {
        unsigned long long prev = atomicCAS(&c_key[slot], 0ull, key);
        if (prev == 0ull) { atomicAdd(&cnt->cache_entries, 1u); break; }
        if (prev == key) break;
        slot = (slot + 1u) & mask;
        if (++probes >= cap) { atomicOr(&cnt->error, KZG_DEVERR_CACHE); return; }
    }
    uint32_t n = con_np[c];
    c_np[slot] = n;
    for (uint32_t p = 0; p < n; ++p) {
        float4 pa = r.pA[4u * c + p];
        float4 im = r.imp[4u * c + p];
        c_pos[4u * slot + p] = make_float4(pa.x, pa.y, pa.z, 0.0f);
        c_imp[4u * slot + p] = make_float4(im.x, im.y, im.z, 0.0f);
    }
}

// Moves every entry of a cache table into one twice (or more) its size: keys are unique, so an
// entry only needs a free slot in its new probe sequence.
__global__ void k_cache_rehash(const unsigned long long* __restrict__ ok, const uint32_t* __restrict__ onp,
                               const float4* __restrict__ opos, const float4* __restrict__ oimp, uint32_t ocap,
                               unsigned long long* nk, uint32_t* nnp, float4* npos, float4* nimp, uint32_t ncap,
                               Counters* cnt) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ocap) return;
    const unsigned long long key = ok[s];
    if (key == 0ull) return;
    const uint32_t mask = ncap - 1u;
    uint32_t slot = hash_key(key) & mask;
    for (uint32_t probes = 0; atomicCAS(&nk[slot], 0ull, key) != 0ull; slot = (slot + 1u) & mask)
        if (++probes >= ncap) { atomicOr(&cnt->error, KZG_DEVERR_CACHE); return; }
    nnp[slot] = onp[s];
    for (uint32_t p = 0; p < 4; ++p) {
        npos[4u * slot + p] = opos[4u * s + p];
        nimp[4u * slot + p] = oimp[4u * s + p];
    }
}

__global__ void k_cache_scatter(const uint32_t* __restrict__ slots, const unsigned long long* __restrict__ keys,
                                const uint32_t* __restrict__ np, const float4* __restrict__ pos,
                                const float4* __restrict__ imp, uint32_t n, unsigned long long* c_key, uint32_t* c_np,
                                float4* c_pos, float4* c_imp) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const uint32_t s = slots[e];
    c_key[s] = keys[e];
    c_np[s] = np[e];
    for (uint32_t p = 0; p < 4; ++p) {
        c_pos[4u * s + p] = pos[4u * e + p];
        c_imp[4u * s + p] = imp[4u * e + p];
    }
}

__device__ __forceinline__ bool casts_linear(const DeviceBodies& b, uint32_t i) {
    return b.motion[i] == KZG_MOTION_DYNAMIC && (b.flags[i] & KZG_BODY_LINEAR_CAST) != 0u;
}

// Continuous collision of LinearCast bodies (PhysicsWorld::ClampMotionCCD, PhysicsWorld.cpp:785-802
// and 804-852; a displacement shorter than the body's positive ccdMotionThreshold is left as it is).
// The reference runs it inside
// the position loop, body by body in slot order, so a body sees the bodies before it already
// moved.  Per body: candidates are the bodies whose fat bounds overlap the swept bounds grown by
// 0.1 (not itself, not a sensor, layer and mask both ways), each placed where that loop has it at
// that moment (lower slots moved: LinearCast ones by their clamped displacement, others by v dt
// with their rotation integrated), cast against, and the smallest fraction wins (ties: the smaller
// slot, the reference's first hit).  The motion stops max_pen short of the hit and the approaching
// normal velocity is removed.
//
// Order only matters through a LinearCast candidate of lower slot whose own motion may be clamped
// (displacement above max_pen).  k_ccd_init writes the displacement of every LinearCast body with
// nothing to clamp (round[slot] = 0) and marks the others pending (kPending); a body's velocity
// may change when it is clamped, so "clampable" is read from the round stamp, never from the
// velocity.  k_ccd_deps lists each pending body's predecessors (its clampable lower-slot
// candidates).  Round r (k_ccd_round, one warp per body, r = 1..kCcdRounds) solves every pending
// body whose predecessors all finished in an earlier round, so each sees final displacements, and
// stamps it r; k_ccd_serial walks what is left in slot order on one block.  The result is the
// sequential one.
constexpr uint32_t kCcdThreads = 256;
constexpr uint32_t kNoHit = 0xFFFFFFFFu;

struct CcdBody {
    const ShapeDev* sh;
    Quat q0;
    Vec3 t0, lv, disp, dir;
    float dist;
    AABB sweep;
    uint32_t li, mi;
};

__device__ __forceinline__ CcdBody ccd_body(const ShapeTables& T, const DeviceBodies& b, uint32_t i, float dt) {
    CcdBody c;
    c.sh = &T.shapes[b.shape[i]];
    c.q0 = Q4(b.rot[i]);
    c.t0 = V3(b.pos[i]);
    c.lv = V3(b.lv[i]);
    c.disp = c.lv * dt;
    c.dist = c.disp.len();
    c.dir = c.disp / c.dist;
    const AABB local{Vec3(c.sh->lmn[0], c.sh->lmn[1], c.sh->lmn[2]), Vec3(c.sh->lmx[0], c.sh->lmx[1], c.sh->lmx[2])};
    AABB sweep = aabb_merge(aabb_transformed(local, c.q0, c.t0), aabb_transformed(local, c.q0, c.t0 + c.disp));
    const Vec3 margin(0.1f, 0.1f, 0.1f);
    c.sweep = AABB{sweep.mn - margin, sweep.mx + margin};
    c.li = b.layer[i];
    c.mi = b.mask[i];
    return c;
}

__device__ __forceinline__ bool ccd_candidate(const DeviceBodies& b, const CcdBody& c, uint32_t i, uint32_t j) {
    if (j == i || (b.flags[j] & KZG_BODY_SENSOR)) return false;
    if ((b.layer[j] & c.mi) == 0u || (c.li & b.mask[j]) == 0u) return false;
    return aabb_overlaps(AABB{V3(b.fat_mn[j]), V3(b.fat_mx[j])}, c.sweep);
}

struct CcdHit {
    float frac;
    uint32_t slot;
    Vec3 n;
};

// This lane's share of body i's candidates (j = lane, lane + nl, ...): the smallest fraction, the
// first such j of the lane on a tie.
// `best` (shared by the lanes working on body i): the smallest fraction any of them has found, as
// int bits (fractions are >= 0), so a lane's advancement stops early once it cannot win.
// Whether body j's position was already integrated when the position loop reaches body i: the loop
// walks the active list (PhysicsWorld.cpp:785-802), which is slot order while nothing has slept;
// with sleeping on, by active-list position, and a sleeping body is never integrated.
__device__ __forceinline__ bool integrated_before(const DeviceBodies& b, uint32_t j, uint32_t i, bool by_rank) {
    return by_rank ? (b.act[j] != 0u && b.apos[j] < b.apos[i]) : j < i;
}

__device__ CcdHit ccd_scan(const ShapeTables& T, const DeviceBodies& b, uint32_t n, uint32_t i, const CcdBody& c,
                           float dt, const float4* disp, uint32_t lane, uint32_t nl, int* best, bool by_rank) {
    CcdHit h{1.0f, kNoHit, Vec3(0.0f, 1.0f, 0.0f)};
    for (uint32_t j = lane; j < n; j += nl) {
        if (!ccd_candidate(b, c, i, j)) continue;
        Vec3 tj = V3(b.pos[j]);
        Quat qj = Q4(b.rot[j]);
        if (b.motion[j] != KZG_MOTION_STATIC && integrated_before(b, j, i, by_rank)) {  // already integrated this step
            tj = tj + (casts_linear(b, j) ? V3(disp[j]) : V3(b.lv[j]) * dt);
            const Vec3 avj = V3(b.av[j]);
            if (avj.len2() > 0.0f) qj = integrate_rotation(qj, avj, dt);
        }
        float frac;
        Vec3 nrm;
        if (cast_shape(T, Body{c.sh, c.q0, c.t0}, c.dir, c.dist, Body{&T.shapes[b.shape[j]], qj, tj}, frac, nrm,
                       best) &&
            frac < h.frac) {
            h.frac = frac;
            h.slot = j;
            h.n = nrm;
            atomicMin(best, __float_as_int(frac));
        }
    }
    return h;
}

__device__ __forceinline__ bool ccd_better(const CcdHit& o, const CcdHit& m) {
    return o.slot != kNoHit && (m.slot == kNoHit || o.frac < m.frac || (o.frac == m.frac && o.slot < m.slot));
}

__device__ __forceinline__ void ccd_finish(const DeviceBodies& b, uint32_t i, const CcdBody& c, const CcdHit& h,
                                           float max_pen, float4* disp) {
    Vec3 d = c.disp;
    if (h.slot != kNoHit) {
        float stop = h.frac * c.dist - max_pen;
        if (stop < 0.0f) stop = 0.0f;
        d = c.dir * stop;
        const float vn = c.lv.dot(h.n);
        if (vn < 0.0f) b.lv[i] = F4(c.lv - h.n * vn, 0.0f);
    }
    disp[i] = F4(d, 0.0f);
}

constexpr uint32_t kPending = 0xFFFFFFFFu;

// Sort keys of the LinearCast bodies by active-list position (sleeping ones last).
__global__ void k_ccd_rank_keys(const DeviceBodies b, const uint32_t* __restrict__ list, uint32_t nlist, uint32_t* keys) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nlist) keys[k] = b.act[list[k]] ? b.apos[list[k]] : 0xFFFFFFFFu;
}
constexpr uint32_t kCcdRounds = 64;
constexpr uint32_t kCcdMaxDeps = 8;  // more predecessors than this: solved by k_ccd_serial

__global__ void k_ccd_init(DeviceBodies b, uint32_t n, const uint32_t* __restrict__ list, uint32_t nlist, float dt,
                           float max_pen, float4* disp, uint32_t* round) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlist) return;
    const uint32_t i = list[k];
    if (!b.act[i]) {  // asleep: not integrated this step
        round[i] = 0u;
        return;
    }
    const Vec3 d = V3(b.lv[i]) * dt;
    const float dist = d.len(), thr = b.prm1[i].w;  // per-body ccdMotionThreshold (PhysicsWorld.cpp:806-807)
    if (casts_linear(b, i) && dist > max_pen && !(thr > 0.0f && dist < thr)) {
        round[i] = kPending;
    } else {
        if (casts_linear(b, i)) disp[i] = F4(d, 0.0f);
        round[i] = 0u;
    }
}

// Each pending body's predecessors: its clampable (pending) LinearCast candidates of lower slot,
// in slot order, at most kCcdMaxDeps (a count above that sends the body to k_ccd_serial).
__global__ void k_ccd_deps(DeviceBodies b, const ShapeDev* __restrict__ shapes, uint32_t n,
                           const uint32_t* __restrict__ list, uint32_t nlist, float dt, const uint32_t* round,
                           uint32_t* deps, uint32_t* ndeps, bool by_rank) {
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (k >= nlist) return;
    const uint32_t i = list[k];
    if (round[i] != kPending) return;
    const ShapeTables T{shapes, nullptr, nullptr, nullptr};
    const CcdBody c = ccd_body(T, b, i, dt);
    uint32_t cnt = 0;
    const uint32_t jend = by_rank ? n : i;
    for (uint32_t j0 = 0; j0 < jend && cnt <= kCcdMaxDeps; j0 += 32u) {
        const uint32_t j = j0 + lane;
        const bool dep = j < jend && integrated_before(b, j, i, by_rank) && casts_linear(b, j) &&
                         round[j] == kPending && ccd_candidate(b, c, i, j);
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, dep);
        const uint32_t pos = cnt + __popc(m & ((1u << lane) - 1u));
        if (dep && pos < kCcdMaxDeps) deps[k * kCcdMaxDeps + pos] = j;
        cnt += __popc(m);
    }
    if (lane == 0) ndeps[k] = cnt;
}

__global__ void k_ccd_round(ShapeTables T, DeviceBodies b, uint32_t n, const uint32_t* __restrict__ list,
                            uint32_t nlist, float dt, float max_pen, float4* disp, uint32_t* round,
                            const uint32_t* __restrict__ deps, const uint32_t* __restrict__ ndeps, uint32_t r,
                            bool by_rank) {
    const uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (k >= nlist) return;
    const uint32_t i = list[k];
    if (round[i] != kPending) return;
    const uint32_t nd = ndeps[k];
    if (nd > kCcdMaxDeps) return;
    const bool wait = lane < nd && round[deps[k * kCcdMaxDeps + lane]] >= r;  // a predecessor not finished
    if (__any_sync(0xFFFFFFFFu, wait)) return;
    __shared__ int s_best[kThreads / 32];
    int* best = &s_best[threadIdx.x >> 5];
    if (lane == 0) *best = __float_as_int(1.0f);
    __syncwarp();
    const CcdBody c = ccd_body(T, b, i, dt);
    CcdHit h = ccd_scan(T, b, n, i, c, dt, disp, lane, 32u, best, by_rank);
    for (uint32_t off = 16; off > 0; off >>= 1) {
        CcdHit o;
        o.frac = __shfl_down_sync(0xFFFFFFFFu, h.frac, off);
        o.slot = __shfl_down_sync(0xFFFFFFFFu, h.slot, off);
        o.n.x = __shfl_down_sync(0xFFFFFFFFu, h.n.x, off);
        o.n.y = __shfl_down_sync(0xFFFFFFFFu, h.n.y, off);
        o.n.z = __shfl_down_sync(0xFFFFFFFFu, h.n.z, off);
        if (ccd_better(o, h)) h = o;
    }
    if (lane == 0) {
        ccd_finish(b, i, c, h, max_pen, disp);
        round[i] = r;
    }
}

__global__ void __launch_bounds__(kCcdThreads) k_ccd_serial(ShapeTables T, DeviceBodies b, uint32_t n,
                                                            const uint32_t* __restrict__ list, uint32_t nlist,
                                                            float dt, float max_pen, float4* disp,
                                                            const uint32_t* __restrict__ round, bool by_rank) {
    __shared__ float s_frac[kCcdThreads];
    __shared__ uint32_t s_slot[kCcdThreads];
    __shared__ float4 s_norm[kCcdThreads];
    __shared__ uint32_t s_slot_of[kCcdThreads];
    __shared__ int s_best;
    const uint32_t tid = threadIdx.x;
    for (uint32_t k0 = 0; k0 < nlist; k0 += kCcdThreads) {
        __syncthreads();
        uint32_t mine = kNoHit;
        if (k0 + tid < nlist) {
            const uint32_t i = list[k0 + tid];
            if (round[i] == kPending) mine = i;
        }
        s_slot_of[tid] = mine;
        __syncthreads();
        for (uint32_t kk = 0; kk < kCcdThreads; ++kk) {
            const uint32_t i = s_slot_of[kk];
            if (i == kNoHit) continue;
            if (tid == 0) s_best = __float_as_int(1.0f);
            __syncthreads();
            const CcdBody c = ccd_body(T, b, i, dt);
            const CcdHit h = ccd_scan(T, b, n, i, c, dt, disp, tid, kCcdThreads, &s_best, by_rank);
            s_frac[tid] = h.frac;
            s_slot[tid] = h.slot;
            s_norm[tid] = F4(h.n, 0.0f);
            __syncthreads();
            for (uint32_t w = kCcdThreads / 2; w > 0; w >>= 1) {
                if (tid < w) {
                    const CcdHit o{s_frac[tid + w], s_slot[tid + w], V3(s_norm[tid + w])};
                    const CcdHit m{s_frac[tid], s_slot[tid], V3(s_norm[tid])};
                    if (ccd_better(o, m)) {
                        s_frac[tid] = o.frac;
                        s_slot[tid] = o.slot;
                        s_norm[tid] = s_norm[tid + w];
                    }
                }
                __syncthreads();
            }
            if (tid == 0) ccd_finish(b, i, c, CcdHit{s_frac[0], s_slot[0], V3(s_norm[0])}, max_pen, disp);
            __syncthreads();
        }
    }
}

__global__ void k_integrate_pos(DeviceBodies b, uint32_t n, float dt, int vel_bias, const float4* __restrict__ ccd_disp) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t mt = b.motion[i];
    if (mt != KZG_MOTION_STATIC && b.act[i]) {  // IntegratePositions and the pseudo-velocity pass walk the active list
        Vec3 p = V3(b.pos[i]);
        Quat q = Q4(b.rot[i]);
        Vec3 lv = V3(b.lv[i]), av = V3(b.av[i]);
        p = p + ((ccd_disp && casts_linear(b, i)) ? V3(ccd_disp[i]) : lv * dt);
        if (av.len2() > 0.0f) q = integrate_rotation(q, av, dt);
        if (!vel_bias) {
            Vec3 pl = V3(b.plv[i]), pa = V3(b.pav[i]);
            if (pl.len2() > 0.0f) p = p + pl * dt;
            if (pa.len2() > 0.0f) q = integrate_rotation(q, pa, dt);
            b.plv[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            b.pav[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        b.pos[i] = F4(p, 0.0f);
        b.rot[i] = F4q(q);
        if (mt == KZG_MOTION_DYNAMIC) {
            Mat3 R = q.to_mat3();
            Mat3 W = (R * M3(&b.iil[3 * i])) * R.transposed();
            b.iiw[3 * i] = F4(W.c0, 0.0f);
            b.iiw[3 * i + 1] = F4(W.c1, 0.0f);
            b.iiw[3 * i + 2] = F4(W.c2, 0.0f);
        }
    }
    b.force[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    b.torque[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// ComputeStateHash words (PhysicsWorld.cpp:1152-1172); the FNV-1a fold runs on the host.
__global__ void k_hash_words(DeviceBodies b, uint32_t n, unsigned long long* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = b.pos[i], q = b.rot[i], l = b.lv[i], a = b.av[i];
    float v[13] = {p.x, p.y, p.z, q.x, q.y, q.z, q.w, l.x, l.y, l.z, a.x, a.y, a.z};
    out[14ull * i] = b.packed[i];
    for (int k = 0; k < 13; ++k) out[14ull * i + 1 + k] = (unsigned long long)(long long)(v[k] * 100000.0f);
}

// ---------------------------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------------------------
#define KZG_CK(x)                                                        \
    do {                                                                 \
        cudaError_t e_ = (x);                                            \
        if (e_ != cudaSuccess) {                                         \
            ctx.err = std::string(#x) + ": " + cudaGetErrorString(e_);   \
            return KZG_ERR_CUDA;                                         \
        }                                                                \
    } while (0)

// ---------------------------------------------------------------------------------------------
// manifold cache table: growth (PhysicsWorld::GetOrCreateCached, PhysicsWorld.cpp:418-433) and
// snapshot loads
// ---------------------------------------------------------------------------------------------
namespace {
struct CacheTable {
    unsigned long long* key = nullptr;
    uint32_t* np = nullptr;
    float4 *pos = nullptr, *imp = nullptr;
    cudaError_t alloc(uint32_t cap, cudaStream_t st) {
        cudaError_t e = cudaMalloc((void**)&key, sizeof(unsigned long long) * cap);
        if (e == cudaSuccess) e = cudaMalloc((void**)&np, sizeof(uint32_t) * cap);
        if (e == cudaSuccess) e = cudaMalloc((void**)&pos, sizeof(float4) * 4 * (size_t)cap);
        if (e == cudaSuccess) e = cudaMalloc((void**)&imp, sizeof(float4) * 4 * (size_t)cap);
        if (e == cudaSuccess) e = cudaMemsetAsync(key, 0, sizeof(unsigned long long) * cap, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(np, 0, sizeof(uint32_t) * cap, st);
        return e;
    }
    void release() {
        for (void* p : {(void*)key, (void*)np, (void*)pos, (void*)imp})
            if (p) cudaFree(p);
        key = nullptr; np = nullptr; pos = nullptr; imp = nullptr;
    }
};
void swap_in(Ctx& ctx, CacheTable& t, uint32_t cap) {
    CacheTable old{ctx.c_key, ctx.c_np, ctx.c_pos, ctx.c_imp};
    ctx.c_key = t.key; ctx.c_np = t.np; ctx.c_pos = t.pos; ctx.c_imp = t.imp;
    ctx.cache_cap = cap;
    ctx.graph_dirty = true;  // the captured step holds the old table's addresses
    old.release();
}
constexpr uint32_t kMaxCacheCap = 1u << 31;
}  // namespace

kzg_status settle_sleep_count(Ctx& ctx) {
    if (!ctx.sleep_count_pending) return KZG_OK;
    ctx.sleep_count_pending = false;
    k_sleep_count_ref<<<1, 256, kSleepCountSmem * (sizeof(uint32_t) + 1), ctx.stream>>>(
        ctx.b, ctx.dcnt, ctx.alist, ctx.con_a, ctx.con_b, ctx.con_bits, ctx.joints, ctx.njoints, ctx.suf,
        reinterpret_cast<uint8_t*>(ctx.smin));
    KZG_CK(cudaGetLastError());
    KZG_CK(cudaMemcpyAsync(&ctx.hcnt->sleep_islands, &ctx.dcnt->sleep_islands, sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, ctx.stream));
    KZG_CK(cudaStreamSynchronize(ctx.stream));
    ctx.stats.num_islands = ctx.hcnt->sleep_islands;
    return KZG_OK;
}

kzg_status cache_reserve(Ctx& ctx, uint64_t entries) {
    uint64_t cap = ctx.cache_cap;
    while (entries * 10u >= cap * 7u && cap < kMaxCacheCap) cap *= 2u;
    if (cap == ctx.cache_cap) return KZG_OK;
    if (ctx.cache_fixed) return KZG_OK;
    KZG_CK(cudaGetLastError());
    CacheTable t;
    cudaError_t e = t.alloc((uint32_t)cap, ctx.stream);
    if (e != cudaSuccess) {
        t.release();
        (void)cudaGetLastError();
        ctx.err = "manifold cache: cannot grow the table to " + std::to_string(cap) + " slots";
        return KZG_ERR_CAPACITY;
    }
    k_cache_rehash<<<blocks_for(ctx.cache_cap), kThreads, 0, ctx.stream>>>(
        ctx.c_key, ctx.c_np, ctx.c_pos, ctx.c_imp, ctx.cache_cap, t.key, t.np, t.pos, t.imp, (uint32_t)cap, ctx.dcnt);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
    if (e != cudaSuccess) {
        t.release();
        ctx.err = std::string("CUDA error: ") + cudaGetErrorString(e);
        return KZG_ERR_CUDA;
    }
    swap_in(ctx, t, (uint32_t)cap);
    return KZG_OK;
}

kzg_status cache_reset(Ctx& ctx, uint32_t cap) {
    if (cap == 0 || (cap & (cap - 1u)) != 0) {
        ctx.err = "manifold cache capacity must be a power of two";
        return KZG_ERR_INVALID;
    }
    if (cap == ctx.cache_cap) {
        KZG_CK(cudaMemsetAsync(ctx.c_key, 0, sizeof(unsigned long long) * cap, ctx.stream));
        KZG_CK(cudaMemsetAsync(ctx.c_np, 0, sizeof(uint32_t) * cap, ctx.stream));
        KZG_CK(cudaStreamSynchronize(ctx.stream));
        return KZG_OK;
    }
    CacheTable t;
    cudaError_t e = t.alloc(cap, ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
    if (e != cudaSuccess) {
        t.release();
        (void)cudaGetLastError();
        ctx.err = "manifold cache: cannot allocate " + std::to_string(cap) + " slots";
        return KZG_ERR_CAPACITY;
    }
    swap_in(ctx, t, cap);
    return KZG_OK;
}

kzg_status cache_scatter(Ctx& ctx, const uint32_t* slots, const unsigned long long* keys, const uint32_t* np,
                         const float4* pos, const float4* imp, uint32_t n) {
    if (n == 0) return KZG_OK;
    for (uint32_t e = 0; e < n; ++e)
        if (slots[e] >= ctx.cache_cap) {
            ctx.err = "manifold cache: slot out of range";
            return KZG_ERR_INVALID;
        }
    const size_t bytes = n * (sizeof(uint32_t) * 2 + sizeof(unsigned long long) + sizeof(float4) * 8) + 16;
    uint8_t* tmp = nullptr;
    KZG_CK(cudaMalloc((void**)&tmp, bytes));
    unsigned long long* dk = reinterpret_cast<unsigned long long*>(tmp);
    float4* dpos = reinterpret_cast<float4*>(tmp + sizeof(unsigned long long) * n + (n & 1u ? 8 : 0));
    float4* dimp = dpos + 4 * (size_t)n;
    uint32_t* ds = reinterpret_cast<uint32_t*>(dimp + 4 * (size_t)n);
    uint32_t* dn = ds + n;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpy(dk, keys, sizeof(unsigned long long) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dpos, pos, sizeof(float4) * 4 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dimp, imp, sizeof(float4) * 4 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ds, slots, sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dn, np, sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_cache_scatter<<<blocks_for(n), kThreads, 0, ctx.stream>>>(ds, dk, dn, dpos, dimp, n, ctx.c_key, ctx.c_np,
                                                                   ctx.c_pos, ctx.c_imp);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
    cudaFree(tmp);
    KZG_CK(e);
    return KZG_OK;
}

static kzg_status fetch_counters(Ctx& ctx) {
    KZG_CK(cudaMemcpyAsync(ctx.hcnt, ctx.dcnt, sizeof(Counters), cudaMemcpyDeviceToHost, ctx.stream));
    KZG_CK(cudaStreamSynchronize(ctx.stream));
    return KZG_OK;
}

size_t cub_temp_bytes(uint32_t max_items) {
    size_t a = 0, b = 0, c = 0, d = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (uint32_t*)nullptr, (uint32_t*)nullptr, (int)max_items);
    cub::DeviceRadixSort::SortKeys(nullptr, b, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                   (int)max_items);
    cub::DeviceScan::ExclusiveSum(nullptr, c, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)max_items);
    cub::DeviceRadixSort::SortPairs(nullptr, d, (uint32_t*)nullptr, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, (int)max_items);
    return std::max(std::max(a, b), std::max(c, d));
}

size_t pack_elements(uint32_t points, uint32_t* cap) {
    *cap = std::min(points, kPackCapMax);
    return (size_t)kClusterGrid * kPackArrays * *cap;
}

size_t cluster_id_words(uint32_t max_cons) { return 2ull * kClusterGrid * kClusterBodies + 2ull * max_cons; }

// Whether this device can hold one k_solve_cluster cluster (checked once in configure_kernels).
static bool g_cluster_ok = false;

cudaError_t configure_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_solve_cta<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * kCtaBodiesMax * sizeof(float4)));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_solve_cta<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(2 * kCtaBodiesMax * sizeof(float4)));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_sleep_count_ref, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kSleepCountSmem * (sizeof(uint32_t) + 1)));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_narrow_epa, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kEpaWarps * sizeof(EpaWarpSmem)));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_narrow_epa, cudaFuncAttributePreferredSharedMemoryCarveout, 100);  // 4 CTAs per SM
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_schedule_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(3 * kSchedCtaBodies * sizeof(uint32_t)));
    if (e != cudaSuccess) return e;
    // the cluster solve needs kClusterCtas co-resident CTAs with 192 KB of shared memory each
    for (const void* f : {(const void*)k_solve_cluster<false>, (const void*)k_solve_cluster<true>}) {
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * kClusterSlots * sizeof(float4)));
        if (e != cudaSuccess) return e;
        if (kClusterCtas > 8) {
            e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (e != cudaSuccess) return e;
        }
    }
    {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(kClusterCtas * kClusterGrid);
        lc.blockDim = dim3(kClusterThreads);
        lc.dynamicSmemBytes = 2 * kClusterSlots * sizeof(float4);
        cudaLaunchAttribute at;
        at.id = cudaLaunchAttributeClusterDimension;
        at.val.clusterDim.x = kClusterCtas;
        at.val.clusterDim.y = 1;
        at.val.clusterDim.z = 1;
        lc.attrs = &at;
        lc.numAttrs = 1;
        int nclusters = 0, nclusters_scalar = 0;
        g_cluster_ok = cudaOccupancyMaxActiveClusters(&nclusters, (void*)k_solve_cluster<false>, &lc) == cudaSuccess &&
                       cudaOccupancyMaxActiveClusters(&nclusters_scalar, (void*)k_solve_cluster<true>, &lc) ==
                           cudaSuccess &&
                       nclusters > 0 && nclusters_scalar > 0;
        cudaGetLastError();
    }
    return mlp_configure_kernels();
}

static int bits_for(uint32_t v) {
    int b = 1;
    while (b < 32 && (1ull << b) <= v) ++b;
    return b;
}

// Stage boundary event (not inside a graph capture: events recorded by graph nodes cannot be
// timed, so a replayed graph is timed as a whole).
static cudaError_t mark(Ctx& ctx, int i) {
    return ctx.capturing ? cudaSuccess : cudaEventRecord(ctx.ev[i], ctx.stream);
}

// Issues one step after the pair list is in ctx.pairs and the pair count is on the device.
// No host synchronisation: every count lives on the device, grids and sorts are sized by the
// context's capacities and kernels stop at the device counts, so the sequence can be captured in
// a CUDA graph.
static kzg_status record_after_pairs(Ctx& ctx, float dt) {
    cudaStream_t st = ctx.stream;
    const uint32_t nb = ctx.nbodies;
    const uint32_t P = ctx.cfg.max_pairs, R = 4u * P;
    ShapeTables T{ctx.shapes, ctx.hull_verts, ctx.face_sizes, ctx.face_idx};
    KZG_CK(mark(ctx, 1));
    k_narrow<<<blocks_for(P, 128), 128, 0, st>>>(T, ctx.b, ctx.pairs, ctx.dcnt, ctx.m_count, ctx.m_data, ctx.m_key,
                                                 ctx.epa_list, static_cast<GjkOut*>(ctx.epa_gjk), ctx.epa_gjk_cap);
    k_narrow_epa<<<152u * 8u, kEpaWarps * 32, kEpaWarps * sizeof(EpaWarpSmem), st>>>(
        T, ctx.b, ctx.pairs, ctx.dcnt, ctx.epa_list, static_cast<const GjkOut*>(ctx.epa_gjk), ctx.epa_gjk_cap,
        ctx.m_count, ctx.m_data, ctx.m_key, &ctx.dcnt->error);
    KZG_CK(mark(ctx, 2));
    k_con_flags<<<blocks_for(P), kThreads, 0, st>>>(ctx.m_count, ctx.m_key, ctx.dcnt, ctx.con_flag);
    size_t tb = ctx.cub_tmp_bytes;
    KZG_CK(cub::DeviceScan::ExclusiveSum(ctx.cub_tmp, tb, ctx.con_flag, ctx.con_index, (int)P, st));
    k_build_constraints<<<blocks_for(P), kThreads, 0, st>>>(
        ctx.pairs, ctx.con_flag, ctx.con_index, ctx.m_count, ctx.m_data, ctx.m_key, ctx.b, ctx.dcnt, ctx.con_pair,
        ctx.con_a, ctx.con_b, ctx.con_np, ctx.con_bits, ctx.con_fr, ctx.con_key, ctx.r, ctx.c_key, ctx.c_np, ctx.c_pos,
        ctx.c_imp, ctx.cache_cap, ctx.ws.warm_start,
        (ctx.mlp.logging || (ctx.mlp.enabled && ctx.mlp.have)) ? ctx.miss_rows : nullptr, ctx.miss_prior);
    // The wake rule, BuildIslands' compact indices over the active list and the active list's order
    // matter whenever a body may be inactive: with sleeping on, or after a body was deactivated by a
    // call (SetBodyActive, DeactivateBody, a loaded world).  With every body active they change
    // nothing, and the step skips them.
    const bool sleeping = ctx.ws.allow_sleeping != 0;
    const bool listed = sleeping || !ctx.all_active;
    if (listed) {
        k_wake<<<1, 32, 0, st>>>(ctx.b, ctx.dcnt, ctx.con_a, ctx.con_b, ctx.alist);
        ++ctx.launches;
    }
    k_integrate_vel<<<blocks_for(nb), kThreads, 0, st>>>(
        ctx.b, nb, make_float3(ctx.ws.gravity[0], ctx.ws.gravity[1], ctx.ws.gravity[2]), dt);
    ctx.launches += 7;  // narrow (2), flags, scan (2), build, integrate
    KZG_CK(mark(ctx, 3));
    PrepParams pp{dt, ctx.ss.baumgarte, ctx.ss.penetration_slop, ctx.ss.restitution_threshold, ctx.ss.max_bias_velocity};
    k_prepare<<<blocks_for(R), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.con_a, ctx.con_b, ctx.con_np, ctx.r, pp);
    ctx.launches += mlp_after_prepare(ctx, dt);
    const uint32_t nj = ctx.njoints;
    if (nj) k_joint_prepare<<<blocks_for(nj), kThreads, 0, st>>>(ctx.b, ctx.joints, nj);
    const uint32_t* node = nullptr;  // island nodes (active list in use); null: every dynamic body is its own
    if (listed) {
        k_act_flags<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, nb, ctx.act_flag);
        tb = ctx.cub_tmp_bytes;
        KZG_CK(cub::DeviceScan::ExclusiveSum(ctx.cub_tmp, tb, ctx.act_flag, ctx.act_scan, (int)nb, st));
        k_act_index<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, ctx.act_flag, ctx.act_scan,
                                                         ctx.dyn2slot);
        k_nodes<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, nb, ctx.dyn2slot, ctx.node, ctx.uf);
        node = ctx.node;
        ctx.launches += 5;  // flags, scan (2), index, nodes
    } else {
        k_uf_init<<<blocks_for(nb), kThreads, 0, st>>>(ctx.uf, nb);
        ++ctx.launches;
    }
    k_uf_union<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.con_a, ctx.con_b, ctx.con_bits, node, ctx.uf);
    if (nj) k_joint_union<<<blocks_for(nj), kThreads, 0, st>>>(ctx.b, ctx.joints, nj, node, ctx.uf);
    if (listed) {
        KZG_CK(cudaMemsetAsync(ctx.root_mark, 0, sizeof(uint32_t) * nb, st));
        k_mark_roots<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, nb, ctx.uf, ctx.root_mark);
        k_count_marks<<<blocks_for(nb), kThreads, 0, st>>>(ctx.root_mark, nb, ctx.dcnt);
        ctx.launches += 2;
    } else {
        k_count_roots<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, nb, ctx.uf, ctx.dcnt);
        ++ctx.launches;
    }
    const int kbits = bits_for(nb);
    const uint32_t pad = (1u << kbits) - 1u;
    k_island_keys<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.con_a, ctx.con_b, ctx.con_bits, node, ctx.uf,
                                                      ctx.isl_key, ctx.isl_con_in, P, pad);
    tb = ctx.cub_tmp_bytes;
    KZG_CK(cub::DeviceRadixSort::SortPairs(ctx.cub_tmp, tb, ctx.isl_key, ctx.isl_key_sorted, ctx.isl_con_in,
                                           ctx.isl_con, (int)P, 0, kbits, st));
    k_island_heads<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.isl_key_sorted, ctx.isl_head, pad);
    tb = ctx.cub_tmp_bytes;
    KZG_CK(cub::DeviceScan::ExclusiveSum(ctx.cub_tmp, tb, ctx.isl_head, ctx.isl_pts, (int)P, st));
    k_island_starts<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.isl_key_sorted, ctx.isl_head, ctx.isl_pts,
                                                        ctx.isl_start, pad);
    const bool lpt = ctx.tune.island_order == KZG_ISLANDS_LARGEST_FIRST;
    if (lpt) {
        KZG_CK(cudaMemsetAsync(ctx.isl_bins, 0, sizeof(uint32_t) * 32, st));
        k_island_bin_count<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.isl_start, ctx.isl_bins);
        k_island_bin_offsets<<<1, 32, 0, st>>>(ctx.isl_bins);
        k_island_bin_scatter<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.isl_start, ctx.isl_bins, ctx.isl_order);
        ctx.launches += 3;
    }
    if (nj) {
        k_joint_keys<<<blocks_for(nj), kThreads, 0, st>>>(ctx.b, ctx.joints, nj, node, ctx.uf, ctx.jkeys);
        tb = ctx.cub_tmp_bytes;
        KZG_CK(cub::DeviceRadixSort::SortKeys(ctx.cub_tmp, tb, ctx.jkeys, ctx.jkeys_sorted, (int)nj, 0, 64, st));
        KZG_CK(cudaMemsetAsync(ctx.jflag, 0, sizeof(uint32_t) * (P + 1), st));
        k_joint_islands<<<blocks_for(nj), kThreads, 0, st>>>(ctx.jkeys_sorted, nj, ctx.dcnt, ctx.isl_key_sorted,
                                                             ctx.isl_start, ctx.jisl, ctx.jisl_cisl, ctx.jflag);
        ctx.launches += 8;  // prepare, union, keys, sort (4 passes), islands
    }
    SchedBufs SB{ctx.isl_start, ctx.isl_con, ctx.con_a, ctx.con_b, ctx.con_np, ctx.con_bits, ctx.r.bias,
                 ctx.b.inv_mass, ctx.is_large, ctx.brec, ctx.body_stamp, ctx.body_loc, ctx.isl_bodies,
                 ctx.last_g, 2u * ctx.cfg.max_pairs, ctx.con_la, ctx.con_lb, ctx.first_w, ctx.first_b,
                 ctx.ids_tmp, ctx.lvl_tmp, ctx.lvl_count, ctx.wl_list, ctx.vl_list, ctx.bl_list, ctx.wl_off,
                 ctx.vl_off, ctx.bl_off, ctx.isl_meta, ctx.isl_small, ctx.isl_large,
                 std::min(ctx.tune.small_island_constraints, kSchedSmallCons),
                 std::min(ctx.tune.warp_island_bodies, kWarpBodies), nj ? ctx.jflag : nullptr, ctx.wait_limit,
                 lpt ? ctx.isl_order : nullptr, ctx.ss.use_simd_solver ? 0u : 1u};
    k_schedule_warp<<<152u * 16u, 128, 0, st>>>(SB, ctx.dcnt);
    k_schedule_cta<<<152u * 2u, kSchedCtaThreads, 3 * kSchedCtaBodies * sizeof(uint32_t), st>>>(SB, ctx.dcnt);
    ctx.launches += 16;  // prepare, union-find (2), island sort (4 CUB passes), heads, scan (2), starts, schedule (2)
    KZG_CK(mark(ctx, 4));
    SolveBufs SV{ctx.isl_start, ctx.con_a, ctx.con_b, ctx.con_bits, ctx.con_la, ctx.con_lb, ctx.isl_meta,
                 ctx.isl_bodies, ctx.wl_list, ctx.vl_list, ctx.bl_list, ctx.wl_off, ctx.vl_off, ctx.bl_off,
                 ctx.isl_small, ctx.isl_large, ctx.r, ctx.b, ctx.ss.velocity_iterations,
                 ctx.ss.position_iterations, ctx.ss.warm_start_factor, ctx.ss.use_velocity_bias,
                 ctx.ss.residual_tolerance, ctx.ss.max_velocity_iterations, ctx.brec, ctx.pk,
                 g_cluster_ok ? ctx.pk_cap : 0u, ctx.isl_con, ctx.cfg.max_pairs, ctx.cl_ids,
                 nj ? ctx.joints : nullptr, ctx.jkeys_sorted, ctx.jisl, ctx.jisl_cisl,
                 lpt ? ctx.isl_order : nullptr, nj ? ctx.jflag : nullptr,
                 std::min(ctx.tune.warp_island_bodies, kWarpBodies)};
    // the batch solver's and the scalar solver's kernels are separate instantiations (kScalar)
    const bool simd = ctx.ss.use_simd_solver != 0;
    auto* k_warp = simd ? k_solve_warp<false> : k_solve_warp<true>;
    auto* k_cta = simd ? k_solve_cta<false> : k_solve_cta<true>;
    auto* k_big = simd ? k_solve_big<false> : k_solve_big<true>;
    k_warp<<<152u * 16u, kWarpsPerBlock * 32, kWarpsPerBlock * 2 * kWarpBodies * sizeof(float4), st>>>(SV, ctx.dcnt);
    k_cta<<<152u * 2u, kCtaThreads, 2 * kCtaBodiesMax * sizeof(float4), st>>>(SV, ctx.dcnt, kCtaBodiesMax);
    if (g_cluster_ok) {
        auto* kern = simd ? k_solve_cluster<false> : k_solve_cluster<true>;
        kern<<<kClusterCtas * kClusterGrid, kClusterThreads, 2 * kClusterSlots * sizeof(float4), st>>>(
            SV, ctx.dcnt, kCtaBodiesMax);
        ++ctx.launches;
    }
    k_big<<<152u, kBigThreads, 0, st>>>(SV, ctx.dcnt, kCtaBodiesMax);
    ctx.launches += 3;
    if (nj) {
        auto* k_joint = simd ? k_solve_joint<false> : k_solve_joint<true>;
        k_joint<<<152u * 8u, kJointThreads, 0, st>>>(SV, ctx.dcnt);
        ++ctx.launches;
    }
    ctx.launches += mlp_after_solve(ctx, dt);
    KZG_CK(mark(ctx, 5));
    k_cache_store<<<blocks_for(P), kThreads, 0, st>>>(ctx.dcnt, ctx.con_key, ctx.con_np, ctx.r, ctx.c_key, ctx.c_np,
                                                      ctx.c_pos, ctx.c_imp, ctx.cache_cap);
    const bool ccd = ctx.ws.use_ccd && ctx.nccd > 0;
    if (ccd) {
        ShapeTables T{ctx.shapes, ctx.hull_verts, ctx.face_sizes, ctx.face_idx};
        const float mp = ctx.ws.ccd_max_penetration;
        // the position loop's order: the active list's (slot order while every body is active)
        const uint32_t* list = ctx.ccd_list;
        if (listed) {
            k_ccd_rank_keys<<<blocks_for(ctx.nccd), kThreads, 0, st>>>(ctx.b, ctx.ccd_list, ctx.nccd, ctx.ccd_rank_keys);
            size_t tbc = ctx.cub_tmp_bytes;
            KZG_CK(cub::DeviceRadixSort::SortPairs(ctx.cub_tmp, tbc, ctx.ccd_rank_keys, ctx.ccd_keys_sorted,
                                                   ctx.ccd_list, ctx.ccd_sorted, (int)ctx.nccd, 0, 32, st));
            list = ctx.ccd_sorted;
            ctx.launches += 5;
        }
        k_ccd_init<<<blocks_for(ctx.nccd), kThreads, 0, st>>>(ctx.b, nb, list, ctx.nccd, dt, mp, ctx.ccd_disp,
                                                               ctx.ccd_state);
        k_ccd_deps<<<blocks_for(32u * ctx.nccd), kThreads, 0, st>>>(ctx.b, ctx.shapes, nb, list, ctx.nccd,
                                                                    dt, ctx.ccd_state, ctx.ccd_deps, ctx.ccd_ndeps,
                                                                    listed);
        for (uint32_t r = 1; r <= kCcdRounds; ++r)
            k_ccd_round<<<blocks_for(32u * ctx.nccd), kThreads, 0, st>>>(T, ctx.b, nb, list, ctx.nccd, dt, mp,
                                                                         ctx.ccd_disp, ctx.ccd_state, ctx.ccd_deps,
                                                                         ctx.ccd_ndeps, r, listed);
        k_ccd_serial<<<1, kCcdThreads, 0, st>>>(T, ctx.b, nb, list, ctx.nccd, dt, mp, ctx.ccd_disp,
                                                ctx.ccd_state, listed);
        ctx.launches += 3 + kCcdRounds;
    }
    k_integrate_pos<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, nb, dt, ctx.ss.use_velocity_bias,
                                                         ccd ? ctx.ccd_disp : nullptr);
    ctx.launches += 2;
    if (nj) {
        k_joint_positions<<<blocks_for(nj), kThreads, 0, st>>>(ctx.b, ctx.joints, ctx.jkeys_sorted, ctx.jisl,
                                                               ctx.dcnt, ctx.ss.position_iterations);
        ++ctx.launches;
    }
    if (sleeping) {  // UpdateSleeping (PhysicsWorld.cpp:866-951)
        const float lin2 = ctx.ws.sleep_linear_threshold * ctx.ws.sleep_linear_threshold;
        const float ang2 = ctx.ws.sleep_angular_threshold * ctx.ws.sleep_angular_threshold;
        k_sleep_begin<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, nb, lin2, ang2, dt, ctx.suf,
                                                           ctx.smin);
        k_sleep_union<<<blocks_for(P), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.con_a, ctx.con_b, ctx.con_bits, ctx.suf);
        if (nj) k_sleep_union_joints<<<blocks_for(nj), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.joints, nj, ctx.suf);
        k_sleep_min<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, ctx.suf, ctx.smin);
        k_sleep_mark<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, ctx.suf, ctx.smin,
                                                          ctx.ws.sleep_time_threshold, ctx.smark);
        k_sleep_remove<<<1, 32, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, ctx.smark);
        k_sleep_count<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.dcnt, ctx.alist, ctx.suf);
        ctx.launches += nj ? 7 : 6;
    }
    KZG_CK(mark(ctx, 6));
    KZG_CK(cudaGetLastError());
    return KZG_OK;
}

static kzg_status finish_stats(Ctx& ctx, uint32_t graph_steps = 0) {
    Counters& h = *ctx.hcnt;
    if (!ctx.all_active && h.nact == ctx.nbodies) {  // every body active again: back to the short step
        ctx.all_active = true;
        ctx.graph_dirty = true;
    }
    kzg_stats& s = ctx.stats;
    s.num_bodies = ctx.nbodies;
    s.num_broadphase_pairs = h.npairs;
    s.num_contact_constraints = h.ncons;
    s.num_contact_points = h.npoints;
    // WorldStats::numIslands: BuildIslands' count, replaced by UpdateSleeping's when that pass ran
    // (the exact one is counted on demand, settle_sleep_count)
    s.num_islands = (ctx.ws.allow_sleeping && h.nsleep_n) ? h.sleep_islands : h.nroots;
    ctx.sleep_count_pending = ctx.ws.allow_sleeping && h.nsleep_n;
    s.num_active_bodies = h.nact;
    s.cache_capacity = ctx.cache_cap;
    s.num_epa_pairs = h.nepa;
    s.num_batches = h.batches;
    s.max_velocity_levels = h.max_vlev;
    s.max_bias_levels = h.max_blev;
    s.cache_entries = h.cache_entries;
    s.device_error = h.error;
    s.kernel_launches = ctx.launches;
    s.max_velocity_iterations_used = h.max_iters;
    s.point_velocity_iterations = h.pt_iters;
    memcpy(&s.final_residual, &h.res_bits, sizeof(float));
    if (graph_steps) {  // replayed graph: its mean step time, no stage split
        float ms = 0.0f;
        KZG_CK(cudaEventElapsedTime(&ms, ctx.ev[0], ctx.ev[6]));
        s.broadphase_ms = s.narrowphase_ms = s.constraints_ms = s.schedule_ms = s.solve_ms = s.integrate_ms = 0.0f;
        s.step_ms = ms / (float)graph_steps;
    } else {
        KZG_CK(cudaEventElapsedTime(&s.broadphase_ms, ctx.ev[0], ctx.ev[1]));
        KZG_CK(cudaEventElapsedTime(&s.narrowphase_ms, ctx.ev[1], ctx.ev[2]));
        KZG_CK(cudaEventElapsedTime(&s.constraints_ms, ctx.ev[2], ctx.ev[3]));
        KZG_CK(cudaEventElapsedTime(&s.schedule_ms, ctx.ev[3], ctx.ev[4]));
        KZG_CK(cudaEventElapsedTime(&s.solve_ms, ctx.ev[4], ctx.ev[5]));
        KZG_CK(cudaEventElapsedTime(&s.integrate_ms, ctx.ev[5], ctx.ev[6]));
        KZG_CK(cudaEventElapsedTime(&s.step_ms, ctx.ev[0], ctx.ev[6]));
    }
    // A wait that gave up is a warning: its work was redone by the waiting kernel, the step is complete.
    if (h.error & ~KZG_DEVERR_WAIT) {
        ctx.err = "device error word " + std::to_string(h.error) + " (see KZG_DEVERR_*)";
        return (h.error & (KZG_DEVERR_PAIRS | KZG_DEVERR_CACHE)) ? KZG_ERR_CAPACITY : KZG_ERR_DEVICE;
    }
    return KZG_OK;
}

// One canonical step (GPU broad phase).  Stepped directly it reads the pair count back once (the pair
// sort covers that count); while a graph is captured it issues no host synchronisation.
static kzg_status record_canonical(Ctx& ctx, float dt) {
    cudaStream_t st = ctx.stream;
    KZG_CK(cudaPeekAtLastError());
    const uint32_t nb = ctx.nbodies, P = ctx.cfg.max_pairs;
    const uint32_t kb = (uint32_t)bits_for(nb);  // bits of a packed id (packed ids are slots)
    ctx.launches = 0;
    k_begin_step<<<1, 32, 0, st>>>(ctx.dcnt);
    KZG_CK(mark(ctx, 0));
    k_aabb<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, ctx.shapes, nb, 1.0f / ctx.cell_size, ctx.is_large,
                                                ctx.cell_keys, ctx.cell_vals, ctx.ws.fixed_timestep);
    size_t tb = ctx.cub_tmp_bytes;
    KZG_CK(cub::DeviceRadixSort::SortPairs(ctx.cub_tmp, tb, ctx.cell_keys, ctx.cell_keys_sorted, ctx.cell_vals,
                                           ctx.cell_vals_sorted, (int)nb, 0, 64, st));
    const uint32_t nsmall = nb - ctx.nlarge;
    k_find_pairs<<<blocks_for(nb), kThreads, 0, st>>>(ctx.b, nb, ctx.cell_keys_sorted, ctx.cell_vals_sorted, nsmall,
                                                      1.0f / ctx.cell_size, ctx.is_large, ctx.large_list,
                                                      ctx.large_off, ctx.nworlds, ctx.pair_keys, ctx.dcnt, P, kb);
    k_clamp_pairs<<<1, 1, 0, st>>>(ctx.dcnt, P);
    // The pair sort's size: in a captured graph the capacity, the keys past the pair count padded to
    // sort last; stepped directly, the pair count itself, read back here (one round trip instead of
    // radix passes over the whole capacity).
    uint32_t nsort = P;
    if (ctx.capturing) {
        k_pad_keys<<<blocks_for(P), kThreads, 0, st>>>(ctx.pair_keys, ctx.dcnt, P);
        ++ctx.launches;
    } else {
        KZG_CK(cudaMemcpyAsync(&ctx.hcnt->npairs, &ctx.dcnt->npairs, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        KZG_CK(cudaStreamSynchronize(st));
        nsort = std::min(ctx.hcnt->npairs, P);
    }
    if (nsort) {
        tb = ctx.cub_tmp_bytes;
        KZG_CK(cub::DeviceRadixSort::SortKeys(ctx.cub_tmp, tb, ctx.pair_keys, ctx.pair_keys_sorted, (int)nsort, 0,
                                              2 * kb, st));
        k_unpack_pairs<<<blocks_for(nsort), kThreads, 0, st>>>(ctx.pair_keys_sorted, ctx.dcnt, ctx.pairs, kb);
    }
    ctx.launches += 15;  // begin, aabb, cell sort (4 CUB passes), find pairs, clamp, key sort (4+), unpack
    return record_after_pairs(ctx, dt);
}

// Capture one canonical step into a CUDA graph (once per dt and configuration).
static kzg_status ensure_graph(Ctx& ctx, float dt) {
    if (ctx.graph_exec && !ctx.graph_dirty && ctx.graph_dt == dt) return KZG_OK;
    KZG_CK(cudaGetLastError());
    if (ctx.graph_exec) cudaGraphExecDestroy(ctx.graph_exec);
    ctx.graph_exec = nullptr;
    cudaGraph_t g = nullptr;
    KZG_CK(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
    ctx.capturing = true;
    kzg_status s = record_canonical(ctx, dt);
    ctx.capturing = false;
    cudaError_t e = cudaStreamEndCapture(ctx.stream, &g);
    if (s != KZG_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    KZG_CK(e);
    e = cudaGraphInstantiate(&ctx.graph_exec, g, 0);
    cudaGraphDestroy(g);
    KZG_CK(e);
    ctx.graph_dt = dt;
    ctx.graph_dirty = false;
    ctx.graph_launches = ctx.launches;
    return KZG_OK;
}

// New cache entries one step may add: at most one per contact constraint, so at most the pair
// count; the last step's pair count (or the body count, if larger) stands for the next one's.
static uint64_t cache_step_estimate(const Ctx& ctx) {
    return std::max<uint64_t>(std::max<uint64_t>(ctx.hcnt->npairs, ctx.nbodies), 1u);
}

kzg_status step_canonical(Ctx& ctx, float dt, uint32_t nsteps) {
    kzg_status s = fetch_counters(ctx);  // cache entries as the device holds them
    if (s != KZG_OK) return s;
    if (ctx.use_graph) {
        // Replayed in runs that fit the cache: before each run the table is grown to hold two
        // steps' worth of new entries below 0.7 load, and the run is as long as that headroom lasts.
        KZG_CK(cudaEventRecord(ctx.ev[0], ctx.stream));
        for (uint32_t done = 0; done < nsteps;) {
            const uint64_t est = cache_step_estimate(ctx), have = ctx.hcnt->cache_entries;
            s = cache_reserve(ctx, have + 2u * est);
            if (s != KZG_OK) return s;
            s = ensure_graph(ctx, dt);
            if (s != KZG_OK) return s;
            const uint64_t room = (uint64_t)ctx.cache_cap * 7u / 10u;
            uint64_t run = room > have ? (room - have) / est : 0u;
            run = std::min<uint64_t>(std::max<uint64_t>(run, 1u), nsteps - done);
            for (uint64_t i = 0; i < run; ++i) KZG_CK(cudaGraphLaunch(ctx.graph_exec, ctx.stream));
            done += (uint32_t)run;
            if (done < nsteps) {
                s = fetch_counters(ctx);
                if (s != KZG_OK) return s;
            }
        }
        KZG_CK(cudaEventRecord(ctx.ev[6], ctx.stream));
        ctx.frame += nsteps;
        ctx.launches = ctx.graph_launches;
        s = fetch_counters(ctx);
        if (s != KZG_OK) return s;
        return finish_stats(ctx, nsteps);
    }
    for (uint32_t i = 0; i < nsteps; ++i) {
        s = cache_reserve(ctx, (uint64_t)ctx.hcnt->cache_entries + cache_step_estimate(ctx));
        if (s != KZG_OK) return s;
        ++ctx.frame;
        s = record_canonical(ctx, dt);
        if (s != KZG_OK) return s;
        s = fetch_counters(ctx);
        if (s != KZG_OK) return s;
        s = finish_stats(ctx);
        if (s != KZG_OK) return s;
    }
    return KZG_OK;
}

kzg_status step_external(Ctx& ctx, const uint32_t* host_pairs, uint32_t np, float dt) {
    cudaStream_t st = ctx.stream;
    if (np > ctx.cfg.max_pairs) {
        ctx.err = "pair count exceeds kzg_config.max_pairs";
        return KZG_ERR_CAPACITY;
    }
    kzg_status s = fetch_counters(ctx);
    if (s != KZG_OK) return s;
    s = cache_reserve(ctx, (uint64_t)ctx.hcnt->cache_entries + np);  // at most one new entry per pair
    if (s != KZG_OK) return s;
    ++ctx.frame;
    ctx.launches = np > 0 ? 3 : 2;
    k_begin_step<<<1, 32, 0, st>>>(ctx.dcnt);
    KZG_CK(cudaEventRecord(ctx.ev[0], st));
    if (ctx.nbodies) k_fat<<<blocks_for(ctx.nbodies), kThreads, 0, st>>>(ctx.b, ctx.shapes, ctx.nbodies, ctx.ws.fixed_timestep);
    if (np > 0) {
        KZG_CK(cudaMemcpyAsync(ctx.pair_keys, host_pairs, sizeof(uint32_t) * 2 * np, cudaMemcpyHostToDevice, st));
        k_pairs_from_packed<<<blocks_for(np), kThreads, 0, st>>>((const uint32_t*)ctx.pair_keys, np, ctx.b,
                                                                 ctx.nbodies, ctx.pairs);
    }
    KZG_CK(cudaMemcpyAsync(&ctx.dcnt->npairs, &np, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    s = record_after_pairs(ctx, dt);
    if (s != KZG_OK) return s;
    s = fetch_counters(ctx);
    if (s != KZG_OK) return s;
    return finish_stats(ctx);
}

// PhysicsWorld::SetBodyActive / ActivateBody / DeactivateBody (PhysicsWorld.cpp:108-111, 132-133;
// BodyManager.cpp:133-160) for a list of packed BodyIDs, one after another in the given order; stale
// ids are skipped.  One thread: the active list is order-dependent.
__device__ void activate_slot(DeviceBodies& b, uint32_t* alist, uint32_t& size, uint32_t x) {
    if (b.act[x]) return;
    b.act[x] = 1u;
    b.sleep_t[x] = 0.0f;
    b.apos[x] = size;
    alist[size++] = x;
}
__device__ void deactivate_slot(DeviceBodies& b, uint32_t* alist, uint32_t& size, uint32_t x) {
    if (!b.act[x]) return;
    b.act[x] = 0u;
    b.lv[x] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    b.av[x] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint32_t at = b.apos[x], last = size - 1u;
    if (at != last) {
        const uint32_t moved = alist[last];
        alist[at] = moved;
        b.apos[moved] = at;
    }
    b.apos[x] = kInvalid;
    --size;
}
__device__ __forceinline__ bool live_slot(const DeviceBodies& b, uint32_t id, uint32_t nb, uint32_t* x) {
    *x = id & 0x00FFFFFFu;
    return *x < nb && b.packed[*x] == id;
}

__global__ void k_set_active(DeviceBodies b, Counters* cnt, uint32_t* alist, const uint32_t* __restrict__ ids, uint32_t n,
                             uint32_t nb, int active) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t size = cnt->nact;
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t x;
        if (!live_slot(b, ids[k], nb, &x)) continue;
        if (active) activate_slot(b, alist, size, x);
        else deactivate_slot(b, alist, size, x);
    }
    cnt->nact = size;
}

// PhysicsWorld's convenience body operations (PhysicsWorld.cpp:135-205; Body.h:149-203) in the given
// order; one thread, since waking appends to the active list.
__device__ void set_world_inertia(DeviceBodies& b, uint32_t x, const Quat& q) {  // UpdateWorldInertia (Body.h:121-124)
    const Mat3 R = q.to_mat3();
    const Mat3 W = (R * M3(&b.iil[3 * x])) * R.transposed();
    b.iiw[3 * x] = F4(W.c0, 0.0f);
    b.iiw[3 * x + 1] = F4(W.c1, 0.0f);
    b.iiw[3 * x + 2] = F4(W.c2, 0.0f);
}
__global__ void k_edit_bodies(DeviceBodies b, Counters* cnt, uint32_t* alist, const kzg_body_edit* __restrict__ e,
                              uint32_t n, uint32_t nb) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t size = cnt->nact;
    for (uint32_t k = 0; k < n; ++k) {
        const kzg_body_edit ed = e[k];
        uint32_t x;
        if (!live_slot(b, ed.body, nb, &x)) continue;
        const bool dyn = b.motion[x] == KZG_MOTION_DYNAMIC;
        const Vec3 v0(ed.v[0], ed.v[1], ed.v[2]), v1(ed.v[3], ed.v[4], ed.v[5]);
        switch (ed.op) {
            case KZG_EDIT_SET_POSITION: b.pos[x] = F4(v0, 0.0f); break;
            case KZG_EDIT_SET_ROTATION: {
                const Quat q = Quat(ed.v[0], ed.v[1], ed.v[2], ed.v[3]).normalized();
                b.rot[x] = F4q(q);
                set_world_inertia(b, x, q);
                break;
            }
            case KZG_EDIT_SET_TRANSFORM: {
                const Quat q(ed.v[3], ed.v[4], ed.v[5], ed.v[6]);
                b.pos[x] = F4(v0, 0.0f);
                b.rot[x] = F4q(q);
                set_world_inertia(b, x, q);
                break;
            }
            case KZG_EDIT_SET_LINEAR_VELOCITY: b.lv[x] = F4(v0, 0.0f); break;
            case KZG_EDIT_SET_ANGULAR_VELOCITY: b.av[x] = F4(v0, 0.0f); break;
            case KZG_EDIT_ADD_FORCE:
                if (dyn) b.force[x] = F4(V3(b.force[x]) + v0, 0.0f);
                break;
            case KZG_EDIT_ADD_FORCE_AT_POINT:
                if (dyn) {
                    b.force[x] = F4(V3(b.force[x]) + v0, 0.0f);
                    b.torque[x] = F4(V3(b.torque[x]) + (v1 - V3(b.pos[x])).cross(v0), 0.0f);
                }
                break;
            case KZG_EDIT_ADD_TORQUE:
                if (dyn) b.torque[x] = F4(V3(b.torque[x]) + v0, 0.0f);
                break;
            case KZG_EDIT_ADD_IMPULSE:
                if (dyn) b.lv[x] = F4(V3(b.lv[x]) + v0 * b.inv_mass[x], 0.0f);
                break;
            case KZG_EDIT_ADD_IMPULSE_AT_POINT:
                if (dyn) {
                    b.lv[x] = F4(V3(b.lv[x]) + v0 * b.inv_mass[x], 0.0f);
                    const Vec3 r = v1 - V3(b.pos[x]);
                    b.av[x] = F4(V3(b.av[x]) + M3(&b.iiw[3 * x]) * r.cross(v0), 0.0f);
                }
                break;
            case KZG_EDIT_ACTIVATE: activate_slot(b, alist, size, x); continue;
            case KZG_EDIT_DEACTIVATE: deactivate_slot(b, alist, size, x); continue;
            default: continue;
        }
        if (ed.wake) activate_slot(b, alist, size, x);
    }
    cnt->nact = size;
}

cudaError_t edit_bodies(Ctx& ctx, const kzg_body_edit* dev_edits, uint32_t n) {
    k_edit_bodies<<<1, 1, 0, ctx.stream>>>(ctx.b, ctx.dcnt, ctx.alist, dev_edits, n, ctx.nbodies);
    cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : cudaStreamSynchronize(ctx.stream);
}

// Host transfers through one contiguous staging buffer (the state-hash scratch, 28 floats per body):
// one plain copy each way instead of strided copies with 12- and 16-byte rows.
__global__ void k_scatter_forces(DeviceBodies b, const float* __restrict__ ft, uint32_t first, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* f = ft + 6ull * i;
    b.force[first + i] = make_float4(f[0], f[1], f[2], 0.0f);
    b.torque[first + i] = make_float4(f[3], f[4], f[5], 0.0f);
}
__global__ void k_gather_transforms(const DeviceBodies b, float* out, uint32_t first, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = b.pos[first + i], q = b.rot[first + i];
    float* o = out + 7ull * i;
    o[0] = p.x; o[1] = p.y; o[2] = p.z;
    o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
}
kzg_status upload_forces(Ctx& ctx, const float* host_ft, uint32_t first, uint32_t n) {
    if (n == 0) return KZG_OK;
    float* stage = reinterpret_cast<float*>(ctx.hash_words);
    KZG_CK(cudaMemcpyAsync(stage, host_ft, sizeof(float) * 6ull * n, cudaMemcpyHostToDevice, ctx.stream));
    k_scatter_forces<<<blocks_for(n), kThreads, 0, ctx.stream>>>(ctx.b, stage, first, n);
    KZG_CK(cudaGetLastError());
    return KZG_OK;
}
kzg_status download_transforms(Ctx& ctx, float* host_out, uint32_t first, uint32_t n) {
    if (n == 0) return KZG_OK;
    float* stage = reinterpret_cast<float*>(ctx.hash_words);
    k_gather_transforms<<<blocks_for(n), kThreads, 0, ctx.stream>>>(ctx.b, stage, first, n);
    KZG_CK(cudaGetLastError());
    KZG_CK(cudaMemcpyAsync(host_out, stage, sizeof(float) * 7ull * n, cudaMemcpyDeviceToHost, ctx.stream));
    KZG_CK(cudaStreamSynchronize(ctx.stream));
    return KZG_OK;
}

cudaError_t set_bodies_active(Ctx& ctx, const uint32_t* dev_ids, uint32_t n, int active) {
    k_set_active<<<1, 1, 0, ctx.stream>>>(ctx.b, ctx.dcnt, ctx.alist, dev_ids, n, ctx.nbodies, active);
    cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : cudaStreamSynchronize(ctx.stream);
}

cudaError_t init_new_bodies(Ctx& ctx, uint32_t first, uint32_t n) {
    if (n == 0) return cudaSuccess;
    k_init_bodies<<<blocks_for(n), kThreads, 0, ctx.stream>>>(ctx.b, ctx.shapes, first, n, ctx.alist, ctx.dcnt);
    k_grow_active<<<1, 1, 0, ctx.stream>>>(ctx.dcnt, n);
    cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : cudaStreamSynchronize(ctx.stream);
}

kzg_status hash_state(Ctx& ctx, uint64_t* out) {
    const uint32_t nb = ctx.nbodies;
    std::vector<unsigned long long> w(14ull * nb);
    if (nb) {
        k_hash_words<<<blocks_for(nb), kThreads, 0, ctx.stream>>>(ctx.b, nb, ctx.hash_words);
        KZG_CK(cudaMemcpyAsync(w.data(), ctx.hash_words, sizeof(unsigned long long) * w.size(), cudaMemcpyDeviceToHost,
                               ctx.stream));
        KZG_CK(cudaStreamSynchronize(ctx.stream));
    }
    uint64_t h = 1469598103934665603ull;
    for (unsigned long long v : w) {
        h ^= v;
        h *= 1099511628211ull;
    }
    *out = h;
    return KZG_OK;
}

}  // namespace kzg
