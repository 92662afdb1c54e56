// kzg_schedule.cuh - per-island solve schedule (included by kzg_solver.cuh).
//
// For every island this builds, bit-compatible with the reference:
//   * the greedy first-fit batches of contact points (at most 4 per batch, no body - static ones
//     included - twice in a batch, sensors skipped; PhysicsWorld.cpp:680-717);
//   * the dependency levels of the three sequential sweeps of SolveIsland (:666-743):
//       warm start : every point in island constraint order
//       velocity   : batch order
//       bias       : points with positionBias > 0, island constraint order, constraints with a
//                    massive body only (ContactSolver.cpp:263-267)
//     A point's level is one more than the last level of the same sweep on either of its dynamic
//     bodies; all points of one level touch distinct dynamic bodies and commute exactly.
//
// Only the first-fit itself is sequential.  In a CTA island one warp runs it over a shared-memory
// table of the open batches (first_fit_warp: 32 candidates per ballot against 16-bit body
// codes).  Small islands, and islands whose open batches outgrow that table, run it on one lane
// with union-find "next usable batch" skip structures stored in 64-byte batch records, so each
// point costs O(its bodies' degree) instead of the reference's O(batches): one structure skips
// full batches, and one per hub body (the island's planes) also skips batches already holding
// that hub.  Local body indices, hub detection, the level sweeps (32-item warp windows resolved
// with shuffles) and the level sorts run in parallel.  Small islands take one warp, large ones
// one CTA.
#pragma once

namespace kzg {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kWarpBodies = 384;      // island velocities staged per warp (warp-per-island solve)
constexpr uint32_t kWarpsPerBlock = 4;
constexpr uint32_t kCtaThreads = 256;
constexpr uint32_t kCtaBodiesMax = 6400;   // island velocities staged per CTA (2 x 16 B x 6400 = 200 KB)
constexpr uint32_t kSchedSmallCons = 128;  // islands with at most this many constraints: warp schedule
constexpr uint32_t kSchedWarpBodies = 2 * kSchedSmallCons;
constexpr uint32_t kSchedCtaBodies = 16384;  // per-sweep level table in shared memory (3 x 64 KB)

struct SchedBufs {
    const uint32_t *isl_start, *isl_con, *con_a, *con_b, *con_np, *con_bits;
    const float4* bias;
    const float* inv_mass;
    const uint8_t* is_large;   // planes and other grid-bypassing bodies: hub candidates
    uint4* brec;               // batch records (64 B): {nx, hub0 nx, hub1 nx, count}, 8 bodies, 4 rows
    uint32_t *body_stamp, *body_loc;
    uint32_t *isl_bodies;      // per island dynamic bodies, region 2*s0
    uint32_t *last_g;          // level tables when they do not fit shared memory: 3 x (2P)
    uint32_t last_stride;
    uint32_t *con_la, *con_lb; // per constraint local index of A / B (kNone if not dynamic)
    uint32_t *first_w, *first_b;  // per sorted constraint position: first warm / bias level
    uint32_t *vitems, *vlev;   // per point region: velocity items in batch order and their level
    uint32_t *lvl_count;
    uint32_t *wl_list, *vl_list, *bl_list, *wl_off, *vl_off, *bl_off, *meta;
    uint32_t *small_list, *large_list;
    uint32_t small_cons;   // islands with at most this many constraints: warp schedule (<= kSchedSmallCons)
    uint32_t warp_bodies;  // islands with at most this many dynamic bodies: warp solve (<= kWarpBodies)
    const uint32_t* jflag; // per island: 1 when joints share it (solved with them by k_solve_big), or null
    uint32_t spin_limit;   // polls before the streamed velocity sweep's wait gives up
    const uint32_t* order; // largest-first island order taken from shared counters, or null: island order
    uint32_t scalar;       // SolverSettings::useSIMDSolver = false: no batches; the velocity sweep visits
                           // every point in island order, so its levels are the warm start's
};

struct SchedShared {  // per island scratch living in shared memory
    uint32_t nloc, hub0, hub1, nbt, nv, nw, nb, total, ff_ok;
    uint32_t ff_final;   // streamed first fit: batches below this are full and their records written
    uint32_t ff_done;    // 0 running, 1 done (nbt set), 2 gave up
    uint32_t stream_ok;  // the velocity level sweep ran behind the first fit
};

__device__ __forceinline__ uint32_t* rec(const SchedBufs& S, uint32_t r) { return reinterpret_cast<uint32_t*>(S.brec + 4ull * r); }

// smallest usable batch >= i along skip structure `f` (path halving; links only point forward)
__device__ __forceinline__ uint32_t nx_find(const SchedBufs& S, uint32_t rb, uint32_t f, uint32_t i) {
    for (;;) {
        uint32_t p = rec(S, rb + i)[f];
        if (p == i) return i;
        uint32_t gp = rec(S, rb + p)[f];
        rec(S, rb + i)[f] = gp;
        i = gp;
    }
}

__device__ __forceinline__ bool rec_has(const uint32_t* r, uint32_t x) {
    const uint32_t n = 2 * r[3];
    for (uint32_t k = 0; k < n; ++k)
        if (r[4 + k] == x) return true;
    return false;
}

// Exclusive scan of v over a group of `nthreads` threads (tid < nthreads); returns the prefix and
// writes the group total to *total.  tmp: at least 33 words of shared memory.
template <typename Sync>
__device__ uint32_t group_scan(uint32_t v, uint32_t tid, uint32_t nthreads, uint32_t* tmp, uint32_t* total, Sync sync) {
    const uint32_t lane = tid & 31u, warp = tid >> 5, nwarps = (nthreads + 31) >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) tmp[warp] = x;
    sync();
    if (tid == 0) {
        uint32_t run = 0;
        for (uint32_t w = 0; w < nwarps; ++w) { uint32_t t = tmp[w]; tmp[w] = run; run += t; }
        tmp[32] = run;
    }
    sync();
    const uint32_t r = tmp[warp] + x - v;
    *total = tmp[32];
    sync();
    return r;
}

// One 32-item window of a sequential level sweep, resolved by one warp.  Item i has dynamic body
// slots (la, lb) in the level table `last` (kNone if absent) and occupies `len` consecutive levels;
// returns its first level and advances `last` exactly as a sequential pass would.
__device__ __forceinline__ uint32_t level_window(uint32_t* last, bool valid, uint32_t la, uint32_t lb, uint32_t len,
                                                 uint32_t lane) {
    const unsigned full = 0xffffffffu;
    if (!valid) { la = kNone; lb = kNone; len = 0; }
    uint32_t base = 0;
    if (la != kNone) base = last[la];
    if (lb != kNone) base = max(base, last[lb]);
    bool supA = false, supB = false;
    for (uint32_t j = 0; j < 32; ++j) {
        const uint32_t aj = __shfl_sync(full, la, j), bj = __shfl_sync(full, lb, j);
        const uint32_t ej = __shfl_sync(full, base, j) + __shfl_sync(full, len, j);
        const bool hitA = la != kNone && (la == aj || la == bj);
        const bool hitB = lb != kNone && (lb == aj || lb == bj);
        if (lane > j && (hitA || hitB) && ej > base) base = ej;
        if (j > lane) { supA |= hitA; supB |= hitB; }
    }
    const uint32_t end = base + len;
    __syncwarp();
    if (la != kNone && !supA) last[la] = end;
    if (lb != kNone && !supB) last[lb] = end;
    __syncwarp();
    return base + 1;
}

// Counting sort of one sweep's points by level into list/off (order inside a level is free).
// The level counters live in shared memory (scnt, scap words) when they fit.
template <typename Sync, typename Emit>
__device__ void level_sort(const SchedBufs& S, uint32_t loff, uint32_t base, uint32_t nlev, uint32_t tid,
                           uint32_t nthreads, uint32_t* tmp, uint32_t* list, uint32_t* off, Emit emit, Sync sync,
                           uint32_t* scnt = nullptr, uint32_t scap = 0) {
    uint32_t* cnt = (scnt && nlev < scap) ? scnt : S.lvl_count + loff;
    for (uint32_t l = tid; l <= nlev; l += nthreads) cnt[l] = 0;
    sync();
    emit([&](uint32_t lvl, uint32_t) { atomicAdd(&cnt[lvl - 1], 1u); });
    sync();
    // exclusive scan of cnt[0..nlev) in chunks owned by each thread
    const uint32_t chunk = (nlev + nthreads - 1) / nthreads;
    const uint32_t lo = min(nlev, tid * chunk), hi = min(nlev, lo + chunk);
    uint32_t part = 0;
    for (uint32_t l = lo; l < hi; ++l) part += cnt[l];
    uint32_t total;
    uint32_t run = group_scan(part, tid, nthreads, tmp, &total, sync);
    for (uint32_t l = lo; l < hi; ++l) {
        const uint32_t c = cnt[l];
        off[loff + l] = run;
        cnt[l] = run;
        run += c;
    }
    if (tid == 0) off[loff + nlev] = total;
    sync();
    emit([&](uint32_t lvl, uint32_t row) { list[base + atomicAdd(&cnt[lvl - 1], 1u)] = row; });
    sync();
}

// ---------------------------------------------------------------------------------------------
// Warp first-fit over a shared-memory table of the open batches (CTA islands).
//
// Only batches with fewer than 4 points can take a point, so the table holds just those ("slots",
// in batch order) with the island-local codes of their non-hub bodies (at most 6, 16 bits each),
// plus, per hub, the list of open batches that do not hold that hub.  A point without a hub scans
// the slots from the first open one; a point with a hub scans that hub's list.  Each step tests
// 32 consecutive candidates with one ballot, and the first candidate without a shared body is the
// reference's first fit; if none is left the point opens a new batch.  Full batches are dropped by
// compacting the table when it fills.  If the open batches alone outgrow it (or the island has too
// many bodies for 16-bit codes), the caller falls back to the one-lane skip-structure version.
//
// Body codes: a dynamic body's local index; any other non-hub body (a static or kinematic body
// that is not one of the island's two hubs) gets nloc + its index in a 256-entry hash table.
constexpr uint32_t kFfSlots = 8192;
constexpr uint32_t kFfCodes = 256;
constexpr uint32_t kFfBytes = kFfSlots * (12 + 4 + 2 + 2 + 2 + 1) + kFfCodes * 4;
constexpr uint32_t kFfH0 = 8u, kFfH1 = 16u;
constexpr uint32_t kFfDead = 0xFFFFu;
constexpr uint32_t kFfMaxLocal = 0xFFFFu - kFfCodes - 1u;

struct FfTable {
    uint32_t *bod0, *bod1, *bod2;  // per slot: up to 6 body codes, two per word (ff_shift_codes)
    uint32_t* bid;                 // per slot: batch index
    uint16_t *list0, *list1;       // per hub: slots of the open batches without that hub, batch order
    uint16_t* remap;               // compaction: old slot -> new slot
    uint8_t* cnt;                  // per slot: points (bits 0-2) | kFfH0 | kFfH1
    uint32_t* keys;                // code table: body index per entry (kNone = empty)
};

__device__ __forceinline__ FfTable ff_table_of(void* smem_v) {
    uint8_t* smem = static_cast<uint8_t*>(smem_v);
    FfTable T;
    T.bod0 = reinterpret_cast<uint32_t*>(smem);
    T.bod1 = reinterpret_cast<uint32_t*>(smem + 4u * kFfSlots);
    T.bod2 = reinterpret_cast<uint32_t*>(smem + 8u * kFfSlots);
    T.bid = reinterpret_cast<uint32_t*>(smem + 12u * kFfSlots);
    T.list0 = reinterpret_cast<uint16_t*>(smem + 16u * kFfSlots);
    T.list1 = reinterpret_cast<uint16_t*>(smem + 18u * kFfSlots);
    T.remap = reinterpret_cast<uint16_t*>(smem + 20u * kFfSlots);
    T.cnt = smem + 22u * kFfSlots;
    T.keys = reinterpret_cast<uint32_t*>(smem + 23u * kFfSlots);
    return T;
}

__device__ __forceinline__ uint32_t ff_hash(uint32_t x) { return (x * 0x9E3779B1u) >> 24; }

// Insert a body into the code table; false when the table is full.
__device__ __forceinline__ bool ff_insert(const FfTable& T, uint32_t x) {
    uint32_t h = ff_hash(x);
    for (uint32_t probe = 0; probe < kFfCodes; ++probe, h = (h + 1) & (kFfCodes - 1)) {
        const uint32_t prev = atomicCAS(&T.keys[h], kNone, x);
        if (prev == kNone || prev == x) return true;
    }
    return false;
}

__device__ __forceinline__ uint32_t ff_code(const FfTable& T, uint32_t x, uint32_t loc, uint32_t nloc) {
    if (loc != kNone) return loc;
    uint32_t h = ff_hash(x);
    for (uint32_t probe = 0; probe < kFfCodes; ++probe, h = (h + 1) & (kFfCodes - 1))
        if (T.keys[h] == x) return nloc + h;
    return kFfDead;  // not reached: every non-hub body of a batched constraint was inserted
}

__device__ __forceinline__ bool ff_holds(uint32_t w, uint32_t x) { return (w & 0xFFFFu) == x || (w >> 16) == x; }

// Drop full batches from the slots and the hub lists (whole warp).
__device__ void ff_compact(const FfTable& T, uint32_t& ns, uint32_t& nl0, uint32_t& nl1, uint32_t lane) {
    const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
    uint32_t out = 0;
    for (uint32_t base = 0; base < ns; base += 32) {
        const uint32_t i = base + lane;
        bool live = false;
        uint32_t bid = 0, cn = 0, w0 = 0, w1 = 0, w2 = 0;
        if (i < ns) {
            cn = T.cnt[i];
            live = (cn & 7u) < 4u;
            bid = T.bid[i];
            w0 = T.bod0[i];
            w1 = T.bod1[i];
            w2 = T.bod2[i];
        }
        const unsigned m = __ballot_sync(full, live);
        const uint32_t idx = out + __popc(m & lt);
        __syncwarp();
        if (i < ns) T.remap[i] = live ? (uint16_t)idx : (uint16_t)kFfDead;
        if (live) {
            T.cnt[idx] = (uint8_t)cn;
            T.bid[idx] = bid;
            T.bod0[idx] = w0;
            T.bod1[idx] = w1;
            T.bod2[idx] = w2;
        }
        out += __popc(m);
        __syncwarp();
    }
    ns = out;
    for (int f = 0; f < 2; ++f) {
        uint16_t* L = f ? T.list1 : T.list0;
        const uint32_t flag = f ? kFfH1 : kFfH0;
        const uint32_t n = f ? nl1 : nl0;
        uint32_t o = 0;
        for (uint32_t base = 0; base < n; base += 32) {
            const uint32_t i = base + lane;
            uint32_t s2 = kFfDead;
            bool live = false;
            if (i < n) {
                s2 = T.remap[L[i]];
                live = s2 != kFfDead && !(T.cnt[s2] & flag);
            }
            const unsigned m = __ballot_sync(full, live);
            const uint32_t idx = o + __popc(m & lt);
            __syncwarp();
            if (live) L[idx] = (uint16_t)s2;
            o += __popc(m);
            __syncwarp();
        }
        if (f) nl1 = o; else nl0 = o;
    }
    __syncwarp();
}

// A slot's body codes form a 96-bit shift register over its three code words (newest in the low
// half of word 0, empty halves 0xFFFF): a point adds its non-hub codes by shifting them in.  At most
// six codes are ever added (three points of two bodies; a batch's fourth point fills it and its
// codes are never read again), so nothing valid is shifted out.
__device__ __forceinline__ void ff_shift_codes(uint32_t& w0, uint32_t& w1, uint32_t& w2, uint32_t x0, uint32_t x1,
                                               bool hub) {
    if (hub) {
        w2 = __funnelshift_l(w1, w2, 16);
        w1 = __funnelshift_l(w0, w1, 16);
        w0 = (w0 << 16) | x0;
    } else {
        w2 = w1;
        w1 = w0;
        w0 = x0 | (x1 << 16);
    }
}

// First-fit batches of one island's points (whole warp).  Returns the number of batches, or kNone
// when the open batches do not fit the table.
//
// All points of a constraint share its two bodies, so point p's first fit (searched after point
// p-1's batch, PhysicsWorld.cpp:688-706) is the p-th open candidate, in batch order, that holds
// neither body: one scan serves the whole constraint, and the points are placed by the lanes that
// found their candidates.  Constraint fields are fetched two 32-constraint windows ahead.
__device__ uint32_t first_fit_warp(const SchedBufs& S, uint32_t s0, uint32_t s1, uint32_t rb, uint32_t hub0,
                                   uint32_t hub1, uint32_t nloc, uint8_t* smem, uint32_t lane,
                                   volatile uint32_t* pub = nullptr) {
    const unsigned full = 0xffffffffu, lt = (1u << lane) - 1u;
    const FfTable T = ff_table_of(smem);
    uint32_t ns = 0, nbt = 0, nl0 = 0, nl1 = 0, head = 0, head0 = 0, head1 = 0;
    // The slots head .. head + 31, held in registers (one per lane) while constraints are placed
    // into them; lanes past the table's last slot stand for the batches that would be opened next
    // (in batch order, after every existing one).  Written back - opened batches appended to the
    // table and to the hub lists - before any other access to the table.
    bool win = false, wdirty = false;
    uint32_t wcnt = 4u, ww0 = 0, ww1 = 0, ww2 = 0, wbid = 0, wns = 0;
    auto win_flush = [&]() {
        if (win && wdirty) {
            const uint32_t i = head + lane;
            const bool made = i >= wns && i < ns;  // opened while the window was held
            if (i < ns) {
                T.cnt[i] = (uint8_t)wcnt;
                T.bod0[i] = ww0;
                T.bod1[i] = ww1;
                T.bod2[i] = ww2;
                if (made) T.bid[i] = wbid;
            }
            const unsigned m0 = __ballot_sync(full, made && !(wcnt & kFfH0));
            const unsigned m1 = __ballot_sync(full, made && !(wcnt & kFfH1));
            if ((m0 >> lane) & 1u) T.list0[nl0 + __popc(m0 & lt)] = (uint16_t)i;
            if ((m1 >> lane) & 1u) T.list1[nl1 + __popc(m1 & lt)] = (uint16_t)i;
            nl0 += __popc(m0);
            nl1 += __popc(m1);
        }
        win = false;
        wdirty = false;
        __syncwarp();
    };
    // this lane's slot takes a point of (x0, x1) (x1 == x0 for a hub constraint, hflag its hub)
    auto win_fits = [&](uint32_t x0, uint32_t x1, uint32_t hflag) -> bool {
        const uint32_t p0 = x0 | (x0 << 16), p1 = x1 | (x1 << 16);  // SIMD 16-bit compares
        const uint32_t hit = (__vcmpeq2(ww0, p0) | __vcmpeq2(ww1, p0) | __vcmpeq2(ww2, p0)) |
                             (__vcmpeq2(ww0, p1) | __vcmpeq2(ww1, p1) | __vcmpeq2(ww2, p1));
        return (wcnt & 7u) < 4u && !(wcnt & hflag) && hit == 0u;
    };
    // win_place on the lanes with `sel`, written without divergent branches: every lane computes the
    // new slot state and keeps it only if selected (`opens`: the slot is a batch opened now, `bid`).
    auto win_place_if = [&](bool sel, uint32_t x0, uint32_t x1, uint32_t hflag, uint32_t row, bool opens, uint32_t bid) {
        const uint32_t kk = wcnt & 7u;
        uint32_t n0 = ww0, n1 = ww1, n2 = ww2;
        ff_shift_codes(n0, n1, n2, x0, x1, hflag != 0u);
        const bool sh = sel && kk + 1 < 4u;  // a full batch's codes are never read again
        ww0 = sh ? n0 : ww0;
        ww1 = sh ? n1 : ww1;
        ww2 = sh ? n2 : ww2;
        wbid = (sel && opens) ? bid : wbid;
        wcnt = sel ? ((kk + 1) | (wcnt & (kFfH0 | kFfH1)) | hflag) : wcnt;
        if (sel) {
            uint32_t* r = rec(S, rb + wbid);
            r[12 + kk] = row;
            r[3] = kk + 1;
        }
    };
    auto win_load = [&]() {  // skip the full prefix for good, then hold the next 32 slots
        for (;;) {
            const uint32_t i = head + lane;
            wcnt = i < kFfSlots ? 0u : 4u;  // past the last slot: a batch to open (none past the table)
            ww0 = 0xFFFFFFFFu;
            ww1 = 0xFFFFFFFFu;
            ww2 = 0xFFFFFFFFu;
            bool live = true;
            if (i < ns) {
                wcnt = T.cnt[i];
                ww0 = T.bod0[i];
                ww1 = T.bod1[i];
                ww2 = T.bod2[i];
                wbid = T.bid[i];
                live = (wcnt & 7u) < 4u;
            }
            const unsigned livem = __ballot_sync(full, live);
            if (livem & 1u) break;
            head += livem ? (uint32_t)(__ffs(livem) - 1) : 32u;
        }
        wns = ns;
        win = true;
        wdirty = false;
        if (pub) {  // every batch before the first open one is full, its records written
            const uint32_t fb = __shfl_sync(full, head < ns ? wbid : nbt, 0);
            __syncwarp();
            __threadfence_block();
            if (lane == 0) *pub = fb;
        }
    };
    // The plane's leading contacts (canonical pair order lists a plane's pairs first): every point
    // holds hub0, so each opens its own batch, the way the slow path below would open it - placed
    // here 32 constraints at a time.
    uint32_t sp = s0;  // the first constraint of the main loop
    while (hub0 != kNone && sp < s1) {
        const uint32_t t = sp + lane;
        uint32_t c = 0, bits = 1u, a = 0, b = 0, np = 0, la = kNone, lb = kNone;
        if (t < s1) {
            c = S.isl_con[t]; bits = S.con_bits[c]; a = S.con_a[c]; b = S.con_b[c]; np = S.con_np[c];
            la = S.con_la[c]; lb = S.con_lb[c];
        }
        const bool live = t < s1 && !(bits & 1u);
        const bool plane = live && (a == hub0 || b == hub0);
        const unsigned stopm = __ballot_sync(full, t < s1 && live && !plane);
        const uint32_t e = stopm ? (uint32_t)(__ffs(stopm) - 1) : min(32u, s1 - sp);
        const uint32_t mine = (plane && lane < e) ? np : 0u;
        uint32_t x = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(full, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        const uint32_t total = __shfl_sync(full, x, 31);
        if (ns + total > kFfSlots - 1024u) return kNone;
        const uint32_t off = x - mine;
        const uint32_t code = mine ? ff_code(T, a == hub0 ? b : a, a == hub0 ? lb : la, nloc) : 0u;
        for (uint32_t p = 0; p < mine; ++p) {
            const uint32_t sl = ns + off + p, j = nbt + off + p;
            T.bid[sl] = j;
            T.bod0[sl] = code | 0xFFFF0000u;
            T.bod1[sl] = 0xFFFFFFFFu;
            T.bod2[sl] = 0xFFFFFFFFu;
            T.cnt[sl] = (uint8_t)(1u | kFfH0);
            uint32_t* r = rec(S, rb + j);
            r[3] = 1;
            r[12] = 4u * c + p;
            T.list1[nl1 + off + p] = (uint16_t)sl;
        }
        ns += total;
        nbt += total;
        nl1 += total;
        sp += e;
        if (stopm) break;
    }
    __syncwarp();
    // pipeline: id of the constraint two windows ahead, fields of the next window
    auto load_id = [&](uint32_t w0) -> uint32_t { return w0 + lane < s1 ? S.isl_con[w0 + lane] : kNone; };
    uint32_t nx_c = load_id(sp), nx_bits = 1u, nx_a = 0, nx_b = 0, nx_np = 0, nx_la = kNone, nx_lb = kNone;
    if (nx_c != kNone) {
        nx_bits = S.con_bits[nx_c]; nx_a = S.con_a[nx_c]; nx_b = S.con_b[nx_c]; nx_np = S.con_np[nx_c];
        nx_la = S.con_la[nx_c]; nx_lb = S.con_lb[nx_c];
    }
    uint32_t id2 = load_id(sp + 32);
    for (uint32_t w0 = sp; w0 < s1; w0 += 32) {
        const uint32_t mc = nx_c, mbits = nx_bits, ma = nx_a, mb = nx_b, mnp = nx_np, mla = nx_la, mlb = nx_lb;
        nx_c = id2;  // fields of the next window start loading now
        nx_bits = 1u; nx_np = 0; nx_la = kNone; nx_lb = kNone;
        if (nx_c != kNone) {
            nx_bits = S.con_bits[nx_c]; nx_a = S.con_a[nx_c]; nx_b = S.con_b[nx_c]; nx_np = S.con_np[nx_c];
            nx_la = S.con_la[nx_c]; nx_lb = S.con_lb[nx_c];
        }
        id2 = load_id(w0 + 64);
        // decode this lane's constraint: body codes and hub
        uint32_t dx = 0, meta = 0;  // meta: np | hub + 1 << 4 | sensor << 6
        if (mc != kNone) {
            const int ha = ma == hub0 ? 0 : (ma == hub1 ? 1 : -1);
            const int hb = mb == hub0 ? 0 : (mb == hub1 ? 1 : -1);
            const int hub = ha >= 0 ? ha : hb;
            const bool sensor = (mbits & 1u) != 0u;
            uint32_t x0 = kFfDead, x1 = kFfDead;
            if (!sensor) {
                const uint32_t ca = ha >= 0 ? kFfDead : ff_code(T, ma, mla, nloc);
                const uint32_t cb = hb >= 0 ? kFfDead : ff_code(T, mb, mlb, nloc);
                x0 = hub < 0 ? ca : (ha >= 0 ? cb : ca);
                x1 = hub < 0 ? cb : x0;
            }
            dx = x0 | (x1 << 16);
            meta = mnp | ((uint32_t)(hub + 1) << 4) | (sensor ? 64u : 0u);
        } else {
            meta = 64u;
        }
        const uint32_t m = min(32u, s1 - w0);
        // Constraint fields of window positions k and k + 1 are carried from step to step; those of
        // k + 2 and k + 3 are shuffled in at the start of each step, off the dependent chain of the
        // placements, and become the next step's.
        uint32_t fa_md = __shfl_sync(full, meta, 0), fa_c = __shfl_sync(full, mc, 0), fa_x = __shfl_sync(full, dx, 0);
        const uint32_t k1 = min(1u, m - 1u);
        uint32_t fb_md = __shfl_sync(full, meta, k1), fb_c = __shfl_sync(full, mc, k1), fb_x = __shfl_sync(full, dx, k1);
        for (uint32_t k = 0; k < m; ++k) {
            const uint32_t k2 = min(k + 2u, m - 1u), k3 = min(k + 3u, m - 1u);
            const uint32_t fc_md = __shfl_sync(full, meta, k2), fc_c = __shfl_sync(full, mc, k2),
                           fc_x = __shfl_sync(full, dx, k2);
            const uint32_t fd_md = __shfl_sync(full, meta, k3), fd_c = __shfl_sync(full, mc, k3),
                           fd_x = __shfl_sync(full, dx, k3);
            bool two = false;  // this step placed positions k and k + 1
            do {
            const uint32_t md = fa_md;
            if (md & 64u) break;  // sensors are never batched (:690)
            const uint32_t c = fa_c, xx = fa_x;
            const uint32_t np = md & 15u, x0 = xx & 0xFFFFu, x1 = xx >> 16;
            const int hub = (int)((md >> 4) & 3u) - 1;
            const uint32_t hflag = hub == 0 ? kFfH0 : (hub == 1 ? kFfH1 : 0u);
            // the next constraint's fields, fetched up front so that its fits overlap this one's
            const uint32_t mdB = fb_md;
            const uint32_t cB = fb_c, xxB = fb_x;
            const bool canB = k + 1 < m && !(mdB & 64u);
            const uint32_t npB = mdB & 15u, x0B = xxB & 0xFFFFu, x1B = xxB >> 16;
            const uint32_t hB = (mdB >> 4) & 3u;
            const uint32_t hfB = hB == 1u ? kFfH0 : (hB == 2u ? kFfH1 : 0u);
            // ---- fast path: the first np lanes of the held window that take a point (sliding the
            // window once past its full batches if it has to)
            bool done = false;
            for (int attempt = 0; attempt < 2; ++attempt) {
                if (!win) win_load();
                const bool ok = win_fits(x0, x1, hflag);
                const bool okBl = win_fits(x0B, x1B, hfB);  // on the state before this constraint
                const unsigned okm = __ballot_sync(full, ok);
                const unsigned okBraw = __ballot_sync(full, okBl);
                if ((uint32_t)__popc(okm) >= np) {
                    const uint32_t rank = __popc(okm & lt);
                    const bool sel = ok && rank < np;
                    const uint32_t vfirst = ns - head;  // first lane that opens a batch
                    const unsigned newm = __ballot_sync(full, sel && lane >= vfirst);
                    const uint32_t nnew = __popc(newm);
                    // The next constraint rides along when the window serves it too: its fits are taken
                    // on the same window state, minus the lanes this one fills up and, if they share a
                    // body or a hub, the lanes this one takes.
                    bool pair = false;
                    unsigned okB = 0;
                    if (canB) {
                        const bool share = x0 == x0B || x0 == x1B || x1 == x0B || x1 == x1B || (hfB & hflag);
                        const unsigned selm = __ballot_sync(full, sel);
                        const unsigned fullm = __ballot_sync(full, sel && (wcnt & 7u) + 1u == 4u);
                        okB = okBraw & ~fullm & (share ? ~selm : ~0u);
                        pair = (uint32_t)__popc(okB) >= npB;
                    }
                    win_place_if(sel, x0, x1, hflag, 4u * c + rank, lane >= vfirst, nbt + (lane - vfirst));
                    ns += nnew;
                    nbt += nnew;
                    if (pair) {
                        const uint32_t rankB = __popc(okB & lt);
                        const bool selB = ((okB >> lane) & 1u) && rankB < npB;
                        const uint32_t vB = ns - head;
                        const unsigned newB = __ballot_sync(full, selB && lane >= vB);
                        win_place_if(selB, x0B, x1B, hfB, 4u * cB + rankB, lane >= vB, nbt + (lane - vB));
                        ns += __popc(newB);
                        nbt += __popc(newB);
                        ++k;
                        two = true;
                    }
                    wdirty = true;
                    done = true;
                    break;
                }
                if (attempt == 0 && (__shfl_sync(full, wcnt, 0) & 7u) >= 4u) {
                    win_flush();  // full batches at the front: slide and try again
                    continue;
                }
                break;
            }
            if (done) break;
            win_flush();  // the table is read and written directly below
            const uint16_t* L = hub == 0 ? T.list0 : T.list1;
            const uint32_t nL = hub < 0 ? ns : (hub == 0 ? nl0 : nl1);
            uint32_t pos = hub < 0 ? head : (hub == 0 ? head0 : head1);
            uint32_t placed = 0;
            // ---- scan: the first np open candidates holding neither body take the points
            while (placed < np && pos < nL) {
                const uint32_t i = pos + lane;
                bool live = false, ok = false;
                uint32_t s = 0, cn = 0;
                if (i < nL) {
                    s = hub < 0 ? i : L[i];
                    cn = T.cnt[s];
                    live = (cn & 7u) < 4u && !(cn & hflag);
                    if (live) {
                        const uint32_t w0c = T.bod0[s], w1c = T.bod1[s], w2c = T.bod2[s];
                        ok = !(ff_holds(w0c, x0) || ff_holds(w1c, x0) || ff_holds(w2c, x0) ||
                               ff_holds(w0c, x1) || ff_holds(w1c, x1) || ff_holds(w2c, x1));
                    }
                }
                const unsigned livem = __ballot_sync(full, live);
                const unsigned okm = __ballot_sync(full, ok);
                const uint32_t hd = hub < 0 ? head : (hub == 0 ? head0 : head1);
                if (pos == hd) {  // skip a dead prefix for good
                    const uint32_t adv = livem ? (uint32_t)(__ffs(livem) - 1) : (pos + 32 <= nL ? 32u : 0u);
                    if (hub < 0) head += adv; else if (hub == 0) head0 += adv; else head1 += adv;
                }
                const uint32_t take = min((uint32_t)__popc(okm), np - placed);
                if (ok) {
                    const uint32_t rank = __popc(okm & lt);
                    if (rank < take) {  // place point placed + rank into this candidate
                        const uint32_t kk = cn & 7u;
                        if (kk + 1 < 4u) {  // a full batch's codes are never read again
                            uint32_t c0 = T.bod0[s], c1 = T.bod1[s], c2 = T.bod2[s];
                            ff_shift_codes(c0, c1, c2, x0, x1, hub >= 0);
                            T.bod0[s] = c0;
                            T.bod1[s] = c1;
                            T.bod2[s] = c2;
                        }
                        T.cnt[s] = (uint8_t)((kk + 1) | (cn & (kFfH0 | kFfH1)) | hflag);
                        uint32_t* r = rec(S, rb + T.bid[s]);
                        r[12 + kk] = 4u * c + placed + rank;
                        r[3] = kk + 1;
                    }
                }
                placed += take;
                pos += 32;
            }
            // ---- the remaining points open new batches
            const uint32_t rem = np - placed;
            if (rem) {
                if (ns + rem > kFfSlots) {
                    ff_compact(T, ns, nl0, nl1, lane);
                    head = 0;
                    head0 = 0;
                    head1 = 0;
                    if (ns + rem > kFfSlots - 1024u) return kNone;
                }
                if (lane < rem) {
                    const uint32_t sl = ns + lane, j = nbt + lane;
                    T.bid[sl] = j;
                    T.bod0[sl] = hub < 0 ? (x0 | (x1 << 16)) : (x0 | 0xFFFF0000u);
                    T.bod1[sl] = 0xFFFFFFFFu;
                    T.bod2[sl] = 0xFFFFFFFFu;
                    T.cnt[sl] = (uint8_t)(1u | hflag);
                    uint32_t* r = rec(S, rb + j);
                    r[3] = 1;
                    r[12] = 4u * c + placed + lane;
                    if (hub != 0) T.list0[nl0 + lane] = (uint16_t)sl;
                    if (hub != 1) T.list1[nl1 + lane] = (uint16_t)sl;
                }
                ns += rem;
                nbt += rem;
                if (hub != 0) nl0 += rem;
                if (hub != 1) nl1 += rem;
            }
            __syncwarp();
            } while (false);
            if (two) {
                fa_md = fc_md; fa_c = fc_c; fa_x = fc_x;
                fb_md = fd_md; fb_c = fd_c; fb_x = fd_x;
            } else {
                fa_md = fb_md; fa_c = fb_c; fa_x = fb_x;
                fb_md = fc_md; fb_c = fc_c; fb_x = fc_x;
            }
        }
    }
    win_flush();
    return nbt;
}

// One level sweep of an island on one warp, with the level table `last` (nloc words, any memory):
// 0 velocity (batch order, one level per point; local bodies staged per item in vl_list / bl_list),
// 1 warm start (all points) and 2 bias (points with positionBias > 0) in constraint order, the
// points of a constraint on consecutive levels.  Writes the levels and the sweep's level count.
__device__ void level_sweep(const SchedBufs& S, SchedShared* sh, uint32_t sweep, uint32_t* last, uint32_t s0,
                            uint32_t s1, uint32_t base, uint32_t lane) {
    const uint32_t nloc = sh->nloc;
    for (uint32_t k = lane; k < nloc; k += 32) last[k] = 0;
    __syncwarp();
    uint32_t top = 0;
    if (sweep == 0) {
        const uint32_t nvit = sh->total;
        uint32_t nla = kNone, nlb = kNone;  // the next window's bodies, loaded a window ahead
        if (lane < nvit) { nla = S.vl_list[base + lane]; nlb = S.bl_list[base + lane]; }
        for (uint32_t w0 = 0; w0 < nvit; w0 += 32) {
            const uint32_t i = w0 + lane, la = nla, lb = nlb;
            const bool v = i < nvit;
            nla = kNone;
            nlb = kNone;
            if (i + 32 < nvit) { nla = S.vl_list[base + i + 32]; nlb = S.bl_list[base + i + 32]; }
            const uint32_t lvl = level_window(last, v, la, lb, 1u, lane);
            if (v) { S.vlev[base + i] = lvl; top = max(top, lvl); }
        }
    } else {
        for (uint32_t w0 = s0; w0 < s1; w0 += 32) {
            const uint32_t s = w0 + lane;
            bool v = s < s1;
            uint32_t c = v ? S.isl_con[s] : 0u, len = 0;
            if (v) {
                const uint32_t np = S.con_np[c];
                if (sweep == 1) {
                    len = np;
                } else if (!(S.inv_mass[S.con_a[c]] <= 0.0f && S.inv_mass[S.con_b[c]] <= 0.0f)) {
                    for (uint32_t p = 0; p < np; ++p) len += S.bias[4u * c + p].y > 0.0f ? 1u : 0u;
                }
                v = len > 0;
            }
            const uint32_t lvl = level_window(last, v, v ? S.con_la[c] : kNone, v ? S.con_lb[c] : kNone, len, lane);
            if (s < s1) (sweep == 1 ? S.first_w : S.first_b)[s] = v ? lvl : 0u;
            if (v) top = max(top, lvl + len - 1);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(0xffffffffu, top, o));
    if (lane == 0) (sweep == 0 ? sh->nv : (sweep == 1 ? sh->nw : sh->nb)) = top;
    __syncwarp();
}

// The velocity level sweep run on its own warp behind the first fit (streamed first fit): batches
// below sh->ff_final are full and final, so their points sit at 4 * batch + slot in batch order and
// can be levelled while the first fit goes on; once it is done the rest (batches not full) follow.
// Returns false - the caller then runs the sweep itself - if the first fit gave up.  The wait is
// bounded: past S.spin_limit polls it raises KZG_DEVERR_WAIT and gives up (the caller's sweep then
// gives the same levels, so the step's result is unchanged).
__device__ bool velocity_stream(const SchedBufs& S, Counters* cnt, SchedShared* sh, uint32_t* last, uint32_t rb,
                                uint32_t base, uint32_t lane) {
    const unsigned full = 0xffffffffu;
    const uint32_t nloc = sh->nloc;
    for (uint32_t k = lane; k < nloc; k += 32) last[k] = 0;
    __syncwarp();
    volatile uint32_t* vfin = &sh->ff_final;
    volatile uint32_t* vdone = &sh->ff_done;
    uint32_t b = 0, top = 0, spins = 0;
    for (;;) {
        uint32_t fin = 0, done = 0;
        for (;;) {  // until 8 more batches are final, or the first fit is over
            if (lane == 0) {
                done = *vdone;
                fin = *vfin;
            }
            done = __shfl_sync(full, done, 0);
            fin = __shfl_sync(full, fin, 0);
            if (done || fin >= b + 8) break;
            if (++spins > S.spin_limit) {
                if (lane == 0) atomicOr(&cnt->error, KZG_DEVERR_WAIT);
                return false;
            }
            __nanosleep(128);
        }
        __threadfence_block();
        if (done == 2u) return false;
        if (fin < b + 8) break;  // done: the rest below
        const uint32_t row = rec(S, rb + b + (lane >> 2))[12 + (lane & 3u)];
        const uint32_t c = row >> 2;
        const uint32_t lvl = level_window(last, true, S.con_la[c], S.con_lb[c], 1u, lane);
        S.vitems[base + 4 * b + lane] = row;
        S.vlev[base + 4 * b + lane] = lvl;
        top = max(top, lvl);
        b += 8;
    }
    const uint32_t nbt = sh->nbt;  // the batches from b on, in batch order
    uint32_t pos = 4 * b;
    for (uint32_t j0 = b; j0 < nbt; j0 += 32) {
        const uint32_t j = j0 + lane;
        const uint32_t* r = rec(S, rb + j);
        const uint32_t cj = j < nbt ? r[3] : 0u;
        uint32_t x = cj;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(full, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        for (uint32_t k = 0; k < cj; ++k) S.vitems[base + pos + x - cj + k] = r[12 + k];
        pos += __shfl_sync(full, x, 31);
    }
    __syncwarp();
    for (uint32_t w0 = 4 * b; w0 < pos; w0 += 32) {
        const uint32_t i = w0 + lane;
        const bool v = i < pos;
        const uint32_t row = v ? S.vitems[base + i] : 0u, c = row >> 2;
        const uint32_t lvl = level_window(last, v, v ? S.con_la[c] : kNone, v ? S.con_lb[c] : kNone, 1u, lane);
        if (v) {
            S.vlev[base + i] = lvl;
            top = max(top, lvl);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(full, top, o));
    if (lane == 0) {
        sh->nv = top;
        sh->total = pos;
    }
    __syncwarp();
    return true;
}

template <typename Sync>
__device__ void schedule_island(const SchedBufs& S, Counters* cnt, uint32_t isl, uint32_t tid, uint32_t nthreads,
                                SchedShared* sh, uint32_t* tmp, uint32_t* last_sm, uint32_t last_cap, bool ff_table,
                                Sync sync) {
    const uint32_t s0 = S.isl_start[isl], s1 = S.isl_start[isl + 1];
    const uint32_t base = 4u * s0;     // point region
    const uint32_t loff = base + isl;  // level-offset region
    const uint32_t rb = base + isl;    // batch-record region (npts + 1 records)
    const uint32_t boff = 2u * s0;     // body region
    const uint32_t lane = tid & 31u, warp = tid >> 5;

    // ---- A: local indices of the island's dynamic bodies, hub candidates (large bodies)
    if (tid == 0) { sh->nloc = 0; sh->hub0 = kNone; sh->hub1 = kNone; sh->ff_ok = ff_table ? 1u : 0u; }
    const FfTable T = ff_table_of(last_sm);
    if (ff_table)
        for (uint32_t k = tid; k < kFfCodes; k += nthreads) T.keys[k] = kNone;
    sync();
    // (the constraint loops take kA constraints per thread at once so that their loads overlap)
    constexpr uint32_t kA = 4;
    const uint32_t frame = cnt->frame;
    for (uint32_t t0 = s0 + tid; t0 < s1; t0 += kA * nthreads) {
        uint32_t cc[kA], bb[kA], xa[kA], xb[kA], ea[kA], eb[kA];
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) cc[j] = t0 + j * nthreads < s1 ? S.isl_con[t0 + j * nthreads] : kNone;
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) {
            bb[j] = cc[j] != kNone ? S.con_bits[cc[j]] : 0u;
            xa[j] = cc[j] != kNone ? S.con_a[cc[j]] : 0u;
            xb[j] = cc[j] != kNone ? S.con_b[cc[j]] : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) {  // first touch of a dynamic body this frame: a local index
            ea[j] = (bb[j] & 2u) ? atomicExch(&S.body_stamp[xa[j]], frame) : frame;
            eb[j] = (bb[j] & 4u) ? atomicExch(&S.body_stamp[xb[j]], frame) : frame;
        }
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) {
            if (cc[j] == kNone) continue;
            const uint32_t xs[2] = {xa[j], xb[j]}, es[2] = {ea[j], eb[j]};
            for (int q = 0; q < 2; ++q) {
                const uint32_t x = xs[q];
                if (bb[j] & (2u << q)) {
                    if (es[q] != frame) {
                        const uint32_t l = atomicAdd(&sh->nloc, 1u);
                        S.body_loc[x] = l;
                        S.isl_bodies[boff + l] = x;
                    }
                } else if (S.is_large[x] && !(bb[j] & 1u)) {
                    atomicMin(&sh->hub0, x);
                }
            }
        }
    }
    sync();
    for (uint32_t t0 = s0 + tid; t0 < s1; t0 += kA * nthreads) {
        uint32_t cc[kA], bb[kA], xa[kA], xb[kA], la[kA], lb[kA];
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) cc[j] = t0 + j * nthreads < s1 ? S.isl_con[t0 + j * nthreads] : kNone;
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) {
            bb[j] = cc[j] != kNone ? S.con_bits[cc[j]] : 0u;
            xa[j] = cc[j] != kNone ? S.con_a[cc[j]] : 0u;
            xb[j] = cc[j] != kNone ? S.con_b[cc[j]] : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) {
            la[j] = (bb[j] & 2u) ? S.body_loc[xa[j]] : kNone;
            lb[j] = (bb[j] & 4u) ? S.body_loc[xb[j]] : kNone;
        }
#pragma unroll
        for (uint32_t j = 0; j < kA; ++j) {
            if (cc[j] == kNone) continue;
            S.con_la[cc[j]] = la[j];
            S.con_lb[cc[j]] = lb[j];
            const uint32_t xs[2] = {xa[j], xb[j]};
            for (int q = 0; q < 2; ++q)
                if (!(bb[j] & (2u << q)) && S.is_large[xs[q]] && !(bb[j] & 1u) && xs[q] != sh->hub0)
                    atomicMin(&sh->hub1, xs[q]);
        }
    }
    sync();
    if (ff_table) {  // codes of the non-dynamic, non-hub bodies of batched constraints
        const uint32_t hub0 = sh->hub0, hub1 = sh->hub1;
        bool ok = true;
        for (uint32_t s = s0 + tid; s < s1; s += nthreads) {
            const uint32_t c = S.isl_con[s], bits = S.con_bits[c];
            if (bits & 1u) continue;
            const uint32_t xs[2] = {S.con_a[c], S.con_b[c]};
            for (int q = 0; q < 2; ++q)
                if (!(bits & (2u << q)) && xs[q] != hub0 && xs[q] != hub1) ok = ok && ff_insert(T, xs[q]);
        }
        if (!ok) sh->ff_ok = 0u;
        sync();
    }

    // ---- B: first-fit batching: one warp over the shared-memory table, else one lane.  When the
    // island's level tables do not fit shared memory anyway, warps 1 and 2 meanwhile run the warm
    // and bias level sweeps, which do not depend on the batches.
    // Warp 3 then runs the velocity level sweep right behind the first fit (velocity_stream).
    const uint32_t nwarps = (nthreads + 31) >> 5;
    const bool early = nwarps >= 3 && sh->nloc > last_cap;
    const bool table_ff = !S.scalar && ff_table && sh->ff_ok && sh->nloc <= kFfMaxLocal;
    const bool stream = early && table_ff && nwarps >= 4;
    if (tid == 0) {
        sh->ff_final = 0;
        sh->ff_done = 0;
        sh->stream_ok = 0;
    }
    sync();
    if (table_ff && warp == 0) {
        const uint32_t r = first_fit_warp(S, s0, s1, rb, sh->hub0, sh->hub1, sh->nloc, reinterpret_cast<uint8_t*>(last_sm),
                                          lane, stream ? &sh->ff_final : nullptr);
        __syncwarp();
        __threadfence_block();
        if (lane == 0) {
            sh->nbt = r;
            __threadfence_block();
            *(volatile uint32_t*)&sh->ff_done = r == kNone ? 2u : 1u;
        }
    }
    if (early && (warp == 1 || warp == 2)) level_sweep(S, sh, warp, S.last_g + warp * S.last_stride + boff, s0, s1, base, lane);
    if (stream && warp == 3) {
        const bool ok = velocity_stream(S, cnt, sh, S.last_g + boff, rb, base, lane);
        if (lane == 0) sh->stream_ok = ok ? 1u : 0u;
    }
    sync();
    const bool batched = table_ff && sh->nbt != kNone;
    const bool streamed = batched && sh->stream_ok != 0u;
    sync();
    if (S.scalar && tid == 0) sh->nbt = 0;
    if (!batched && !S.scalar && tid == 0) {
        const uint32_t hub0 = sh->hub0, hub1 = sh->hub1;
        uint32_t* r0 = rec(S, rb);
        r0[0] = 0; r0[1] = 0; r0[2] = 0;
        uint32_t nbt = 0;
        for (uint32_t s = s0; s < s1; ++s) {
            const uint32_t c = S.isl_con[s];
            if (S.con_bits[c] & 1u) continue;  // sensors are never batched (:690)
            const uint32_t a = S.con_a[c], b = S.con_b[c], np = S.con_np[c];
            const int ha = a == hub0 ? 0 : (a == hub1 ? 1 : -1);
            const int hb = b == hub0 ? 0 : (b == hub1 ? 1 : -1);
            const uint32_t f = ha >= 0 ? 1u + ha : (hb >= 0 ? 1u + hb : 0u);
            const uint32_t other = ha >= 0 ? b : a;
            uint32_t from = 0;
            for (uint32_t p = 0; p < np; ++p) {
                uint32_t j = nx_find(S, rb, f, from);
                if (f != 0) {
                    while (j < nbt && rec_has(rec(S, rb + j), other)) j = nx_find(S, rb, f, j + 1);
                } else {
                    while (j < nbt) {
                        const uint32_t* r = rec(S, rb + j);
                        if (!rec_has(r, a) && !rec_has(r, b)) break;
                        j = nx_find(S, rb, 0, j + 1);
                    }
                }
                uint32_t* r = rec(S, rb + j);
                if (j == nbt) {  // open a new batch; the record past it becomes the sentinel
                    r[3] = 0;
                    ++nbt;
                    uint32_t* t = rec(S, rb + nbt);
                    t[0] = nbt; t[1] = nbt; t[2] = nbt;
                }
                const uint32_t k = r[3];
                r[4 + 2 * k] = a;
                r[5 + 2 * k] = b;
                r[12 + k] = 4u * c + p;
                r[3] = k + 1;
                if (k + 1 == 4u) { r[0] = j + 1; r[1] = j + 1; r[2] = j + 1; }
                if (ha == 0 || hb == 0) r[1] = j + 1;
                if (ha == 1 || hb == 1) r[2] = j + 1;
                from = j + 1;
            }
        }
        sh->nbt = nbt;
    }
    sync();

    // ---- C: velocity items in batch order (the streamed sweep wrote them)
    const uint32_t nbt = sh->nbt;
    if (!streamed) {
        const uint32_t chunk = (nbt + nthreads - 1) / nthreads;
        const uint32_t lo = min(nbt, tid * chunk), hi = min(nbt, lo + chunk);
        uint32_t part = 0;
        for (uint32_t j = lo; j < hi; ++j) part += rec(S, rb + j)[3];
        uint32_t total;
        uint32_t pos = group_scan(part, tid, nthreads, tmp, &total, sync);
        for (uint32_t j = lo; j < hi; ++j) {  // rows, and their local bodies for the velocity sweep
            const uint32_t* r = rec(S, rb + j);
            for (uint32_t k = 0; k < r[3]; ++k, ++pos) {
                const uint32_t row = r[12 + k];
                S.vitems[base + pos] = row;
                S.vl_list[base + pos] = S.con_la[row >> 2];
                S.bl_list[base + pos] = S.con_lb[row >> 2];
            }
        }
        if (tid == 0) sh->total = total;
    }
    sync();

    // ---- D: the level sweeps left, one warp each (or one after another on a single warp); the
    // velocity sweep alone gets all of the shared memory when the others ran during B
    const uint32_t nloc = sh->nloc;
    const uint32_t nvit = sh->total;
    for (uint32_t sweep = 0; sweep < 3; ++sweep) {
        if (early && sweep != 0) continue;
        if ((streamed || S.scalar) && sweep == 0) continue;
        const uint32_t owner = nwarps >= 3 ? sweep : 0;
        if (warp != owner) continue;
        uint32_t* last = (early ? nloc <= 3u * last_cap : nloc <= last_cap)
                             ? last_sm + (nwarps >= 3 && !early ? sweep * last_cap : 0)
                             : S.last_g + sweep * S.last_stride + boff;
        level_sweep(S, sh, sweep, last, s0, s1, base, lane);
    }
    sync();

    // ---- E: sort each sweep's points by level
    const uint32_t nw = sh->nw, nb = sh->nb, nv = S.scalar ? nw : sh->nv;
    const uint32_t scap = nthreads >= 64 ? 3u * last_cap : 0u;  // CTA: the level tables' shared memory is free now
    // The emitters walk kU items per thread at once so that their loads overlap.
    constexpr uint32_t kU = 8;
    // the warm start's points in constraint order (and, under the scalar solver, the velocity sweep's)
    auto emit_warm = [&](auto put) {
        for (uint32_t t0 = s0 + tid; t0 < s1; t0 += kU * nthreads) {
            uint32_t cc[kU], ff[kU], nn[kU];
#pragma unroll
            for (uint32_t j = 0; j < kU; ++j) {
                const uint32_t t = t0 + j * nthreads;
                cc[j] = t < s1 ? S.isl_con[t] : 0u;
                ff[j] = t < s1 ? S.first_w[t] : 0u;
            }
#pragma unroll
            for (uint32_t j = 0; j < kU; ++j) nn[j] = t0 + j * nthreads < s1 ? S.con_np[cc[j]] : 0u;
#pragma unroll
            for (uint32_t j = 0; j < kU; ++j)
                for (uint32_t p = 0; p < nn[j]; ++p) put(ff[j] + p, 4u * cc[j] + p);
        }
    };
    if (S.scalar) {
        level_sort(S, loff, base, nw, tid, nthreads, tmp, S.vl_list, S.vl_off, emit_warm, sync, last_sm, scap);
    } else {
        level_sort(S, loff, base, nv, tid, nthreads, tmp, S.vl_list, S.vl_off,
                   [&](auto put) {
                       for (uint32_t i0 = tid; i0 < nvit; i0 += kU * nthreads) {
                           uint32_t lv[kU], rw[kU];
#pragma unroll
                           for (uint32_t j = 0; j < kU; ++j) {
                               const uint32_t i = i0 + j * nthreads;
                               lv[j] = i < nvit ? S.vlev[base + i] : 0u;
                               rw[j] = i < nvit ? S.vitems[base + i] : 0u;
                           }
#pragma unroll
                           for (uint32_t j = 0; j < kU; ++j)
                               if (lv[j]) put(lv[j], rw[j]);
                       }
                   },
                   sync, last_sm, scap);
    }
    level_sort(S, loff, base, nw, tid, nthreads, tmp, S.wl_list, S.wl_off, emit_warm, sync, last_sm, scap);
    level_sort(S, loff, base, nb, tid, nthreads, tmp, S.bl_list, S.bl_off,
               [&](auto put) {
                   for (uint32_t t0 = s0 + tid; t0 < s1; t0 += kU * nthreads) {
                       uint32_t cc[kU], ff[kU], nn[kU];
#pragma unroll
                       for (uint32_t j = 0; j < kU; ++j) {
                           const uint32_t t = t0 + j * nthreads;
                           ff[j] = t < s1 ? S.first_b[t] : 0u;
                           cc[j] = ff[j] ? S.isl_con[t] : 0u;
                       }
#pragma unroll
                       for (uint32_t j = 0; j < kU; ++j) nn[j] = ff[j] ? S.con_np[cc[j]] : 0u;
                       float by[kU][4];
#pragma unroll
                       for (uint32_t j = 0; j < kU; ++j)
#pragma unroll
                           for (uint32_t p = 0; p < 4; ++p) by[j][p] = p < nn[j] ? S.bias[4u * cc[j] + p].y : 0.0f;
#pragma unroll
                       for (uint32_t j = 0; j < kU; ++j) {
                           uint32_t k = 0;
#pragma unroll
                           for (uint32_t p = 0; p < 4; ++p)
                               if (p < nn[j] && by[j][p] > 0.0f) put(ff[j] + k++, 4u * cc[j] + p);
                       }
                   }
               },
               sync, last_sm, scap);

    if (tid == 0) {
        S.meta[4 * isl + 0] = nw;
        S.meta[4 * isl + 1] = nv;
        S.meta[4 * isl + 2] = nb;
        S.meta[4 * isl + 3] = nloc;
        if (S.jflag && S.jflag[isl]) {
        } else if (nloc <= S.warp_bodies) {
            S.small_list[atomicAdd(&cnt->nsmall, 1u)] = isl;
        } else {
            S.large_list[atomicAdd(&cnt->nlarge, 1u)] = isl;
        }
        atomicAdd(&cnt->batches, nbt);
        atomicMax(&cnt->max_vlev, nv);
        atomicMax(&cnt->max_blev, nb);
    }
    sync();
}

struct SchedWarpSync {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct SchedCtaSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// Islands with at most kSchedSmallCons constraints: one warp each.
__global__ void __launch_bounds__(128, 8) k_schedule_warp(SchedBufs S, Counters* cnt) {
    __shared__ SchedShared sh[4];
    __shared__ uint32_t tmp[4][33];
    __shared__ uint32_t last[4][kSchedWarpBodies];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t n = cnt->nislands;
    for (uint32_t k = blockIdx.x * 4 + warp;; k += gridDim.x * 4) {
        if (S.order) {  // largest first: the next island from the shared counter
            uint32_t t = 0;
            if (lane == 0) t = atomicAdd(&cnt->nx_sched_w, 1u);
            k = __shfl_sync(0xffffffffu, t, 0);
        }
        if (k >= n) break;
        const uint32_t isl = S.order ? S.order[k] : k;
        if (S.isl_start[isl + 1] - S.isl_start[isl] > S.small_cons) continue;
        schedule_island(S, cnt, isl, lane, 32u, &sh[warp], tmp[warp], last[warp], kSchedWarpBodies, false,
                        SchedWarpSync{});
    }
}

// Larger islands: one CTA each.
static_assert(kFfBytes <= 3 * kSchedCtaBodies * sizeof(uint32_t), "first-fit table must fit the level tables' shared memory");
constexpr uint32_t kSchedCtaThreads = 512;  // the parallel stages (local ids, level sorts) scale with it
__global__ void __launch_bounds__(kSchedCtaThreads, 1) k_schedule_cta(SchedBufs S, Counters* cnt) {
    extern __shared__ uint32_t last_sm[];
    __shared__ SchedShared sh;
    __shared__ uint32_t tmp[33];
    __shared__ uint32_t next;
    const uint32_t n = cnt->nislands;
    for (uint32_t k = blockIdx.x;; k += gridDim.x) {
        if (S.order) {  // largest first: the next island from the shared counter
            if (threadIdx.x == 0) next = atomicAdd(&cnt->nx_sched_c, 1u);
            __syncthreads();
            k = next;
            __syncthreads();
        }
        if (k >= n) break;
        const uint32_t isl = S.order ? S.order[k] : k;
        if (S.isl_start[isl + 1] - S.isl_start[isl] <= S.small_cons) continue;
        schedule_island(S, cnt, isl, threadIdx.x, blockDim.x, &sh, tmp, last_sm, kSchedCtaBodies, true, SchedCtaSync{});
    }
}

}  // namespace kzg
