/* Oracle (test infrastructure only): the per-step world pipeline restated from the reference.
 *
 *   StepFixed order                    src/World/PhysicsWorld.cpp:245-329
 *   UpdateBroadPhase                   PhysicsWorld.cpp:334-345
 *   dynamic AABB tree + UpdatePairs    src/BroadPhase/BroadPhase.cpp:13-270,368-381,
 *                                      include/Kizuri/BroadPhase/BroadPhase.h:62-104
 *   Collide                            PhysicsWorld.cpp:350-400 (MakePairKey :13-18, SwapManifold :22-29)
 *   manifold cache                     PhysicsWorld.cpp:405-452
 *   BuildContactConstraints            PhysicsWorld.cpp:454-535
 *   IntegrateVelocities                PhysicsWorld.cpp:757-783
 *   Prepare / WarmStart / bias pass    src/Solver/ContactSolver.cpp:18-132, 257-290
 *   BuildIslands / SolveIsland         PhysicsWorld.cpp:587-743
 *   SIMD velocity batch (lane order)   src/Solver/ContactSolverSIMD.cpp:93-256
 *   IntegratePositions / pseudo / inertia  PhysicsWorld.cpp:276-290, 785-802, 854-861
 *   ComputeStateHash                   PhysicsWorld.cpp:1145-1175
 *
 * Lanes of the 4-wide SSE batch never interact, so the batch is evaluated lane by lane with
 * the same per-lane operation sequence; -ffp-contract=off keeps every a*b+c unfused.
 */
#include "kzo.h"
#include "kzo_internal.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NUL 0xFFFFFFFFu

static char g_err[256];
const char* kzo_error(void) { return g_err; }
static void set_err(const char* m) { snprintf(g_err, sizeof g_err, "%s", m); }

/* ----------------------------------------------------------------------------- */
typedef struct { aabb fat, tight; uint32_t parent, c1, c2, user, next; int32_t height; } node_t;

typedef struct {
    v3 pA, pB, rA, rB, laA, laB, n, t1, t2;
    float nm, tm1, tm2, ni, ti1, ti2, sep, rbias, pbias, bimp, fric, rest, nvel;
    uint32_t feature;
} cpc_t;

typedef struct {
    int a, b;
    uint32_t npts;
    cpc_t p[KZO_MAX_MANIFOLD];
    float friction, restitution;
    int sensor, dynA, dynB;
} con_t;

typedef struct {
    uint64_t key;
    uint32_t frame, npts;
    v3 pos[KZO_MAX_MANIFOLD];
    float ni[KZO_MAX_MANIFOLD], ti1[KZO_MAX_MANIFOLD], ti2[KZO_MAX_MANIFOLD];
} cache_t;

/* One joint (Constraints.h:41-277): its creation data, prepared state and accumulated impulses. */
typedef struct {
    uint32_t type, a, b, flags;
    v3 la, lb, lax, lbx, lpa[2], lpb[2];
    qt relrot;
    m3 crot;
    float target, lower, upper, motor_target, motor_max;
    uint32_t modes, motors;
    float six[12];
    /* prepared state and accumulated impulses */
    v3 r0, r1, axis, imp1, imp2;
    m3 m1, m2;
    float sm[2], simp[2], limit_mass, limit_imp, motor_imp, axial_mass, axial_imp, dmass, dimp;
    v3 lin_imp[3], ang_imp[3], axes[3];
} joint_t;

typedef struct { int con; uint32_t pt; } pref_t;
typedef struct { pref_t ref[4]; int a[4], b[4]; uint32_t count; } batch_t;

struct kzo_world {
    /* settings (WorldSettings / SolverSettings) */
    v3 gravity;
    float fixed_dt, baumgarte, slop, rest_thresh, max_bias, ws_factor;
    float sleep_time, sleep_lin, sleep_ang; /* WorldSettings sleep thresholds */
    uint32_t vel_iters, pos_iters;
    int vel_bias, no_ws, threads, pair_mode, sched_stats, scalar_solver;
    float res_tol;     /* > 0: velocity iterations stop once the island's residual is <= res_tol */
    uint32_t res_cap;  /* iteration cap when res_tol > 0 */
    /* shapes */
    int nshapes;
    kzo_shape* shapes;
    /* bodies (slot order) */
    int nb;
    uint32_t *packed, *layer, *mask, *proxy;
    int* shape;
    uint8_t *motion, *sensor;
    uint8_t* ccd;           /* MotionQuality::LinearCast */
    float* ccd_thr;         /* BodySettings::ccdMotionThreshold (Body.h:70) */
    aabb* fat;              /* broad-phase fat bounds per body (the tree leaves' bounds, all pair modes) */
    int use_ccd;            /* WorldSettings::useCCD (default true) */
    float ccd_max_pen;      /* WorldSettings::ccdMaxPenetration (default 0.01) */
    v3 *pos, *lv, *av, *plv, *pav, *force, *torque;
    qt* rot;
    float *inv_mass, *lin_damp, *ang_damp, *grav, *max_lin, *max_ang, *fric, *rest;
    m3 *iil, *iiw;
    int* active;            /* BodyManager::mActiveBodies: the buffer keeps values past nactive (RemoveSwap) */
    int nactive;
    int allow_sleeping;     /* WorldSettings::allowSleeping */
    uint8_t* allow_sleep;   /* BodySettings::allowSleeping */
    uint8_t* is_active;     /* ActivationState::Active */
    float* sleep_timer;     /* MotionProperties::sleepTimer */
    uint32_t st_islands;    /* WorldStats::numIslands as the step leaves it */
    uint32_t st_shared_sleepers; /* islands joined through a sleeping body in the last step (see build_islands) */
    /* broad phase tree */
    node_t* nodes;
    uint32_t nnodes, node_cap, root, free_list, nproxies;
    uint32_t *bp_layer, *bp_mask;
    uint32_t bp_layer_cap;
    /* manifold cache */
    cache_t* cache;
    uint32_t cache_cap, cache_count, frame;
    int cache_mix;  /* 1: mixed slot function (same results, no clustering) */
    /* per step */
    uint32_t* pairs; /* packed A, packed B */
    uint32_t npairs, pairs_cap;
    uint32_t* ext_pairs;
    uint32_t next_pairs;
    kzo_manifold* man;
    uint64_t* keys;
    uint32_t man_cap;
    con_t* cons;
    uint32_t ncons, cons_cap;
    /* islands */
    uint32_t nislands;
    uint32_t* isl_off; /* nislands+1 */
    uint32_t* isl_con;
    uint32_t* island_index; /* Body::mIslandIndex: kept while a body sleeps (stale) */
    /* joints (PhysicsWorld::mConstraints) and their islands */
    joint_t* joints;
    uint32_t njoints;
    uint32_t *isl_joff, *isl_joint; /* nislands+1 offsets, joint indices in joint order */
    int trig_mode;                  /* kzo_set_trig_mode */
    /* stats */
    uint32_t st_points, st_batches, st_max_vl, st_max_bl, st_max_isl_pts, st_sum_vl, st_max_open;
    uint32_t st_max_iters, st_pt_iters;
    float st_final_res;
};

/* ----------------------------------------------------------------------------- */
/* Utilities                                                                     */
/* ----------------------------------------------------------------------------- */
static void* xrealloc(void* p, size_t n) {
    void* q = realloc(p, n ? n : 1);
    if (!q) { fprintf(stderr, "kzo: out of memory\n"); abort(); }
    return q;
}

static int body_of(const kzo_world* w, uint32_t packed) {
    uint32_t slot = packed & 0x00FFFFFFu;
    if (slot >= (uint32_t)w->nb || w->packed[slot] != packed) return -1;
    return (int)slot;
}

static uint64_t pair_key(uint32_t pa, uint32_t pb) {
    if (pa > pb) { uint32_t t = pa; pa = pb; pb = t; }
    return ((uint64_t)pa << 32) | (uint64_t)pb;
}

/* ----------------------------------------------------------------------------- */
/* Dynamic AABB tree (BroadPhase.cpp)                                             */
/* ----------------------------------------------------------------------------- */
static node_t node_default(void) {
    node_t n;
    n.fat = aabb_empty();
    n.tight = aabb_empty();
    n.parent = n.c1 = n.c2 = NUL;
    n.user = 0;
    n.next = NUL;
    n.height = -1;
    return n;
}
static int is_leaf(const kzo_world* w, uint32_t i) { return w->nodes[i].c1 == NUL; }

static uint32_t alloc_node(kzo_world* w) {
    if (w->free_list != NUL) {
        uint32_t id = w->free_list;
        w->free_list = w->nodes[id].next;
        w->nodes[id] = node_default();
        w->nodes[id].next = NUL;
        return id;
    }
    if (w->nnodes == w->node_cap) {
        w->node_cap = w->node_cap ? w->node_cap * 2 : 1024;
        w->nodes = (node_t*)xrealloc(w->nodes, sizeof(node_t) * w->node_cap);
    }
    w->nodes[w->nnodes] = node_default();
    return w->nnodes++;
}
static void free_node(kzo_world* w, uint32_t id) {
    w->nodes[id] = node_default();
    w->nodes[id].next = w->free_list;
    w->nodes[id].height = -1;
    w->free_list = id;
}

static int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

static uint32_t balance(kzo_world* w, uint32_t iA) {
    node_t* N = w->nodes;
    node_t* A = &N[iA];
    if (A->c1 == NUL || A->height < 2) return iA;
    uint32_t iB = A->c1, iC = A->c2;
    node_t *B = &N[iB], *C = &N[iC];
    int32_t bal = C->height - B->height;
    if (bal > 1) {
        uint32_t iF = C->c1, iG = C->c2;
        node_t *F = &N[iF], *G = &N[iG];
        C->c1 = iA;
        C->parent = A->parent;
        A->parent = iC;
        if (C->parent != NUL) {
            if (N[C->parent].c1 == iA) N[C->parent].c1 = iC;
            else N[C->parent].c2 = iC;
        } else {
            w->root = iC;
        }
        if (F->height > G->height) {
            C->c2 = iF; A->c2 = iG; G->parent = iA;
            A->fat = aabb_merge(B->fat, G->fat);
            C->fat = aabb_merge(A->fat, F->fat);
            A->height = 1 + imax(B->height, G->height);
            C->height = 1 + imax(A->height, F->height);
        } else {
            C->c2 = iG; A->c2 = iF; F->parent = iA;
            A->fat = aabb_merge(B->fat, F->fat);
            C->fat = aabb_merge(A->fat, G->fat);
            A->height = 1 + imax(B->height, F->height);
            C->height = 1 + imax(A->height, G->height);
        }
        return iC;
    }
    if (bal < -1) {
        uint32_t iD = B->c1, iE = B->c2;
        node_t *D = &N[iD], *E = &N[iE];
        B->c1 = iA;
        B->parent = A->parent;
        A->parent = iB;
        if (B->parent != NUL) {
            if (N[B->parent].c1 == iA) N[B->parent].c1 = iB;
            else N[B->parent].c2 = iB;
        } else {
            w->root = iB;
        }
        if (D->height > E->height) {
            B->c2 = iD; A->c1 = iE; E->parent = iA;
            A->fat = aabb_merge(C->fat, E->fat);
            B->fat = aabb_merge(A->fat, D->fat);
            A->height = 1 + imax(C->height, E->height);
            B->height = 1 + imax(A->height, D->height);
        } else {
            B->c2 = iE; A->c1 = iD; D->parent = iA;
            A->fat = aabb_merge(C->fat, D->fat);
            B->fat = aabb_merge(A->fat, E->fat);
            A->height = 1 + imax(C->height, D->height);
            B->height = 1 + imax(A->height, E->height);
        }
        return iB;
    }
    return iA;
}

static void insert_leaf(kzo_world* w, uint32_t leaf) {
    if (w->root == NUL) { w->root = leaf; w->nodes[leaf].parent = NUL; return; }
    aabb la = w->nodes[leaf].fat;
    uint32_t index = w->root;
    while (!is_leaf(w, index)) {
        uint32_t c1 = w->nodes[index].c1, c2 = w->nodes[index].c2;
        float area = aabb_area(w->nodes[index].fat);
        aabb comb = aabb_merge(w->nodes[index].fat, la);
        float ca = aabb_area(comb);
        float cost = 2.0f * ca;
        float inh = 2.0f * (ca - area);
        float cost1, cost2;
        {
            aabb m = aabb_merge(la, w->nodes[c1].fat);
            cost1 = is_leaf(w, c1) ? aabb_area(m) + inh : (aabb_area(m) - aabb_area(w->nodes[c1].fat)) + inh;
        }
        {
            aabb m = aabb_merge(la, w->nodes[c2].fat);
            cost2 = is_leaf(w, c2) ? aabb_area(m) + inh : (aabb_area(m) - aabb_area(w->nodes[c2].fat)) + inh;
        }
        if (cost < cost1 && cost < cost2) break;
        index = (cost1 < cost2) ? c1 : c2;
    }
    uint32_t sib = index;
    uint32_t old_parent = w->nodes[sib].parent;
    uint32_t np = alloc_node(w);
    w->nodes[np].parent = old_parent;
    w->nodes[np].fat = aabb_merge(la, w->nodes[sib].fat);
    w->nodes[np].tight = w->nodes[np].fat;
    w->nodes[np].height = w->nodes[sib].height + 1;
    w->nodes[np].user = 0;
    if (old_parent != NUL) {
        if (w->nodes[old_parent].c1 == sib) w->nodes[old_parent].c1 = np;
        else w->nodes[old_parent].c2 = np;
    } else {
        w->root = np;
    }
    w->nodes[np].c1 = sib;
    w->nodes[np].c2 = leaf;
    w->nodes[sib].parent = np;
    w->nodes[leaf].parent = np;
    index = w->nodes[leaf].parent;
    while (index != NUL) {
        index = balance(w, index);
        uint32_t c1 = w->nodes[index].c1, c2 = w->nodes[index].c2;
        w->nodes[index].height = 1 + imax(w->nodes[c1].height, w->nodes[c2].height);
        w->nodes[index].fat = aabb_merge(w->nodes[c1].fat, w->nodes[c2].fat);
        index = w->nodes[index].parent;
    }
}

static void remove_leaf(kzo_world* w, uint32_t leaf) {
    if (leaf == w->root) { w->root = NUL; return; }
    uint32_t parent = w->nodes[leaf].parent;
    uint32_t gp = w->nodes[parent].parent;
    uint32_t sib = (w->nodes[parent].c1 == leaf) ? w->nodes[parent].c2 : w->nodes[parent].c1;
    if (gp != NUL) {
        if (w->nodes[gp].c1 == parent) w->nodes[gp].c1 = sib;
        else w->nodes[gp].c2 = sib;
        w->nodes[sib].parent = gp;
        free_node(w, parent);
        uint32_t index = gp;
        while (index != NUL) {
            index = balance(w, index);
            uint32_t c1 = w->nodes[index].c1, c2 = w->nodes[index].c2;
            w->nodes[index].fat = aabb_merge(w->nodes[c1].fat, w->nodes[c2].fat);
            w->nodes[index].height = 1 + imax(w->nodes[c1].height, w->nodes[c2].height);
            index = w->nodes[index].parent;
        }
    } else {
        w->root = sib;
        w->nodes[sib].parent = NUL;
        free_node(w, parent);
    }
}

static uint32_t create_proxy(kzo_world* w, aabb b, uint32_t user, uint32_t layer, uint32_t mask) {
    uint32_t id = alloc_node(w);
    v3 margin = V(0.1f, 0.1f, 0.1f);
    w->nodes[id].fat = AB(vsub(b.mn, margin), vadd(b.mx, margin));
    w->nodes[id].tight = b;
    w->nodes[id].user = user;
    w->nodes[id].height = 0;
    w->nodes[id].c1 = w->nodes[id].c2 = NUL;
    w->nodes[id].parent = NUL;
    insert_leaf(w, id);
    ++w->nproxies;
    if (id >= w->bp_layer_cap) {
        uint32_t nc = w->bp_layer_cap ? w->bp_layer_cap : 256;
        while (nc <= id) nc *= 2;
        w->bp_layer = (uint32_t*)xrealloc(w->bp_layer, sizeof(uint32_t) * nc);
        w->bp_mask = (uint32_t*)xrealloc(w->bp_mask, sizeof(uint32_t) * nc);
        for (uint32_t i = w->bp_layer_cap; i < nc; ++i) w->bp_layer[i] = w->bp_mask[i] = 0;
        w->bp_layer_cap = nc;
    }
    w->bp_layer[id] = layer;
    w->bp_mask[id] = mask;
    return id;
}

static void move_proxy(kzo_world* w, uint32_t id, aabb b, v3 disp) {
    w->nodes[id].tight = b;
    if (aabb_contains(w->nodes[id].fat, b)) return;
    remove_leaf(w, id);
    v3 margin = V(0.1f, 0.1f, 0.1f);
    v3 d = vabs(disp);
    w->nodes[id].fat = AB(vsub(vsub(b.mn, margin), d), vadd(vadd(b.mx, margin), d));
    insert_leaf(w, id);
}

static void push_pair(kzo_world* w, uint32_t a, uint32_t b) {
    if (w->npairs == w->pairs_cap) {
        w->pairs_cap = w->pairs_cap ? w->pairs_cap * 2 : 1024;
        w->pairs = (uint32_t*)xrealloc(w->pairs, sizeof(uint32_t) * 2 * w->pairs_cap);
    }
    w->pairs[2 * w->npairs] = a;
    w->pairs[2 * w->npairs + 1] = b;
    ++w->npairs;
}

/* QueryPairs (BroadPhase.h:62-104) + UpdatePairs filter (BroadPhase.cpp:368-381). */
static void tree_pairs(kzo_world* w) {
    w->npairs = 0;
    if (w->root == NUL) return;
    uint32_t cap = 1024, sz = 0;
    uint32_t* st = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * 2 * cap);
#define PUSH(a, b)                                                            \
    do {                                                                      \
        if (sz == cap) { cap *= 2; st = (uint32_t*)xrealloc(st, sizeof(uint32_t) * 2 * cap); } \
        st[2 * sz] = (a); st[2 * sz + 1] = (b); ++sz;                         \
    } while (0)
    PUSH(w->root, w->root);
    while (sz > 0) {
        --sz;
        uint32_t n1 = st[2 * sz], n2 = st[2 * sz + 1];
        const node_t* a = &w->nodes[n1];
        if (n1 == n2) {
            if (a->c1 == NUL) continue;
            uint32_t c1 = a->c1, c2 = a->c2;
            PUSH(c1, c1);
            PUSH(c2, c2);
            PUSH(c1, c2);
            continue;
        }
        const node_t* b = &w->nodes[n2];
        if (!aabb_overlaps(a->fat, b->fat)) continue;
        int la = a->c1 == NUL, lb = b->c1 == NUL;
        if (la && lb) {
            if (n1 < n2) {
                if ((w->bp_layer[n1] & w->bp_mask[n2]) == 0) continue;
                if ((w->bp_layer[n2] & w->bp_mask[n1]) == 0) continue;
                if (!aabb_overlaps(w->nodes[n1].tight, w->nodes[n2].tight)) continue;
                push_pair(w, w->nodes[n1].user, w->nodes[n2].user);
            }
            continue;
        }
        uint32_t ac1 = a->c1, ac2 = a->c2, bc1 = b->c1, bc2 = b->c2;
        if (la || (!lb && a->height < b->height)) {
            PUSH(n1, bc1);
            PUSH(n1, bc2);
        } else {
            PUSH(ac1, n2);
            PUSH(ac2, n2);
        }
    }
#undef PUSH
    free(st);
}

/* Canonical pairs: every overlapping pair (tight AABBs, layer filter), MakePairKey order. */
typedef struct { float mnx; int i; } sweep_t;
static int cmp_sweep(const void* a, const void* b) {
    const sweep_t *x = (const sweep_t*)a, *y = (const sweep_t*)b;
    if (x->mnx < y->mnx) return -1;
    if (x->mnx > y->mnx) return 1;
    return x->i - y->i;
}
static int cmp_key(const void* a, const void* b) {
    const uint32_t *x = (const uint32_t*)a, *y = (const uint32_t*)b;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    return 0;
}
static void canonical_pairs(kzo_world* w) {
    w->npairs = 0;
    aabb* bb = (aabb*)xrealloc(NULL, sizeof(aabb) * (size_t)w->nb);
    sweep_t* sw = (sweep_t*)xrealloc(NULL, sizeof(sweep_t) * (size_t)w->nb);
    for (int i = 0; i < w->nb; ++i) {
        bb[i] = kzo_world_bounds(&w->shapes[w->shape[i]], w->rot[i], w->pos[i]);
        sw[i].mnx = bb[i].mn.x;
        sw[i].i = i;
    }
    qsort(sw, (size_t)w->nb, sizeof(sweep_t), cmp_sweep);
    for (int s = 0; s < w->nb; ++s) {
        int i = sw[s].i;
        for (int t = s + 1; t < w->nb && sw[t].mnx <= bb[i].mx.x; ++t) {
            int j = sw[t].i;
            if ((w->layer[i] & w->mask[j]) == 0 || (w->layer[j] & w->mask[i]) == 0) continue;
            if (!aabb_overlaps(bb[i], bb[j])) continue;
            uint32_t pa = w->packed[i], pb = w->packed[j];
            if (pa < pb) push_pair(w, pa, pb); else push_pair(w, pb, pa);
        }
    }
    qsort(w->pairs, w->npairs, sizeof(uint32_t) * 2, cmp_key);
    free(bb);
    free(sw);
}

/* ----------------------------------------------------------------------------- */
/* Manifold cache (PhysicsWorld.cpp:405-452)                                       */
/* ----------------------------------------------------------------------------- */
/* Home slot of a key: the reference's (pa ^ pb) & mask, or (kzo_set_cache_hash(w, 1)) a 64-bit mix.
 * Entries are found by key and never evicted, so the slot function changes no result, only the
 * probe lengths: the reference's one clusters neighbouring ids (long runs of consecutive slots)
 * and makes large worlds quadratic. */
static uint32_t cache_home(const kzo_world* w, uint64_t key, uint32_t mask) {
    if (!w->cache_mix) return (uint32_t)(key ^ (key >> 32)) & mask;
    key ^= key >> 33;
    key *= 0xff51afd7ed558ccdull;
    key ^= key >> 33;
    key *= 0xc4ceb9fe1a85ec53ull;
    key ^= key >> 33;
    return (uint32_t)key & mask;
}

static cache_t* find_cached(kzo_world* w, uint64_t key) {
    if (w->cache_cap == 0) return NULL;
    uint32_t mask = w->cache_cap - 1;
    uint32_t slot = cache_home(w, key, mask);
    for (uint32_t p = 0; p < w->cache_cap; ++p) {
        cache_t* e = &w->cache[slot];
        if (e->key == key && e->frame != 0) return e;
        if (e->frame == 0) return NULL;
        slot = (slot + 1) & mask;
    }
    return NULL;
}

static cache_t* get_or_create_cached(kzo_world* w, uint64_t key) {
    if (w->cache_count * 10u >= w->cache_cap * 7u) {
        uint32_t ncap = w->cache_cap * 2;
        cache_t* nc = (cache_t*)calloc(ncap, sizeof(cache_t));
        uint32_t mask = ncap - 1;
        for (uint32_t i = 0; i < w->cache_cap; ++i) {
            cache_t* e = &w->cache[i];
            if (e->frame == 0) continue;
            uint32_t slot = cache_home(w, e->key, mask);
            while (nc[slot].frame != 0) slot = (slot + 1) & mask;
            nc[slot] = *e;
        }
        free(w->cache);
        w->cache = nc;
        w->cache_cap = ncap;
    }
    uint32_t mask = w->cache_cap - 1;
    uint32_t slot = cache_home(w, key, mask);
    for (;;) {
        cache_t* e = &w->cache[slot];
        if (e->frame == 0) {
            memset(e, 0, sizeof *e);
            e->key = key;
            e->frame = w->frame;
            ++w->cache_count;
            return e;
        }
        if (e->key == key) { e->frame = w->frame; return e; }
        slot = (slot + 1) & mask;
    }
}

/* ----------------------------------------------------------------------------- */
/* Solver pieces (ContactSolver.cpp, ContactSolverSIMD.cpp)                         */
/* ----------------------------------------------------------------------------- */
static float effective_mass(const kzo_world* w, int a, int b, v3 rA, v3 rB, v3 dir) {
    v3 ra = vcross(rA, dir), rb = vcross(rB, dir);
    float k = w->inv_mass[a] + w->inv_mass[b];
    k += vdot(ra, mmulv(&w->iiw[a], ra));
    k += vdot(rb, mmulv(&w->iiw[b], rb));
    return k > KZO_EPS ? 1.0f / k : 0.0f;
}

static void prepare(kzo_world* w, con_t* c, float dt) {
    int A = c->a, B = c->b;
    c->dynA = w->motion[A] == KZO_DYNAMIC;
    c->dynB = w->motion[B] == KZO_DYNAMIC;
    for (uint32_t i = 0; i < c->npts; ++i) {
        cpc_t* p = &c->p[i];
        p->rA = vsub(p->pA, w->pos[A]);
        p->rB = vsub(p->pB, w->pos[B]);
        p->laA = qinv_rotate(w->rot[A], p->rA);
        p->laB = qinv_rotate(w->rot[B], p->rB);
        v3 n = vnormalized_or(p->n, V(0, 1, 0));
        p->n = n;
        v3 t1 = vperp_normalized(n);
        p->t1 = t1;
        p->t2 = vcross(n, t1);
        p->nm = effective_mass(w, A, B, p->rA, p->rB, n);
        p->tm1 = effective_mass(w, A, B, p->rA, p->rB, p->t1);
        p->tm2 = effective_mass(w, A, B, p->rA, p->rB, p->t2);
        v3 vA = vadd(w->lv[A], vcross(w->av[A], vsub(p->pA, w->pos[A])));
        v3 vB = vadd(w->lv[B], vcross(w->av[B], vsub(p->pB, w->pos[B])));
        v3 vr = vsub(vA, vB);
        p->nvel = vdot(vr, n);
        p->rbias = 0;
        if (p->nvel < -w->rest_thresh) p->rbias = -p->rest * p->nvel;
        p->pbias = 0;
        if (p->sep < -w->slop) {
            p->pbias = w->baumgarte / dt * (-p->sep - w->slop);
            p->pbias = fmin_r(p->pbias, w->max_bias);
        }
        p->bimp = 0;
        float mf = p->fric * p->ni;
        p->ti1 = fclamp_r(p->ti1, -mf, mf);
        p->ti2 = fclamp_r(p->ti2, -mf, mf);
        p->ni = fmax_r(p->ni, 0.0f);
    }
}

static void apply_pair(kzo_world* w, int a, int b, v3 rA, v3 rB, v3 imp, int dynA, int dynB) {
    if (dynA) {
        w->lv[a] = vadd(w->lv[a], vmul(imp, w->inv_mass[a]));
        w->av[a] = vadd(w->av[a], mmulv(&w->iiw[a], vcross(rA, imp)));
    }
    if (dynB) {
        w->lv[b] = vsub(w->lv[b], vmul(imp, w->inv_mass[b]));
        w->av[b] = vsub(w->av[b], mmulv(&w->iiw[b], vcross(rB, imp)));
    }
}

static void warm_start(kzo_world* w, con_t* c) {
    for (uint32_t i = 0; i < c->npts; ++i) {
        cpc_t* p = &c->p[i];
        v3 imp = vadd(vadd(vmul(p->n, p->ni), vmul(p->t1, p->ti1)), vmul(p->t2, p->ti2));
        imp = vmul(imp, w->ws_factor);
        apply_pair(w, c->a, c->b, p->rA, p->rB, imp, c->dynA, c->dynB);
    }
}

/* Fixed-point (2^-20 N s) magnitude used by the residual sums: integer sums do not depend on the
 * order of the additions, so every implementation stops after the same iteration. */
static uint64_t res_fixed(float x) { return (uint64_t)(fminf(x, 1e12f) * 1048576.0f); }

/* One lane of SolveVelocityBatchSIMD (ContactSolverSIMD.cpp:93-256).  Adds the lane's share of the
 * island residual: |dImpulse| summed over its three rows (t1, t2, n) to *sd and its accumulated
 * |impulse| (|n| + |t1|) + |t2| to *sl.  The reference has no residual (fixed iteration counts);
 * this one decides when a residual-terminated solve stops. */
static void solve_lane(kzo_world* w, con_t* c, cpc_t* p, uint64_t* sd, uint64_t* sl) {
    int A = c->a, B = c->b;
    v3 rA = qrotate(w->rot[A], p->laA);
    v3 rB = qrotate(w->rot[B], p->laB);
    v3 vA = w->lv[A], wA = w->av[A], vB = w->lv[B], wB = w->av[B];
    const float invA = w->inv_mass[A], invB = w->inv_mass[B];
    const m3* IA = &w->iiw[A];
    const m3* IB = &w->iiw[B];
    const float nb = p->rbias + (w->vel_bias ? p->pbias : 0.0f);
    float nacc = p->ni, t1acc = p->ti1, t2acc = p->ti2;
    float dsum = 0.0f;
    for (int t = 0; t < 3; ++t) {
        v3 dir = t == 0 ? p->t1 : (t == 1 ? p->t2 : p->n);
        v3 wa = vcross(wA, rA), wb = vcross(wB, rB);
        v3 rel = V((vA.x + wa.x) - (vB.x + wb.x), (vA.y + wa.y) - (vB.y + wb.y), (vA.z + wa.z) - (vB.z + wb.z));
        float vdir = vdot(rel, dir);
        float dl;
        if (t < 2) {
            float mass = t == 0 ? p->tm1 : p->tm2;
            float acc = t == 0 ? t1acc : t2acc;
            float lambda = (0.0f - mass) * vdir;
            float maxf = p->fric * nacc;
            float na = acc + lambda;
            float lo = 0.0f - maxf;
            na = na > lo ? na : lo;          /* _mm_max_ps(na, -maxFric) */
            na = na < maxf ? na : maxf;      /* _mm_min_ps(na, maxFric) */
            dl = na - acc;
            if (t == 0) t1acc = na; else t2acc = na;
        } else {
            float lambda = (0.0f - p->nm) * (vdir - nb);
            float na = nacc + lambda;
            na = na > 0.0f ? na : 0.0f;      /* _mm_max_ps(na, 0) */
            dl = na - nacc;
            nacc = na;
        }
        dsum += fabsf(dl);
        v3 imp = V(dir.x * dl, dir.y * dl, dir.z * dl);
        vA = V(vA.x + imp.x * invA, vA.y + imp.y * invA, vA.z + imp.z * invA);
        v3 cA = vcross(rA, imp);
        wA = vadd(wA, mmulv(IA, cA));
        vB = V(vB.x - imp.x * invB, vB.y - imp.y * invB, vB.z - imp.z * invB);
        v3 cB = vcross(rB, imp);
        wB = vsub(wB, mmulv(IB, cB));
    }
    if (c->dynA) { w->lv[A] = vA; w->av[A] = wA; }
    if (c->dynB) { w->lv[B] = vB; w->av[B] = wB; }
    p->ni = nacc;
    p->ti1 = t1acc;
    p->ti2 = t2acc;
    *sd += res_fixed(dsum);
    *sl += res_fixed((fabsf(nacc) + fabsf(t1acc)) + fabsf(t2acc));
}

/* SolveContactVelocity (ContactSolver.cpp:136-181): the scalar path of SolverSettings::useSIMDSolver
 * = false.  Both friction rows use the relative velocity taken before them; the normal row takes it
 * again.  Residual sums as solve_lane's. */
static void solve_point_scalar(kzo_world* w, con_t* c, cpc_t* p, uint64_t* sd, uint64_t* sl) {
    const int A = c->a, B = c->b;
    const v3 rA = qrotate(w->rot[A], p->laA);
    const v3 rB = qrotate(w->rot[B], p->laB);
    v3 vrel = vsub(vadd(w->lv[A], vcross(w->av[A], rA)), vadd(w->lv[B], vcross(w->av[B], rB)));
    float dsum = 0.0f;
    for (int t = 0; t < 2; ++t) {
        const v3 tangent = t == 0 ? p->t1 : p->t2;
        const float mass = t == 0 ? p->tm1 : p->tm2;
        float* accum = t == 0 ? &p->ti1 : &p->ti2;
        float lambda = -mass * vdot(vrel, tangent);
        const float maxf = p->fric * p->ni;
        float ni = *accum + lambda;
        ni = ni < -maxf ? -maxf : (ni > maxf ? maxf : ni); /* math::Clamp, Types.h:55 */
        lambda = ni - *accum;
        *accum = ni;
        dsum += fabsf(lambda);
        apply_pair(w, A, B, rA, rB, vmul(tangent, lambda), c->dynA, c->dynB);
    }
    vrel = vsub(vadd(w->lv[A], vcross(w->av[A], rA)), vadd(w->lv[B], vcross(w->av[B], rB)));
    float bias = p->rbias;
    if (w->vel_bias) bias += p->pbias;
    float lambda = -p->nm * (vdot(vrel, p->n) - bias);
    float ni = p->ni + lambda;
    ni = ni > 0.0f ? ni : 0.0f; /* math::Max, Types.h:54 */
    lambda = ni - p->ni;
    p->ni = ni;
    dsum += fabsf(lambda);
    apply_pair(w, A, B, rA, rB, vmul(p->n, lambda), c->dynA, c->dynB);
    *sd += res_fixed(dsum);
    *sl += res_fixed((fabsf(p->ni) + fabsf(p->ti1)) + fabsf(p->ti2));
}

/* SolveBiasConstraint, ContactSolver.cpp:257-290 */
static void solve_bias(kzo_world* w, con_t* c) {
    int A = c->a, B = c->b;
    if (w->inv_mass[A] <= 0.0f && w->inv_mass[B] <= 0.0f) return;
    for (uint32_t i = 0; i < c->npts; ++i) {
        cpc_t* p = &c->p[i];
        if (p->pbias <= 0.0f) continue;
        v3 rA = qrotate(w->rot[A], p->laA);
        v3 rB = qrotate(w->rot[B], p->laB);
        v3 vr = vsub(vadd(w->plv[A], vcross(w->pav[A], rA)), vadd(w->plv[B], vcross(w->pav[B], rB)));
        float lambda = -p->nm * (vdot(vr, p->n) - p->pbias);
        float ni = fmax_r(p->bimp + lambda, 0.0f);
        lambda = ni - p->bimp;
        p->bimp = ni;
        v3 imp = vmul(p->n, lambda);
        if (c->dynA) {
            w->plv[A] = vadd(w->plv[A], vmul(imp, w->inv_mass[A]));
            w->pav[A] = vadd(w->pav[A], mmulv(&w->iiw[A], vcross(rA, imp)));
        }
        if (c->dynB) {
            w->plv[B] = vsub(w->plv[B], vmul(imp, w->inv_mass[B]));
            w->pav[B] = vsub(w->pav[B], mmulv(&w->iiw[B], vcross(rB, imp)));
        }
    }
}

/* SolveIsland, PhysicsWorld.cpp:666-743 (SIMD path, no joints). */
/* ----------------------------------------------------------------------------- */
/* Joints (Constraints.cpp:1-597, Constraints.h:41-277)                           */
/* ----------------------------------------------------------------------------- */
static m3 m_diag(float s) {
    m3 r;
    r.c[0] = V(1.0f * s, 0.0f * s, 0.0f * s);
    r.c[1] = V(0.0f * s, 1.0f * s, 0.0f * s);
    r.c[2] = V(0.0f * s, 0.0f * s, 1.0f * s);
    return r;
}
static m3 m_skew(v3 v) { /* Mat3::Skew (Math.h:193-197) */
    m3 r;
    r.c[0] = V(0.0f, v.z, -v.y);
    r.c[1] = V(-v.z, 0.0f, v.x);
    r.c[2] = V(v.y, -v.x, 0.0f);
    return r;
}
static m3 m_add(m3 a, m3 b) { m3 r; for (int k = 0; k < 3; ++k) r.c[k] = vadd(a.c[k], b.c[k]); return r; }
static m3 m_sub(m3 a, m3 b) { m3 r; for (int k = 0; k < 3; ++k) r.c[k] = vsub(a.c[k], b.c[k]); return r; }
static m3 m_zero(void) { m3 r; r.c[0] = r.c[1] = r.c[2] = V(0, 0, 0); return r; }
static m3 m_inverse(m3 m) { /* Mat3::Inversed (Math.cpp:27-43): adjugate / determinant */
    v3 r0 = vcross(m.c[1], m.c[2]), r1 = vcross(m.c[2], m.c[0]), r2 = vcross(m.c[0], m.c[1]);
    float det = vdot(m.c[0], r0);
    float inv = det != 0.0f ? 1.0f / det : 0.0f;
    m3 o;
    o.c[0] = vmul(V(r0.x, r1.x, r2.x), inv);
    o.c[1] = vmul(V(r0.y, r1.y, r2.y), inv);
    o.c[2] = vmul(V(r0.z, r1.z, r2.z), inv);
    return o;
}
static void v_basis(v3 n, v3* b, v3* c) { /* Vec3::GetBasis (Math.cpp:9-22) */
    if (n.z < -0.9999999f) {
        *b = V(0.0f, -1.0f, 0.0f);
        *c = V(-1.0f, 0.0f, 0.0f);
    } else {
        const float a = 1.0f / (1.0f + n.z);
        const float bb = -n.x * n.y * a;
        *b = V(1.0f - n.x * n.x * a, bb, -n.x);
        *c = V(bb, 1.0f - n.y * n.y * a, -n.y);
    }
}
static qt q_conj(qt q) { return Q(-q.x, -q.y, -q.z, q.w); }


static m3 point_mass(const kzo_world* w, int a, int b, v3 ra, v3 rb) { /* Constraints.cpp:23-33 */
    m3 K = m_diag(w->inv_mass[a] + w->inv_mass[b]);
    m3 sa = m_skew(ra), sb = m_skew(rb);
    m3 t = mmul(&w->iiw[a], &sa);
    t = mmul(&sa, &t);
    K = m_sub(K, t);
    t = mmul(&w->iiw[b], &sb);
    t = mmul(&sb, &t);
    return m_sub(K, t);
}
static float angular_mass(const kzo_world* w, int a, int b, v3 axis) { /* :35-41 */
    float k = vdot(axis, mmulv(&w->iiw[a], axis)) + vdot(axis, mmulv(&w->iiw[b], axis));
    return k > KZO_EPS ? 1.0f / k : 0.0f;
}
static float linear_mass(const kzo_world* w, int a, int b, v3 ra, v3 rb, v3 axis) { /* :43-52 */
    v3 ca = vcross(ra, axis), cb = vcross(rb, axis);
    float k = w->inv_mass[a] + w->inv_mass[b];
    k += vdot(ca, mmulv(&w->iiw[a], ca));
    k += vdot(cb, mmulv(&w->iiw[b], cb));
    return k > KZO_EPS ? 1.0f / k : 0.0f;
}
static void apply_impulse(kzo_world* w, int a, int b, v3 ra, v3 rb, v3 imp) { /* :8-15 */
    w->lv[a] = vadd(w->lv[a], vmul(imp, w->inv_mass[a]));
    w->av[a] = vadd(w->av[a], mmulv(&w->iiw[a], vcross(ra, imp)));
    w->lv[b] = vsub(w->lv[b], vmul(imp, w->inv_mass[b]));
    w->av[b] = vsub(w->av[b], mmulv(&w->iiw[b], vcross(rb, imp)));
}
static void apply_angular(kzo_world* w, int a, int b, v3 ang) { /* :17-20 */
    w->av[a] = vadd(w->av[a], mmulv(&w->iiw[a], ang));
    w->av[b] = vsub(w->av[b], mmulv(&w->iiw[b], ang));
}
static float j_sin(const kzo_world* w, float x) { return w->trig_mode ? (float)sin((double)x) : sinf(x); }
static float j_cos(const kzo_world* w, float x) { return w->trig_mode ? (float)cos((double)x) : cosf(x); }
static float j_acos(const kzo_world* w, float x) { return w->trig_mode ? (float)acos((double)x) : acosf(x); }
static float j_atan2(const kzo_world* w, float y, float x) {
    return w->trig_mode ? (float)atan2((double)y, (double)x) : atan2f(y, x);
}
static qt rotate_by(const kzo_world* w, qt q, v3 dw) { /* IntegrateRotation(q, dw) (:54-59) with Quat::AxisAngle (Math.cpp:78-83) */
    float a2 = vlen2(dw);
    if (a2 < 1.0e-12f) return q;
    float a = sqrtf(a2);
    v3 ax = vnormalized(vdiv(dw, a));
    float half = a * 0.5f;
    float s = j_sin(w, half);
    qt r = Q(ax.x * s, ax.y * s, ax.z * s, j_cos(w, half));
    return qnormalized(qmul(r, q));
}
static void apply_positional(kzo_world* w, int a, int b, v3 lin, v3 ang) { /* :62-71 */
    w->pos[a] = vadd(w->pos[a], vmul(lin, w->inv_mass[a]));
    w->rot[a] = rotate_by(w, w->rot[a], mmulv(&w->iiw[a], ang));
    w->pos[b] = vsub(w->pos[b], vmul(lin, w->inv_mass[b]));
    w->rot[b] = rotate_by(w, w->rot[b], vneg(mmulv(&w->iiw[b], ang)));
}
static v3 rel_vel(const kzo_world* w, const joint_t* j) {
    return vsub(vadd(w->lv[j->a], vcross(w->av[j->a], j->r0)), vadd(w->lv[j->b], vcross(w->av[j->b], j->r1)));
}
static float hinge_angle(const kzo_world* w, const joint_t* j) { /* HingeConstraint::GetAngle (:361-368) */
    v3 axis = qrotate(w->rot[j->a], j->lax);
    v3 pa = qrotate(w->rot[j->a], j->lpa[0]), pb = qrotate(w->rot[j->b], j->lpb[0]);
    return j_atan2(w, vdot(axis, vcross(pa, pb)), vdot(pa, pb));
}

/* Constructors: world anchors and axes at the bodies' current poses. */
static void joint_init(const kzo_world* w, joint_t* j, const float* f, uint32_t modes, uint32_t motors, const float* six) {
    const int a = (int)j->a, b = (int)j->b;
    v3 anA = V(f[0], f[1], f[2]), anB = V(f[3], f[4], f[5]), axA = V(f[6], f[7], f[8]), axB = V(f[9], f[10], f[11]);
    qt rot = Q(f[12], f[13], f[14], f[15]);
    j->target = f[16]; j->lower = f[17]; j->upper = f[18]; j->motor_target = f[19]; j->motor_max = f[20];
    j->modes = modes; j->motors = motors;
    for (int k = 0; k < 12; ++k) j->six[k] = six[k];
    if (j->type == 0 && (j->flags & 8u)) {
        j->la = anA; j->lb = anB;
    } else if (j->type == 1) {
        j->la = qinv_rotate(w->rot[a], vsub(anA, w->pos[a]));
        j->lb = qinv_rotate(w->rot[b], vsub(anB, w->pos[b]));
    } else {
        j->la = qinv_rotate(w->rot[a], vsub(anA, w->pos[a]));
        j->lb = qinv_rotate(w->rot[b], vsub(anA, w->pos[b]));
    }
    if (j->type == 2) j->relrot = qmul(q_conj(w->rot[a]), w->rot[b]);
    if (j->type == 3) {
        j->lax = qinv_rotate(w->rot[a], vnormalized(axA));
        j->lbx = qinv_rotate(w->rot[b], vnormalized(axB));
        v_basis(j->lax, &j->lpa[0], &j->lpa[1]);
        v_basis(j->lbx, &j->lpb[0], &j->lpb[1]);
        if (!(j->flags & 2u)) { j->lower = -3.14159265358979323846f; j->upper = 3.14159265358979323846f; }
    }
    if (j->type == 4) {
        j->lax = qinv_rotate(w->rot[a], vnormalized(axA));
        j->lbx = qinv_rotate(w->rot[b], vnormalized(axA));
        if (!(j->flags & 2u)) { j->lower = 0.0f; j->upper = 0.0f; }
    }
    if (j->type == 5) j->crot = qtomat(rot);
}

static void joint_prepare(const kzo_world* w, joint_t* j) {
    const int a = (int)j->a, b = (int)j->b;
    j->r0 = qrotate(w->rot[a], j->la);
    j->r1 = qrotate(w->rot[b], j->lb);
    switch (j->type) {
        case 0: j->m1 = m_inverse(point_mass(w, a, b, j->r0, j->r1)); break;
        case 1: {
            v3 d = vsub(vadd(w->pos[b], j->r1), vadd(w->pos[a], j->r0));
            float dist = vlen(d);
            j->axis = dist > KZO_EPS ? vdiv(d, dist) : V(0.0f, 1.0f, 0.0f);
            j->dmass = linear_mass(w, a, b, j->r0, j->r1, j->axis);
            break;
        }
        case 2:
            j->m1 = m_inverse(point_mass(w, a, b, j->r0, j->r1));
            j->m2 = m_inverse(m_add(w->iiw[a], w->iiw[b]));
            break;
        case 3: {
            j->m1 = m_inverse(point_mass(w, a, b, j->r0, j->r1));
            v3 pa[2] = {qrotate(w->rot[a], j->lpa[0]), qrotate(w->rot[a], j->lpa[1])};
            v3 pb[2] = {qrotate(w->rot[b], j->lpb[0]), qrotate(w->rot[b], j->lpb[1])};
            for (int i = 0; i < 2; ++i) {
                v3 axis = vnormalized_or(vadd(pa[i], pb[i]), pa[i]);
                j->sm[i] = angular_mass(w, a, b, axis);
                j->lpa[i] = qinv_rotate(w->rot[a], axis);
            }
            j->limit_mass = angular_mass(w, a, b, qrotate(w->rot[a], j->lax));
            break;
        }
        case 4: {
            v3 axis = qrotate(w->rot[a], j->lax), p[2];
            v_basis(axis, &p[0], &p[1]);
            j->axial_mass = linear_mass(w, a, b, j->r0, j->r1, axis);
            m3 K = point_mass(w, a, b, j->r0, j->r1);
            float k00 = vdot(p[0], mmulv(&K, p[0]));
            float k01 = vdot(p[0], mmulv(&K, p[1]));
            float k11 = vdot(p[1], mmulv(&K, p[1]));
            float det = k00 * k11 - k01 * k01;
            if (fabs_r(det) > 1.0e-12f) {
                float inv = 1.0f / det;
                j->m1.c[0] = vadd(vmul(p[0], k11 * inv), vmul(p[1], -k01 * inv));
                j->m1.c[1] = vadd(vmul(p[0], -k01 * inv), vmul(p[1], k00 * inv));
                j->m1.c[2] = V(0, 0, 0);
            } else {
                j->m1 = m_zero();
            }
            j->m2 = m_inverse(m_add(w->iiw[a], w->iiw[b]));
            break;
        }
        case 5: {
            m3 ra = qtomat(w->rot[a]);
            m3 r = mmul(&ra, &j->crot);
            for (int i = 0; i < 3; ++i) j->axes[i] = r.c[i];
            break;
        }
    }
}

static void joint_warm(kzo_world* w, joint_t* j) {
    const int a = (int)j->a, b = (int)j->b;
    switch (j->type) {
        case 0: apply_impulse(w, a, b, j->r0, j->r1, j->imp1); break;
        case 1: apply_impulse(w, a, b, j->r0, j->r1, vmul(j->axis, j->dimp)); break;
        case 2:
            apply_impulse(w, a, b, j->r0, j->r1, j->imp1);
            apply_angular(w, a, b, j->imp2);
            break;
        case 3:
            apply_impulse(w, a, b, j->r0, j->r1, j->imp1);
            for (int i = 0; i < 2; ++i) apply_angular(w, a, b, vmul(qrotate(w->rot[a], j->lpa[i]), j->simp[i]));
            apply_angular(w, a, b, vmul(qrotate(w->rot[a], j->lax), j->limit_imp + j->motor_imp));
            break;
        case 4:
            apply_impulse(w, a, b, j->r0, j->r1, j->imp1);
            apply_angular(w, a, b, j->imp2);
            apply_impulse(w, a, b, j->r0, j->r1, vmul(qrotate(w->rot[a], j->lax), j->axial_imp));
            break;
        case 5:
            for (int i = 0; i < 3; ++i) {
                apply_impulse(w, a, b, j->r0, j->r1, j->lin_imp[i]);
                apply_angular(w, a, b, j->ang_imp[i]);
            }
            break;
    }
}

static void joint_velocity(kzo_world* w, joint_t* j) {
    const int a = (int)j->a, b = (int)j->b;
    switch (j->type) {
        case 0: {
            v3 imp = mmulv(&j->m1, vneg(rel_vel(w, j)));
            j->imp1 = vadd(j->imp1, imp);
            apply_impulse(w, a, b, j->r0, j->r1, imp);
            break;
        }
        case 1: {
            float lambda = -j->dmass * vdot(rel_vel(w, j), j->axis);
            j->dimp += lambda;
            apply_impulse(w, a, b, j->r0, j->r1, vmul(j->axis, lambda));
            break;
        }
        case 2: {
            v3 li = mmulv(&j->m1, vneg(rel_vel(w, j)));
            j->imp1 = vadd(j->imp1, li);
            apply_impulse(w, a, b, j->r0, j->r1, li);
            v3 ai = mmulv(&j->m2, vneg(vsub(w->av[a], w->av[b])));
            j->imp2 = vadd(j->imp2, ai);
            apply_angular(w, a, b, ai);
            break;
        }
        case 3: {
            v3 li = mmulv(&j->m1, vneg(rel_vel(w, j)));
            j->imp1 = vadd(j->imp1, li);
            apply_impulse(w, a, b, j->r0, j->r1, li);
            v3 wrel = vsub(w->av[a], w->av[b]);
            for (int i = 0; i < 2; ++i) {
                v3 axis = qrotate(w->rot[a], j->lpa[i]);
                float lambda = -j->sm[i] * vdot(wrel, axis);
                j->simp[i] += lambda;
                apply_angular(w, a, b, vmul(axis, lambda));
            }
            if (j->flags & 4u) {
                v3 ha = qrotate(w->rot[a], j->lax);
                float rv = vdot(vsub(w->av[a], w->av[b]), ha);
                float lambda = j->limit_mass * (j->motor_target - rv);
                float ni = fclamp_r(j->motor_imp + lambda, -j->motor_max, j->motor_max);
                lambda = ni - j->motor_imp;
                j->motor_imp = ni;
                apply_angular(w, a, b, vmul(ha, lambda));
            }
            if (j->flags & 2u) {
                v3 ha = qrotate(w->rot[a], j->lax);
                float angle = hinge_angle(w, j);
                float rv = vdot(vsub(w->av[a], w->av[b]), ha);
                float lambda = 0.0f;
                if (angle <= j->lower) {
                    lambda = j->limit_mass * (-rv);
                    j->limit_imp = fmax_r(j->limit_imp + lambda, 0.0f);
                    lambda = j->limit_imp;
                } else if (angle >= j->upper) {
                    lambda = j->limit_mass * (-rv);
                    j->limit_imp = fmin_r(j->limit_imp + lambda, 0.0f);
                    lambda = j->limit_imp;
                } else {
                    j->limit_imp = 0.0f;
                    lambda = 0.0f;
                }
                if (lambda != 0.0f) apply_angular(w, a, b, vmul(ha, lambda));
            }
            break;
        }
        case 4: {
            v3 axis = qrotate(w->rot[a], j->lax);
            v3 vr = rel_vel(w, j);
            v3 vp = vsub(vr, vmul(axis, vdot(vr, axis)));
            v3 pi = vneg(mmulv(&j->m1, vp));
            j->imp1 = vadd(j->imp1, pi);
            apply_impulse(w, a, b, j->r0, j->r1, pi);
            v3 ai = mmulv(&j->m2, vneg(vsub(w->av[a], w->av[b])));
            j->imp2 = vadd(j->imp2, ai);
            apply_angular(w, a, b, ai);
            float rel = vdot(vsub(w->lv[a], w->lv[b]), axis);
            if (j->flags & 4u) {
                float lambda = j->axial_mass * (j->motor_target - rel);
                float ni = fclamp_r(j->motor_imp + lambda, -j->motor_max, j->motor_max);
                lambda = ni - j->motor_imp;
                j->motor_imp = ni;
                apply_impulse(w, a, b, j->r0, j->r1, vmul(axis, lambda));
            } else if (j->flags & 2u) {
                v3 ra = qrotate(w->rot[a], j->la), rb = qrotate(w->rot[b], j->lb);
                float pos = vdot(vsub(vadd(w->pos[b], rb), vadd(w->pos[a], ra)), axis);
                float lambda = 0.0f;
                if (pos <= j->lower) {
                    lambda = j->axial_mass * (-rel);
                    j->axial_imp = fmax_r(j->axial_imp + lambda, 0.0f);
                    lambda = j->axial_imp;
                } else if (pos >= j->upper) {
                    lambda = j->axial_mass * (-rel);
                    j->axial_imp = fmin_r(j->axial_imp + lambda, 0.0f);
                    lambda = j->axial_imp;
                } else {
                    j->axial_imp = 0.0f;
                }
                if (lambda != 0.0f) apply_impulse(w, a, b, j->r0, j->r1, vmul(axis, lambda));
            }
            break;
        }
        case 5: {
            for (int k = 0; k < 3; ++k) { /* SolveLinearAxis (:503-536) */
                const uint32_t mode = (j->modes >> (2 * k)) & 3u;
                const int motor = (j->motors >> k) & 1u;
                if (mode == 0u && !motor) continue;
                v3 dir = j->axes[k];
                float rel = vdot(rel_vel(w, j), dir);
                float mass = linear_mass(w, a, b, j->r0, j->r1, dir);
                float target = 0.0f;
                float lambda = mass * (target - rel);
                if (motor) {
                    target = j->six[k];
                    lambda = mass * (target - rel);
                    float mx = j->six[3 + k];
                    float acc = vdot(j->lin_imp[k], dir);
                    float na = fclamp_r(acc + lambda, -mx, mx);
                    lambda = na - acc;
                } else if (mode == 2u) {
                    lambda = mass * (-rel);
                }
                v3 imp = vmul(dir, lambda);
                j->lin_imp[k] = vadd(j->lin_imp[k], imp);
                apply_impulse(w, a, b, j->r0, j->r1, imp);
            }
            for (int k = 0; k < 3; ++k) { /* SolveAngularAxis (:538-557) */
                const uint32_t mode = (j->modes >> (2 * k + 6)) & 3u;
                const int motor = (j->motors >> (3 + k)) & 1u;
                if (mode == 0u && !motor) continue;
                v3 dir = j->axes[k];
                float rel = vdot(vsub(w->av[a], w->av[b]), dir);
                float mass = angular_mass(w, a, b, dir);
                float lambda;
                if (motor) {
                    lambda = mass * (j->six[6 + k] - rel);
                    float acc = vdot(j->ang_imp[k], dir);
                    float na = fclamp_r(acc + lambda, -j->six[9 + k], j->six[9 + k]);
                    lambda = na - acc;
                } else {
                    lambda = mass * (-rel);
                }
                v3 imp = vmul(dir, lambda);
                j->ang_imp[k] = vadd(j->ang_imp[k], imp);
                apply_angular(w, a, b, imp);
            }
            break;
        }
    }
}

static void joint_position(kzo_world* w, joint_t* j) {
    const int a = (int)j->a, b = (int)j->b;
    v3 ra = qrotate(w->rot[a], j->la), rb = qrotate(w->rot[b], j->lb);
    switch (j->type) {
        case 0: {
            v3 err = vsub(vadd(w->pos[a], ra), vadd(w->pos[b], rb));
            const float slop = 0.001f;
            if (vlen2(err) < slop * slop) return;
            m3 K = m_inverse(point_mass(w, a, b, ra, rb));
            v3 imp = mmulv(&K, vneg(err));
            apply_positional(w, a, b, imp, vcross(ra, imp));
            break;
        }
        case 1: {
            v3 d = vsub(vadd(w->pos[b], rb), vadd(w->pos[a], ra));
            float dist = vlen(d);
            if (dist < KZO_EPS) return;
            v3 axis = vdiv(d, dist);
            float err = dist - j->target;
            float k = linear_mass(w, a, b, ra, rb, axis);
            float lambda = -k * err * 0.2f;
            apply_positional(w, a, b, vmul(axis, lambda), V(0, 0, 0));
            break;
        }
        case 2: case 3: {
            v3 err = vsub(vadd(w->pos[a], ra), vadd(w->pos[b], rb));
            if (vlen2(err) > 1.0e-8f) {
                m3 K = m_inverse(point_mass(w, a, b, ra, rb));
                v3 imp = vmul(mmulv(&K, vneg(err)), 0.2f);
                apply_positional(w, a, b, imp, vcross(ra, imp));
            }
            if (j->type == 3) break;
            qt cur = qmul(q_conj(w->rot[a]), w->rot[b]);
            qt diff = qmul(cur, q_conj(j->relrot));
            if (diff.w < 0.0f) diff = Q(-diff.x, -diff.y, -diff.z, -diff.w);
            float s = sqrtf(fmax_r(0.0f, 1.0f - diff.w * diff.w));
            v3 axis = s >= KZO_EPS ? vdiv(V(diff.x, diff.y, diff.z), s) : V(1.0f, 0.0f, 0.0f);
            float angle = 2.0f * j_acos(w, fclamp_r(diff.w, -1.0f, 1.0f));
            if (fabs_r(angle) > 1.0e-4f) {
                v3 ae = vmul(axis, angle);
                m3 K = m_inverse(m_add(w->iiw[a], w->iiw[b]));
                v3 imp = vmul(mmulv(&K, vneg(ae)), 0.2f);
                apply_positional(w, a, b, V(0, 0, 0), imp);
            }
            break;
        }
        case 4: {
            v3 axis = qrotate(w->rot[a], j->lax);
            v3 err = vsub(vadd(w->pos[a], ra), vadd(w->pos[b], rb));
            err = vsub(err, vmul(axis, vdot(err, axis)));
            if (vlen2(err) > 1.0e-8f) {
                m3 K = m_inverse(point_mass(w, a, b, ra, rb));
                v3 imp = vmul(mmulv(&K, vneg(err)), 0.2f);
                imp = vsub(imp, vmul(axis, vdot(imp, axis)));
                apply_positional(w, a, b, imp, vcross(ra, imp));
            }
            break;
        }
        case 5: {
            v3 err = vsub(vadd(w->pos[a], ra), vadd(w->pos[b], rb));
            for (int k = 0; k < 3; ++k) {
                if (((j->modes >> (2 * k)) & 3u) != 2u) continue;
                v3 dir = j->axes[k];
                float e = vdot(err, dir);
                if (fabs_r(e) < 1.0e-4f) continue;
                float mass = linear_mass(w, a, b, ra, rb, dir);
                v3 imp = vmul(dir, -mass * e * 0.2f);
                apply_positional(w, a, b, imp, vcross(ra, imp));
            }
            break;
        }
    }
}

static void solve_island(kzo_world* w, uint32_t isl, uint32_t* out_batches, uint32_t* out_vl, uint32_t* out_bl,
                         uint32_t* out_pts, uint32_t* out_iters, uint32_t* out_pt_iters, float* out_res) {
    const uint32_t* list = w->isl_con + w->isl_off[isl];
    uint32_t nc = w->isl_off[isl + 1] - w->isl_off[isl];
    const uint32_t* jl = w->isl_joint + w->isl_joff[isl];
    const uint32_t nj = w->isl_joff[isl + 1] - w->isl_joff[isl];
    if (nc == 0 && nj == 0) return;
    for (uint32_t i = 0; i < nc; ++i) warm_start(w, &w->cons[list[i]]);
    for (uint32_t i = 0; i < nj; ++i) joint_warm(w, &w->joints[jl[i]]);

    uint32_t npts = 0;
    for (uint32_t i = 0; i < nc; ++i) npts += w->cons[list[i]].npts;
    batch_t* bt = (batch_t*)xrealloc(NULL, sizeof(batch_t) * (npts ? npts : 1));
    uint32_t nbt = 0, nopen = 0, max_open = 0;
    for (uint32_t i = 0; i < nc && !w->scalar_solver; ++i) {
        con_t* c = &w->cons[list[i]];
        if (c->sensor) continue;
        for (uint32_t p = 0; p < c->npts; ++p) {
            int placed = 0;
            for (uint32_t bi = 0; bi < nbt && !placed; ++bi) {
                batch_t* b = &bt[bi];
                if (b->count >= 4) continue;
                int conflict = 0;
                for (uint32_t k = 0; k < b->count; ++k)
                    if (b->a[k] == c->a || b->a[k] == c->b || b->b[k] == c->a || b->b[k] == c->b) { conflict = 1; break; }
                if (conflict) continue;
                b->ref[b->count].con = (int)list[i];
                b->ref[b->count].pt = p;
                b->a[b->count] = c->a;
                b->b[b->count] = c->b;
                ++b->count;
                if (b->count == 4) --nopen;
                placed = 1;
            }
            if (!placed) {
                batch_t* b = &bt[nbt++];
                b->count = 1;
                b->ref[0].con = (int)list[i];
                b->ref[0].pt = p;
                b->a[0] = c->a;
                b->b[0] = c->b;
                ++nopen;
            }
            if (nopen > max_open) max_open = nopen;
        }
    }
    if (w->sched_stats && max_open > w->st_max_open) w->st_max_open = max_open;  /* racy max: statistics only */
    /* velocity iterations: the fixed count (the reference), or until the island residual - the
     * relative change sum|dImpulse| / sum|impulse| of the iteration - is <= res_tol, at most
     * res_cap iterations */
    const uint32_t iters = w->res_tol > 0.0f ? w->res_cap : w->vel_iters;
    uint32_t used = 0;
    float res = 0.0f;
    for (uint32_t it = 0; it < iters; ++it) {
        uint64_t sd = 0, sl = 0;
        if (w->scalar_solver) {  /* every constraint in island order, sensors included (PhysicsWorld.cpp:723-727) */
            for (uint32_t i = 0; i < nc; ++i) {
                con_t* c = &w->cons[list[i]];
                for (uint32_t p = 0; p < c->npts; ++p) solve_point_scalar(w, c, &c->p[p], &sd, &sl);
            }
        } else {
            for (uint32_t bi = 0; bi < nbt; ++bi)
                for (uint32_t k = 0; k < bt[bi].count; ++k) {
                    con_t* c = &w->cons[bt[bi].ref[k].con];
                    solve_lane(w, c, &c->p[bt[bi].ref[k].pt], &sd, &sl);
                }
        }
        used = it + 1;
        res = sl ? (float)((double)sd / (double)sl) : (sd ? 1.0f : 0.0f);
        if (w->res_tol > 0.0f && (double)sd <= (double)w->res_tol * (double)sl) break;
    }
    uint32_t nbp = 0;
    for (uint32_t bi = 0; bi < nbt; ++bi) nbp += bt[bi].count;
    if (w->scalar_solver) nbp = npts;
    *out_iters = used;
    *out_pt_iters = nbp * used;
    *out_res = res;
    /* joint velocity iterations: the configured count (the residual rule stops contacts only) */
    for (uint32_t it = 0; it < w->vel_iters; ++it)
        for (uint32_t i = 0; i < nj; ++i) joint_velocity(w, &w->joints[jl[i]]);
    if (!w->vel_bias)
        for (uint32_t it = 0; it < w->pos_iters; ++it)
            for (uint32_t i = 0; i < nc; ++i) solve_bias(w, &w->cons[list[i]]);

    if (w->sched_stats) {
        /* Dependency levels of the two Gauss-Seidel sweeps, counting only dynamic bodies. */
        uint32_t* last = (uint32_t*)calloc((size_t)w->nb, sizeof(uint32_t));
        uint32_t vl = 0;
        for (uint32_t i = 0; i < nc && w->scalar_solver; ++i) {  /* the scalar sweep: island order */
            con_t* c = &w->cons[list[i]];
            for (uint32_t p = 0; p < c->npts; ++p) {
                uint32_t l = 0;
                if (c->dynA && last[c->a] > l) l = last[c->a];
                if (c->dynB && last[c->b] > l) l = last[c->b];
                ++l;
                if (c->dynA) last[c->a] = l;
                if (c->dynB) last[c->b] = l;
                if (l > vl) vl = l;
            }
        }
        for (uint32_t bi = 0; bi < nbt; ++bi)
            for (uint32_t k = 0; k < bt[bi].count; ++k) {
                con_t* c = &w->cons[bt[bi].ref[k].con];
                uint32_t l = 0;
                if (c->dynA && last[c->a] > l) l = last[c->a];
                if (c->dynB && last[c->b] > l) l = last[c->b];
                ++l;
                if (c->dynA) last[c->a] = l;
                if (c->dynB) last[c->b] = l;
                if (l > vl) vl = l;
            }
        memset(last, 0, sizeof(uint32_t) * (size_t)w->nb);
        uint32_t bl = 0;
        for (uint32_t i = 0; i < nc; ++i) {
            con_t* c = &w->cons[list[i]];
            if (w->inv_mass[c->a] <= 0.0f && w->inv_mass[c->b] <= 0.0f) continue;
            for (uint32_t p = 0; p < c->npts; ++p) {
                if (c->p[p].pbias <= 0.0f) continue;
                uint32_t l = 0;
                if (c->dynA && last[c->a] > l) l = last[c->a];
                if (c->dynB && last[c->b] > l) l = last[c->b];
                ++l;
                if (c->dynA) last[c->a] = l;
                if (c->dynB) last[c->b] = l;
                if (l > bl) bl = l;
            }
        }
        free(last);
        *out_vl = vl;
        *out_bl = bl;
    }
    *out_batches = nbt;
    *out_pts = npts;
    free(bt);
}

/* ----------------------------------------------------------------------------- */
/* Step                                                                           */
/* ----------------------------------------------------------------------------- */
/* PhysicsWorld::ClampMotionCCD (PhysicsWorld.cpp:804-852) for body i, run inside the position
 * loop (bodies earlier in the active list already moved).  Candidates are the bodies whose fat
 * bounds overlap the swept bounds, visited in slot order (the reference visits its tree; the two
 * differ only when two casts return the same fraction). */
static void clamp_motion_ccd(kzo_world* w, int i, v3* disp) {
    const float dist = vlen(*disp);
    if (dist <= w->ccd_max_pen) return;
    if (w->ccd_thr[i] > 0.0f && dist < w->ccd_thr[i]) return; /* PhysicsWorld.cpp:807 */
    const kzo_shape* sh = &w->shapes[w->shape[i]];
    const v3 dir = vdiv(*disp, dist);
    const qt r0 = w->rot[i];
    const v3 t0 = w->pos[i];
    aabb sweep = kzo_world_bounds(sh, r0, t0);
    sweep = aabb_merge(sweep, kzo_world_bounds(sh, r0, vadd(t0, *disp)));
    sweep = AB(vsub(sweep.mn, V(0.1f, 0.1f, 0.1f)), vadd(sweep.mx, V(0.1f, 0.1f, 0.1f)));
    float best = 1.0f;
    v3 best_n = V(0.0f, 1.0f, 0.0f);
    int hit = 0;
    for (int j = 0; j < w->nb; ++j) {
        if (j == i || w->sensor[j]) continue;
        if ((w->layer[j] & w->mask[i]) == 0u || (w->layer[i] & w->mask[j]) == 0u) continue;
        if (!aabb_overlaps(w->fat[j], sweep)) continue;
        float frac;
        v3 n;
        if (kzo_cast_shape(sh, r0, t0, dir, dist, &w->shapes[w->shape[j]], w->rot[j], w->pos[j], &frac, &n) &&
            frac < best) {
            best = frac;
            best_n = n;
            hit = 1;
        }
    }
    if (!hit) return;
    float stop = best * dist - w->ccd_max_pen;
    if (stop < 0.0f) stop = 0.0f;
    *disp = vmul(dir, stop);
    const float vn = vdot(w->lv[i], best_n);
    if (vn < 0.0f) w->lv[i] = vsub(w->lv[i], vmul(best_n, vn));
}

static uint32_t uf_find(uint32_t* par, uint32_t x) {
    while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; }
    return x;
}
static void uf_union(uint32_t* par, uint32_t* rank, uint32_t a, uint32_t b) {
    a = uf_find(par, a);
    b = uf_find(par, b);
    if (a == b) return;
    if (rank[a] < rank[b]) { uint32_t t = a; a = b; b = t; }
    par[b] = a;
    if (rank[a] == rank[b]) ++rank[a];
}

/* BuildIslands (PhysicsWorld.cpp:587-664).  Active bodies get a compact index in active-list order
 * (dynamic ones; others 0xFFFFFFFF); a sleeping body keeps whatever index it last had, so its
 * contacts join (and are solved in) the island of the active body now holding that index, or of
 * their other body when the index is past the active dynamic count. */
static uint32_t island_of(const kzo_world* w, uint32_t* par, const uint32_t* r2i, uint32_t numDyn, int b) {
    if (w->motion[b] != KZO_DYNAMIC) return NUL;
    const uint32_t idx = w->island_index[b];
    if (idx >= numDyn) return NUL;
    return r2i[uf_find(par, idx)];
}

static void build_islands(kzo_world* w) {
    uint32_t numDyn = 0;
    for (int i = 0; i < w->nactive; ++i) {
        int b = w->active[i];
        w->island_index[b] = w->motion[b] == KZO_DYNAMIC ? numDyn++ : 0xFFFFFFFFu;
    }
    w->nislands = 0;
    w->st_islands = 0;
    if (numDyn == 0) return;
    /* Elements [0, numDyn) are the compact indices.  A sleeping body whose stale index is past
     * numDyn gets a link element: the reference puts each of its contacts in the other body's island
     * and solves those islands concurrently (a race on the sleeping body); linked, they become one
     * island, solved deterministically.  Without such a body the islands are the reference's. */
    uint32_t nel = numDyn;
    uint32_t* link = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * (size_t)w->nb);
    for (int b = 0; b < w->nb; ++b) {
        link[b] = NUL;
        if (w->motion[b] == KZO_DYNAMIC && !w->is_active[b] && w->island_index[b] >= numDyn)
            link[b] = nel++;
    }
    uint32_t* par = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * nel);
    uint32_t* rank = (uint32_t*)calloc(nel, sizeof(uint32_t));
    for (uint32_t i = 0; i < nel; ++i) par[i] = i;
    w->st_shared_sleepers = 0;
    for (uint32_t pass = 0; pass < 2; ++pass) {  /* contacts, then joints (PhysicsWorld.cpp:607-633) */
        const uint32_t n = pass == 0 ? w->ncons : w->njoints;
        for (uint32_t k = 0; k < n; ++k) {
            int a, b;
            if (pass == 0) { a = w->cons[k].a; b = w->cons[k].b; }
            else {
                if (w->joints[k].flags & 1u) continue;
                a = (int)w->joints[k].a; b = (int)w->joints[k].b;
            }
            if (w->motion[a] != KZO_DYNAMIC || w->motion[b] != KZO_DYNAMIC) continue;
            const uint32_t ia = w->island_index[a], ib = w->island_index[b];
            if (ia < numDyn && ib < numDyn) { uf_union(par, rank, ia, ib); continue; }
            const uint32_t x = ia < numDyn ? ia : (ib < numDyn ? ib : NUL);
            const uint32_t l = ia < numDyn ? link[b] : (ib < numDyn ? link[a] : NUL);
            if (x == NUL || l == NUL) continue;
            const uint32_t rl = uf_find(par, l), rx = uf_find(par, x);
            if (rl != l && rl != rx) ++w->st_shared_sleepers;  /* a second island reached the same body */
            uf_union(par, rank, x, l);
        }
    }
    free(link);
    uint32_t* r2i = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * numDyn);
    for (uint32_t i = 0; i < numDyn; ++i) r2i[i] = NUL;
    uint32_t ni = 0;
    for (uint32_t i = 0; i < numDyn; ++i) {
        uint32_t r = uf_find(par, i);
        if (r2i[r] == NUL) r2i[r] = ni++;
    }
    w->nislands = ni;
    w->st_islands = ni;
    uint32_t* isl = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * (w->ncons ? w->ncons : 1));
    w->isl_off = (uint32_t*)xrealloc(w->isl_off, sizeof(uint32_t) * (ni + 1));
    memset(w->isl_off, 0, sizeof(uint32_t) * (ni + 1));
    for (uint32_t ci = 0; ci < w->ncons; ++ci) {
        con_t* c = &w->cons[ci];
        uint32_t is = island_of(w, par, r2i, numDyn, c->a);
        if (is == NUL) is = island_of(w, par, r2i, numDyn, c->b);
        isl[ci] = is;
        if (is != NUL) w->isl_off[is + 1]++;
    }
    for (uint32_t i = 0; i < ni; ++i) w->isl_off[i + 1] += w->isl_off[i];
    w->isl_con = (uint32_t*)xrealloc(w->isl_con, sizeof(uint32_t) * (w->ncons ? w->ncons : 1));
    uint32_t* fill = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * (ni ? ni : 1));
    for (uint32_t i = 0; i < ni; ++i) fill[i] = w->isl_off[i];
    for (uint32_t ci = 0; ci < w->ncons; ++ci)
        if (isl[ci] != NUL) w->isl_con[fill[isl[ci]]++] = ci;
    /* joints of each island in joint order (PhysicsWorld.cpp:656-661) */
    w->isl_joff = (uint32_t*)xrealloc(w->isl_joff, sizeof(uint32_t) * (ni + 1));
    memset(w->isl_joff, 0, sizeof(uint32_t) * (ni + 1));
    uint32_t* jis = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * (w->njoints ? w->njoints : 1));
    for (uint32_t ji = 0; ji < w->njoints; ++ji) {
        const joint_t* j = &w->joints[ji];
        uint32_t is = NUL;
        if (!(j->flags & 1u)) {
            is = island_of(w, par, r2i, numDyn, (int)j->a);
            if (is == NUL) is = island_of(w, par, r2i, numDyn, (int)j->b);
        }
        jis[ji] = is;
        if (is != NUL) w->isl_joff[is + 1]++;
    }
    for (uint32_t i = 0; i < ni; ++i) w->isl_joff[i + 1] += w->isl_joff[i];
    w->isl_joint = (uint32_t*)xrealloc(w->isl_joint, sizeof(uint32_t) * (w->njoints ? w->njoints : 1));
    for (uint32_t i = 0; i < ni; ++i) fill[i] = w->isl_joff[i];
    for (uint32_t ji = 0; ji < w->njoints; ++ji)
        if (jis[ji] != NUL) w->isl_joint[fill[jis[ji]]++] = ji;
    free(jis);
    free(fill);
    free(isl);
    free(r2i);
    free(rank);
    free(par);
}

/* BodyManager::ActivateBody (BodyManager.cpp:133-141): an inactive body becomes active with a zero
 * sleep timer and is appended to the active list. */
static void activate_body(kzo_world* w, int b) {
    if (w->is_active[b]) return;
    w->is_active[b] = 1;
    w->sleep_timer[b] = 0.0f;
    w->active[w->nactive++] = b;
}

/* BodyManager::DeactivateBody (BodyManager.cpp:143-154): velocities zeroed, swap-removed from the
 * active list (the last entry moves into its place; the buffer keeps the old last value). */
static void deactivate_body(kzo_world* w, int b) {
    if (!w->is_active[b]) return;
    w->is_active[b] = 0;
    w->lv[b] = V(0, 0, 0);
    w->av[b] = V(0, 0, 0);
    for (int k = 0; k < w->nactive; ++k)
        if (w->active[k] == b) {
            w->active[k] = w->active[w->nactive - 1];
            --w->nactive;
            break;
        }
}

/* The wake rule of BuildContactConstraints (PhysicsWorld.cpp:473-490): a dynamic body is moving
 * when active, a kinematic one when it has a velocity, a static one never. */
static int body_moving(const kzo_world* w, int b) {
    if (w->motion[b] == KZO_DYNAMIC) return w->is_active[b];
    if (w->motion[b] == KZO_KINEMATIC) return vlen2(w->lv[b]) > 0.0f || vlen2(w->av[b]) > 0.0f;
    return 0;
}

/* UpdateSleeping (PhysicsWorld.cpp:866-951).  Runs over the active list as it was when the pass
 * began (n entries); the deactivation loop reads the list while swap-removals change it, which
 * still visits every original entry once at its original position, and the island count at the end
 * reads the list's buffer past its new end. */
static void update_sleeping(kzo_world* w, float dt) {
    if (!w->allow_sleeping) return;
    const uint32_t n = (uint32_t)w->nactive;
    if (n == 0) return;
    const float lt = w->sleep_lin * w->sleep_lin, at = w->sleep_ang * w->sleep_ang;
    for (uint32_t i = 0; i < n; ++i) {
        const int b = w->active[i];
        if (w->motion[b] != KZO_DYNAMIC || !w->allow_sleep[b]) { w->sleep_timer[b] = 0.0f; continue; }
        if (vlen2(w->lv[b]) < lt && vlen2(w->av[b]) < at) w->sleep_timer[b] += dt;
        else w->sleep_timer[b] = 0.0f;
    }
    uint32_t* par = (uint32_t*)xrealloc(NULL, sizeof(uint32_t) * n);
    uint32_t* rank = (uint32_t*)calloc(n, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) par[i] = i;
    for (uint32_t i = 0; i < n; ++i) w->island_index[w->active[i]] = i;
    for (uint32_t ci = 0; ci < w->ncons; ++ci) {
        const con_t* c = &w->cons[ci];
        if (w->motion[c->a] != KZO_DYNAMIC || w->motion[c->b] != KZO_DYNAMIC) continue;
        const uint32_t ia = w->island_index[c->a], ib = w->island_index[c->b];
        if (ia < n && ib < n) uf_union(par, rank, ia, ib);
    }
    for (uint32_t ji = 0; ji < w->njoints; ++ji) {
        const joint_t* j = &w->joints[ji];
        if (j->flags & 1u) continue;
        if (w->motion[j->a] != KZO_DYNAMIC || w->motion[j->b] != KZO_DYNAMIC) continue;
        const uint32_t ia = w->island_index[j->a], ib = w->island_index[j->b];
        if (ia < n && ib < n) uf_union(par, rank, ia, ib);
    }
    float* mt = (float*)xrealloc(NULL, sizeof(float) * n);
    for (uint32_t i = 0; i < n; ++i) mt[i] = 1.0e18f; /* math::kBigNumber (Types.h:44) */
    for (uint32_t i = 0; i < n; ++i) {
        const int b = w->active[i];
        if (w->motion[b] != KZO_DYNAMIC || !w->allow_sleep[b]) continue;
        const uint32_t r = uf_find(par, i);
        mt[r] = fmin_r(mt[r], w->sleep_timer[b]);
    }
    for (uint32_t i = 0; i < n; ++i) {
        const int b = w->active[i]; /* the original entry i (see above) */
        if (w->motion[b] != KZO_DYNAMIC || !w->allow_sleep[b]) continue;
        if (mt[uf_find(par, i)] >= w->sleep_time) {
            w->lv[b] = V(0, 0, 0);
            w->av[b] = V(0, 0, 0);
            deactivate_body(w, b);
        }
    }
    uint32_t count = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const int b = w->active[i]; /* past the new end: the buffer's leftover values */
        if (w->motion[b] != KZO_DYNAMIC) continue;
        if (uf_find(par, i) == i) ++count;
    }
    w->st_islands = count;
    free(mt);
    free(rank);
    free(par);
}

static void collide_one(kzo_world* w, uint32_t i) {
    uint32_t ida = w->pairs[2 * i], idb = w->pairs[2 * i + 1];
    int A = body_of(w, ida), B = body_of(w, idb);
    w->man[i].n = 0;
    w->keys[i] = 0;
    if (A < 0 || B < 0) return;
    if (w->motion[A] != KZO_DYNAMIC && w->motion[B] != KZO_DYNAMIC) return;
    int swapped = ida > idb;
    int first = swapped ? B : A, second = swapped ? A : B;
    w->keys[i] = pair_key(ida, idb);
    kzo_collide(&w->shapes[w->shape[first]], w->rot[first], w->pos[first], &w->shapes[w->shape[second]],
                w->rot[second], w->pos[second], 0.02f, 1.0e-4f, &w->man[i]);
    if (swapped) {
        kzo_manifold* m = &w->man[i];
        for (uint32_t k = 0; k < m->n; ++k) {
            v3 t = m->pts[k].pA;
            m->pts[k].pA = m->pts[k].pB;
            m->pts[k].pB = t;
            m->pts[k].n = vneg(m->pts[k].n);
        }
    }
}

static void build_constraints(kzo_world* w) {
    w->ncons = 0;
    for (uint32_t i = 0; i < w->npairs; ++i) {
        kzo_manifold* m = &w->man[i];
        if (m->n == 0) continue;
        uint64_t key = w->keys[i];
        if (key == 0) continue;
        int A = body_of(w, w->pairs[2 * i]), B = body_of(w, w->pairs[2 * i + 1]);
        if (A < 0 || B < 0) continue;
        if (w->packed[A] > w->packed[B]) { int t = A; A = B; B = t; }
        /* wake a sleeping dynamic body touched by a moving one, in pair order (:473-490) */
        if (w->motion[A] == KZO_DYNAMIC && !w->is_active[A] && body_moving(w, B)) activate_body(w, A);
        if (w->motion[B] == KZO_DYNAMIC && !w->is_active[B] && body_moving(w, A)) activate_body(w, B);
        cache_t* cached = w->no_ws ? NULL : find_cached(w, key);
        if (w->ncons == w->cons_cap) {
            w->cons_cap = w->cons_cap ? w->cons_cap * 2 : 1024;
            w->cons = (con_t*)xrealloc(w->cons, sizeof(con_t) * w->cons_cap);
        }
        con_t* c = &w->cons[w->ncons++];
        memset(c, 0, sizeof *c);
        c->a = A;
        c->b = B;
        c->sensor = w->sensor[A] || w->sensor[B];
        c->friction = sqrtf(w->fric[A] * w->fric[B]);
        c->restitution = fmax_r(w->rest[A], w->rest[B]);
        c->npts = m->n;
        for (uint32_t p = 0; p < m->n; ++p) {
            cpc_t* q = &c->p[p];
            const kzo_cpoint* s = &m->pts[p];
            q->pA = s->pA; q->pB = s->pB; q->n = s->n; q->sep = s->sep; q->feature = s->feature;
            q->fric = c->friction;
            q->rest = c->restitution;
            q->ni = q->ti1 = q->ti2 = 0;
            if (cached) {
                float best = 0.10f * 0.10f;
                uint32_t bi = NUL;
                for (uint32_t k = 0; k < cached->npts; ++k) {
                    float d = vlen2(vsub(cached->pos[k], s->pA));
                    if (d < best) { best = d; bi = k; }
                }
                if (bi != NUL) { q->ni = cached->ni[bi]; q->ti1 = cached->ti1[bi]; q->ti2 = cached->ti2[bi]; }
            }
        }
    }
}

static void integrate_velocities(kzo_world* w, float dt) {
    for (int k = 0; k < w->nactive; ++k) {
        int i = w->active[k];
        if (w->motion[i] != KZO_DYNAMIC) continue;
        v3 acc = vadd(vmul(w->gravity, w->grav[i]), vmul(w->force[i], w->inv_mass[i]));
        w->lv[i] = vadd(w->lv[i], vmul(acc, dt));
        w->av[i] = vadd(w->av[i], vmul(mmulv(&w->iiw[i], w->torque[i]), dt));
        w->lv[i] = vmul(w->lv[i], 1.0f / (1.0f + w->lin_damp[i] * dt));
        w->av[i] = vmul(w->av[i], 1.0f / (1.0f + w->ang_damp[i] * dt));
        w->lv[i] = vclamp_len(w->lv[i], w->max_lin[i]);
        w->av[i] = vclamp_len(w->av[i], w->max_ang[i]);
        if (!visfinite(w->lv[i]) || !visfinite(w->av[i])) { w->lv[i] = V(0, 0, 0); w->av[i] = V(0, 0, 0); }
    }
}

static void update_world_inertia(kzo_world* w, int i) {
    m3 r = qtomat(w->rot[i]);
    m3 ri = mmul(&r, &w->iil[i]);
    m3 rt = mtranspose(&r);
    w->iiw[i] = mmul(&ri, &rt);
}

int kzo_step(kzo_world* w, float dt) {
    ++w->frame;
    if (w->frame == 0) w->frame = 1;

    /* 1. broad phase.  Every mode keeps the bodies' fat bounds the way the tree's MoveProxy does
     * (BroadPhase.cpp:58-75): continuous collision queries them. */
    for (int k = 0; k < w->nactive; ++k) {
        int i = w->active[k];
        if (w->motion[i] == KZO_STATIC) continue;
        aabb b = kzo_world_bounds(&w->shapes[w->shape[i]], w->rot[i], w->pos[i]);
        if (aabb_contains(w->fat[i], b)) continue;
        v3 d = vabs(vmul(w->lv[i], w->fixed_dt));
        v3 margin = V(0.1f, 0.1f, 0.1f);
        w->fat[i] = AB(vsub(vsub(b.mn, margin), d), vadd(vadd(b.mx, margin), d));
    }
    if (w->pair_mode == KZO_PAIRS_TREE) {
        for (int k = 0; k < w->nactive; ++k) {
            int i = w->active[k];
            if (w->motion[i] == KZO_STATIC) continue;
            aabb b = kzo_world_bounds(&w->shapes[w->shape[i]], w->rot[i], w->pos[i]);
            move_proxy(w, w->proxy[i], b, vmul(w->lv[i], w->fixed_dt));
        }
        tree_pairs(w);
    } else if (w->pair_mode == KZO_PAIRS_CANONICAL) {
        canonical_pairs(w);
    } else {
        w->npairs = 0;
        for (uint32_t i = 0; i < w->next_pairs; ++i) push_pair(w, w->ext_pairs[2 * i], w->ext_pairs[2 * i + 1]);
    }

    /* 2. narrow phase */
    if (w->npairs > w->man_cap) {
        w->man_cap = w->npairs;
        w->man = (kzo_manifold*)xrealloc(w->man, sizeof(kzo_manifold) * w->man_cap);
        w->keys = (uint64_t*)xrealloc(w->keys, sizeof(uint64_t) * w->man_cap);
    }
    int np = (int)w->npairs;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 32) num_threads(w->threads) if (w->threads > 1 && np > 64)
#endif
    for (int i = 0; i < np; ++i) collide_one(w, (uint32_t)i);

    /* 3. constraints with warm start */
    build_constraints(w);
    /* 4. velocities */
    integrate_velocities(w, dt);
    /* 5. solve */
    for (uint32_t ci = 0; ci < w->ncons; ++ci) prepare(w, &w->cons[ci], dt);
    for (uint32_t ji = 0; ji < w->njoints; ++ji)
        if (!(w->joints[ji].flags & 1u)) joint_prepare(w, &w->joints[ji]);
    build_islands(w);
    w->st_batches = w->st_max_vl = w->st_max_bl = w->st_max_isl_pts = w->st_sum_vl = w->st_max_open = 0;
    int ni = (int)w->nislands;
    uint32_t* ib = (uint32_t*)calloc((size_t)(ni ? ni : 1) * 6, sizeof(uint32_t));
    float* ires = (float*)calloc((size_t)(ni ? ni : 1), sizeof(float));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(w->threads) if (w->threads > 1 && ni > 1)
#endif
    for (int i = 0; i < ni; ++i)
        solve_island(w, (uint32_t)i, &ib[6 * i], &ib[6 * i + 1], &ib[6 * i + 2], &ib[6 * i + 3], &ib[6 * i + 4],
                     &ib[6 * i + 5], &ires[i]);
    w->st_max_iters = w->st_pt_iters = 0;
    w->st_final_res = 0.0f;
    for (int i = 0; i < ni; ++i) {
        w->st_batches += ib[6 * i];
        if (ib[6 * i + 1] > w->st_max_vl) w->st_max_vl = ib[6 * i + 1];
        if (ib[6 * i + 2] > w->st_max_bl) w->st_max_bl = ib[6 * i + 2];
        if (ib[6 * i + 3] > w->st_max_isl_pts) w->st_max_isl_pts = ib[6 * i + 3];
        w->st_sum_vl += ib[6 * i + 1];
        if (ib[6 * i + 4] > w->st_max_iters) w->st_max_iters = ib[6 * i + 4];
        w->st_pt_iters += ib[6 * i + 5];
        w->st_final_res = fmaxf(w->st_final_res, ires[i]);
    }
    free(ires);
    free(ib);
    for (uint32_t ci = 0; ci < w->ncons; ++ci) {
        con_t* c = &w->cons[ci];
        cache_t* e = get_or_create_cached(w, pair_key(w->packed[c->a], w->packed[c->b]));
        e->npts = c->npts;
        for (uint32_t p = 0; p < c->npts; ++p) {
            e->pos[p] = c->p[p].pA;
            e->ni[p] = c->p[p].ni;
            e->ti1[p] = c->p[p].ti1;
            e->ti2[p] = c->p[p].ti2;
        }
    }
    /* 6. positions, split-impulse pseudo velocities, inertia */
    for (int k = 0; k < w->nactive; ++k) {
        int i = w->active[k];
        if (w->motion[i] == KZO_STATIC) continue;
        v3 disp = vmul(w->lv[i], dt);
        if (w->use_ccd && w->motion[i] == KZO_DYNAMIC && w->ccd[i]) clamp_motion_ccd(w, i, &disp);
        w->pos[i] = vadd(w->pos[i], disp);
        if (vlen2(w->av[i]) > 0.0f) w->rot[i] = q_integrate(w->rot[i], w->av[i], dt);
    }
    if (!w->vel_bias) {
        for (int k = 0; k < w->nactive; ++k) {
            int i = w->active[k];
            if (w->motion[i] == KZO_STATIC) continue;
            if (vlen2(w->plv[i]) > 0.0f) w->pos[i] = vadd(w->pos[i], vmul(w->plv[i], dt));
            if (vlen2(w->pav[i]) > 0.0f) w->rot[i] = q_integrate(w->rot[i], w->pav[i], dt);
            w->plv[i] = V(0, 0, 0);
            w->pav[i] = V(0, 0, 0);
        }
    }
    for (int k = 0; k < w->nactive; ++k) {
        int i = w->active[k];
        if (w->motion[i] == KZO_DYNAMIC) update_world_inertia(w, i);
    }
    /* 7. joint position correction per island (PhysicsWorld.cpp:293-306, 745-752) */
    for (uint32_t is = 0; is < w->nislands; ++is)
        for (uint32_t it = 0; it < w->pos_iters; ++it)
            for (uint32_t k = w->isl_joff[is]; k < w->isl_joff[is + 1]; ++k) joint_position(w, &w->joints[w->isl_joint[k]]);
    /* 8. sleeping */
    update_sleeping(w, dt);
    /* 9. clear forces */
    for (int i = 0; i < w->nb; ++i) { w->force[i] = V(0, 0, 0); w->torque[i] = V(0, 0, 0); }
    uint32_t pts = 0;
    for (uint32_t ci = 0; ci < w->ncons; ++ci) pts += w->cons[ci].npts;
    w->st_points = pts;
    return 0;
}

/* ----------------------------------------------------------------------------- */
/* Creation / API                                                                 */
/* ----------------------------------------------------------------------------- */
typedef struct { const uint8_t* p; size_t n, off; int bad; } rd_t;
static void rd(rd_t* r, void* dst, size_t k) {
    if (r->off + k > r->n) { r->bad = 1; memset(dst, 0, k); return; }
    memcpy(dst, r->p + r->off, k);
    r->off += k;
}
static uint32_t rd_u32(rd_t* r) { uint32_t v; rd(r, &v, 4); return v; }
static float rd_f32(rd_t* r) { float v; rd(r, &v, 4); return v; }

kzo_world* kzo_create(const uint8_t* scene, size_t scene_len, const uint8_t* resolved, size_t resolved_len) {
    rd_t r = {scene, scene_len, 0, 0};
    if (rd_u32(&r) != 0x43535A4Bu) { set_err("bad scene header"); return NULL; }
    const uint32_t version = rd_u32(&r);
    if (version != 1u && version != 2u) { set_err("bad scene version"); return NULL; }
    kzo_world* w = (kzo_world*)calloc(1, sizeof(kzo_world));
    w->gravity.x = rd_f32(&r); w->gravity.y = rd_f32(&r); w->gravity.z = rd_f32(&r);
    (void)rd_f32(&r); /* scene dt: the caller passes dt to kzo_step */
    w->vel_iters = rd_u32(&r);
    w->pos_iters = rd_u32(&r);
    uint32_t wflags = rd_u32(&r);
    w->baumgarte = rd_f32(&r);
    w->slop = rd_f32(&r);
    w->rest_thresh = rd_f32(&r);
    w->max_bias = rd_f32(&r);
    w->ws_factor = rd_f32(&r);
    /* WorldSettings sleep thresholds (PhysicsWorld.h:25-27); version 1 scenes carry the defaults */
    w->sleep_time = 0.5f; w->sleep_lin = 0.05f; w->sleep_ang = 0.1f;
    if (version >= 2u) { w->sleep_time = rd_f32(&r); w->sleep_lin = rd_f32(&r); w->sleep_ang = rd_f32(&r); }
    w->allow_sleeping = (wflags & 1u) != 0;
    w->vel_bias = (wflags & 2u) != 0;
    w->no_ws = (wflags & 4u) != 0;
    w->scalar_solver = (wflags & 8u) != 0;  /* SolverSettings::useSIMDSolver = false */
    w->fixed_dt = (float)(1.0 / 60.0); /* WorldSettings::fixedTimestep, PhysicsWorld.h:32 */
    w->threads = 1;
    w->root = NUL;
    w->free_list = NUL;

    rd_t rr = {resolved, resolved_len, 0, 0};
    w->nshapes = (int)rd_u32(&r);
    w->shapes = (kzo_shape*)calloc((size_t)w->nshapes, sizeof(kzo_shape));
    for (int i = 0; i < w->nshapes; ++i) {
        kzo_shape* s = &w->shapes[i];
        s->type = (int)rd_u32(&r);
        for (int k = 0; k < 4; ++k) s->p[k] = rd_f32(&r);
        uint32_t npts = rd_u32(&r);
        r.off += 12u * npts; /* hull input cloud: the resolved blob carries the built hull */
        switch (s->type) {
            case KZO_SPHERE: { v3 e = V(s->p[0], s->p[0], s->p[0]); s->local = AB(vneg(e), e); break; }
            case KZO_BOX: { v3 e = V(s->p[0], s->p[1], s->p[2]); s->local = AB(vneg(e), e); break; }
            case KZO_CAPSULE: { v3 e = V(s->p[1], s->p[0] + s->p[1], s->p[1]); s->local = AB(vneg(e), e); break; }
            case KZO_PLANE: {
                const float big = 1.0e6f;
                v3 n = V(s->p[0], s->p[1], s->p[2]);
                v3 ext = vsub(V(big, big, big), vmul(vabs(n), big));
                v3 c = vmul(n, s->p[3]);
                s->local = AB(vsub(c, ext), vadd(c, ext));
                break;
            }
            case KZO_HULL: {
                s->nverts = (int)rd_u32(&rr);
                s->verts = (v3*)calloc((size_t)s->nverts, sizeof(v3));
                for (int k = 0; k < s->nverts; ++k) { s->verts[k].x = rd_f32(&rr); s->verts[k].y = rd_f32(&rr); s->verts[k].z = rd_f32(&rr); }
                s->nfaces = (int)rd_u32(&rr);
                s->sizes = (uint8_t*)calloc((size_t)s->nfaces + 4, 1);
                rd(&rr, s->sizes, (size_t)s->nfaces);
                rr.off = (rr.off + 3u) & ~(size_t)3u;
                s->nidx = (int)rd_u32(&rr);
                s->idx = (uint32_t*)calloc((size_t)s->nidx, sizeof(uint32_t));
                rd(&rr, s->idx, 4u * (size_t)s->nidx);
                aabb b = aabb_empty();
                for (int k = 0; k < s->nverts; ++k) { b.mn = vmin(b.mn, s->verts[k]); b.mx = vmax(b.mx, s->verts[k]); }
                s->local = b;
                break;
            }
            default: set_err("unsupported shape type"); kzo_destroy(w); return NULL;
        }
    }
    int nb = (int)rd_u32(&r);
    w->nb = nb;
#define ALLOC(f, T) w->f = (T*)calloc((size_t)(nb ? nb : 1), sizeof(T))
    ALLOC(packed, uint32_t); ALLOC(layer, uint32_t); ALLOC(mask, uint32_t); ALLOC(proxy, uint32_t);
    ALLOC(shape, int); ALLOC(motion, uint8_t); ALLOC(sensor, uint8_t); ALLOC(ccd, uint8_t); ALLOC(fat, aabb);
    ALLOC(ccd_thr, float);
    ALLOC(pos, v3); ALLOC(lv, v3); ALLOC(av, v3); ALLOC(plv, v3); ALLOC(pav, v3); ALLOC(force, v3); ALLOC(torque, v3);
    ALLOC(rot, qt);
    ALLOC(inv_mass, float); ALLOC(lin_damp, float); ALLOC(ang_damp, float); ALLOC(grav, float);
    ALLOC(max_lin, float); ALLOC(max_ang, float); ALLOC(fric, float); ALLOC(rest, float);
    ALLOC(iil, m3); ALLOC(iiw, m3); ALLOC(active, int); ALLOC(island_index, uint32_t);
    ALLOC(allow_sleep, uint8_t); ALLOC(is_active, uint8_t); ALLOC(sleep_timer, float);
#undef ALLOC
    for (int i = 0; i < nb; ++i) {
        w->shape[i] = (int)rd_u32(&r);
        w->motion[i] = (uint8_t)rd_u32(&r);
        w->pos[i].x = rd_f32(&r); w->pos[i].y = rd_f32(&r); w->pos[i].z = rd_f32(&r);
        w->rot[i].x = rd_f32(&r); w->rot[i].y = rd_f32(&r); w->rot[i].z = rd_f32(&r); w->rot[i].w = rd_f32(&r);
        w->lv[i].x = rd_f32(&r); w->lv[i].y = rd_f32(&r); w->lv[i].z = rd_f32(&r);
        w->av[i].x = rd_f32(&r); w->av[i].y = rd_f32(&r); w->av[i].z = rd_f32(&r);
        w->fric[i] = rd_f32(&r); w->rest[i] = rd_f32(&r);
        w->lin_damp[i] = rd_f32(&r); w->ang_damp[i] = rd_f32(&r); w->grav[i] = rd_f32(&r);
        w->max_lin[i] = rd_f32(&r); w->max_ang[i] = rd_f32(&r);
        (void)rd_f32(&r); (void)rd_f32(&r); /* density, mass override: resolved mass comes in the blob */
        w->layer[i] = rd_u32(&r); w->mask[i] = rd_u32(&r);
        uint32_t fl = rd_u32(&r);
        w->ccd_thr[i] = version >= 2u ? rd_f32(&r) : 0.0f; /* BodySettings::ccdMotionThreshold */
        w->sensor[i] = (fl & 1u) != 0;
        w->allow_sleep[i] = (fl & 2u) != 0;
        w->is_active[i] = 1;            /* BodyManager::CreateBody: active, in the active list */
        w->island_index[i] = 0xFFFFFFFFu;
        w->ccd[i] = (fl & 4u) != 0;
        w->packed[i] = (uint32_t)i; /* BodyID(index, sequence 0).Packed() */
        w->active[i] = i;
        w->inv_mass[i] = rd_f32(&rr);
        for (int c = 0; c < 3; ++c) { w->iil[i].c[c].x = rd_f32(&rr); w->iil[i].c[c].y = rd_f32(&rr); w->iil[i].c[c].z = rd_f32(&rr); }
        if (w->shape[i] < 0 || w->shape[i] >= w->nshapes) { set_err("bad shape index"); kzo_destroy(w); return NULL; }
    }
    w->nactive = nb;
    if (r.bad || rr.bad) { set_err("truncated scene or resolved data"); kzo_destroy(w); return NULL; }
    for (int i = 0; i < nb; ++i) {
        if (w->motion[i] == KZO_DYNAMIC && w->inv_mass[i] > 0.0f) update_world_inertia(w, i);
        aabb b = kzo_world_bounds(&w->shapes[w->shape[i]], w->rot[i], w->pos[i]);
        w->proxy[i] = create_proxy(w, b, w->packed[i], w->layer[i], w->mask[i]);
        w->fat[i] = AB(vsub(b.mn, V(0.1f, 0.1f, 0.1f)), vadd(b.mx, V(0.1f, 0.1f, 0.1f)));
    }
    /* optional joint section, created after every body (PhysicsWorld::AddConstraint) */
    if (r.off < r.n) {
        uint32_t nj = rd_u32(&r);
        if (nj > (uint32_t)(r.n / 156u)) { set_err("bad joint count"); kzo_destroy(w); return NULL; }
        w->joints = (joint_t*)calloc(nj ? nj : 1, sizeof(joint_t));
        for (uint32_t k = 0; k < nj; ++k) {
            joint_t* j = &w->joints[k];
            j->type = rd_u32(&r); j->a = rd_u32(&r); j->b = rd_u32(&r); j->flags = rd_u32(&r);
            float f[21], six[12];
            for (int q = 0; q < 21; ++q) f[q] = rd_f32(&r);
            uint32_t modes = rd_u32(&r), motors = rd_u32(&r);
            for (int q = 0; q < 12; ++q) six[q] = rd_f32(&r);
            if (r.bad || j->type > 5u || j->a >= (uint32_t)nb || j->b >= (uint32_t)nb) {
                set_err("bad joint record");
                kzo_destroy(w);
                return NULL;
            }
            joint_init(w, j, f, modes, motors, six);
            w->njoints = k + 1;
        }
    }
    w->use_ccd = 1;
    w->ccd_max_pen = 0.01f;
    w->cache_cap = 1024;
    w->cache = (cache_t*)calloc(w->cache_cap, sizeof(cache_t));
    return w;
}

void kzo_set_trig_mode(kzo_world* w, int mode) { w->trig_mode = mode; }
void kzo_set_cache_hash(kzo_world* w, int mixed) { w->cache_mix = mixed != 0; }

void kzo_destroy(kzo_world* w) {
    if (!w) return;
    for (int i = 0; i < w->nshapes; ++i) { free(w->shapes[i].verts); free(w->shapes[i].sizes); free(w->shapes[i].idx); }
    free(w->shapes);
    void* ptrs[] = {w->packed, w->layer, w->mask, w->proxy, w->shape, w->motion, w->sensor, w->ccd, w->ccd_thr, w->fat, w->pos, w->lv, w->av,
                    w->plv, w->pav, w->force, w->torque, w->rot, w->inv_mass, w->lin_damp, w->ang_damp, w->grav,
                    w->max_lin, w->max_ang, w->fric, w->rest, w->iil, w->iiw, w->active, w->island_index,
                    w->allow_sleep, w->is_active, w->sleep_timer,
                    w->nodes, w->bp_layer, w->bp_mask, w->cache, w->pairs, w->ext_pairs, w->man, w->keys,
                    w->cons, w->isl_off, w->isl_con, w->joints, w->isl_joff, w->isl_joint};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; ++i) free(ptrs[i]);
    free(w);
}

void kzo_set_threads(kzo_world* w, int t) { w->threads = t > 0 ? t : 1; }
void kzo_set_pair_mode(kzo_world* w, int m) { w->pair_mode = m; }
void kzo_set_schedule_stats(kzo_world* w, int e) { w->sched_stats = e; }
void kzo_set_residual(kzo_world* w, float tol, uint32_t cap) {
    w->res_tol = tol;
    w->res_cap = cap ? cap : 1u;
}
int kzo_set_external_pairs(kzo_world* w, const uint32_t* p, uint32_t n) {
    w->ext_pairs = (uint32_t*)xrealloc(w->ext_pairs, sizeof(uint32_t) * 2 * (n ? n : 1));
    memcpy(w->ext_pairs, p, sizeof(uint32_t) * 2 * n);
    w->next_pairs = n;
    return 0;
}
uint32_t kzo_num_bodies(const kzo_world* w) { return (uint32_t)w->nb; }

void kzo_get_state(const kzo_world* w, float* o) {
    for (int i = 0; i < w->nb; ++i) {
        float* q = o + KZO_STATE_FLOATS * i;
        q[0] = w->pos[i].x; q[1] = w->pos[i].y; q[2] = w->pos[i].z;
        q[3] = w->rot[i].x; q[4] = w->rot[i].y; q[5] = w->rot[i].z; q[6] = w->rot[i].w;
        q[7] = w->lv[i].x; q[8] = w->lv[i].y; q[9] = w->lv[i].z;
        q[10] = w->av[i].x; q[11] = w->av[i].y; q[12] = w->av[i].z;
    }
}
void kzo_set_state(kzo_world* w, const float* in) {
    for (int i = 0; i < w->nb; ++i) {
        const float* q = in + KZO_STATE_FLOATS * i;
        w->pos[i] = V(q[0], q[1], q[2]);
        w->rot[i] = Q(q[3], q[4], q[5], q[6]);
        w->lv[i] = V(q[7], q[8], q[9]);
        w->av[i] = V(q[10], q[11], q[12]);
        if (w->motion[i] == KZO_DYNAMIC) update_world_inertia(w, i);
    }
}

uint64_t kzo_hash(const kzo_world* w) {
    uint64_t h = 1469598103934665603ull;
#define MIX(v) do { h ^= (uint64_t)(v); h *= 1099511628211ull; } while (0)
#define QZ(f) ((uint64_t)(int64_t)((f) * 100000.0f))
    for (int i = 0; i < w->nb; ++i) {
        MIX(w->packed[i]);
        MIX(QZ(w->pos[i].x)); MIX(QZ(w->pos[i].y)); MIX(QZ(w->pos[i].z));
        MIX(QZ(w->rot[i].x)); MIX(QZ(w->rot[i].y)); MIX(QZ(w->rot[i].z)); MIX(QZ(w->rot[i].w));
        MIX(QZ(w->lv[i].x)); MIX(QZ(w->lv[i].y)); MIX(QZ(w->lv[i].z));
        MIX(QZ(w->av[i].x)); MIX(QZ(w->av[i].y)); MIX(QZ(w->av[i].z));
    }
#undef MIX
#undef QZ
    return h;
}

uint32_t kzo_num_pairs(const kzo_world* w) { return w->npairs; }
void kzo_get_pairs(const kzo_world* w, uint32_t* out) { memcpy(out, w->pairs, sizeof(uint32_t) * 2 * w->npairs); }
uint32_t kzo_num_constraints(const kzo_world* w) { return w->ncons; }

static void put3(float* o, v3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
void kzo_get_constraints(const kzo_world* w, uint32_t* hdr, float* pts, float* fr) {
    for (uint32_t ci = 0; ci < w->ncons; ++ci) {
        const con_t* c = &w->cons[ci];
        hdr[3 * ci] = w->packed[c->a];
        hdr[3 * ci + 1] = w->packed[c->b];
        hdr[3 * ci + 2] = c->npts;
        if (fr) { fr[2 * ci] = c->friction; fr[2 * ci + 1] = c->restitution; }
        for (uint32_t p = 0; p < KZO_MAX_MANIFOLD; ++p) {
            float* o = pts + ((size_t)ci * KZO_MAX_MANIFOLD + p) * KZO_PT_FLOATS;
            if (p >= c->npts) { memset(o, 0, sizeof(float) * KZO_PT_FLOATS); continue; }
            const cpc_t* q = &c->p[p];
            put3(o, q->pA); put3(o + 3, q->pB); put3(o + 6, q->n); o[9] = q->sep;
            memcpy(&o[10], &q->feature, 4);
            put3(o + 11, q->rA); put3(o + 14, q->rB); put3(o + 17, q->laA); put3(o + 20, q->laB);
            put3(o + 23, q->t1); put3(o + 26, q->t2);
            o[29] = q->nm; o[30] = q->tm1; o[31] = q->tm2;
            o[32] = q->ni; o[33] = q->ti1; o[34] = q->ti2;
            o[35] = q->rbias; o[36] = q->pbias; o[37] = q->bimp; o[38] = q->nvel;
        }
    }
}

uint32_t kzo_num_active(const kzo_world* w) { return (uint32_t)w->nactive; }
void kzo_get_activity(const kzo_world* w, uint32_t* active_list, uint8_t* active_flags, float* sleep_timers) {
    if (active_list)
        for (int k = 0; k < w->nactive; ++k) active_list[k] = (uint32_t)w->active[k];
    if (active_flags) memcpy(active_flags, w->is_active, (size_t)w->nb);
    if (sleep_timers) memcpy(sleep_timers, w->sleep_timer, sizeof(float) * (size_t)w->nb);
}
uint32_t kzo_shared_sleepers(const kzo_world* w) { return w->st_shared_sleepers; }
/* PhysicsWorld::SetBodyActive (PhysicsWorld.cpp:108-111) for packed ids in order. */
void kzo_set_bodies_active(kzo_world* w, const uint32_t* ids, uint32_t n, int active) {
    for (uint32_t k = 0; k < n; ++k) {
        const int b = body_of(w, ids[k]);
        if (b < 0) continue;
        if (active) activate_body(w, b);
        else deactivate_body(w, b);
    }
}

/* PhysicsWorld's convenience body operations, in order (PhysicsWorld.cpp:109-205, Body.h:149-203):
 * SetBodyPosition/Rotation/Transform, SetLinear/AngularVelocity, AddForce(AtPoint), AddTorque,
 * AddImpulse(AtPoint), each followed by ActivateBody when `wake` is set; Activate/DeactivateBody.
 * The Apply* forms change dynamic bodies only; a stale id is skipped (GetBody returns nullptr). */
void kzo_edit_bodies(kzo_world* w, const kzo_body_edit* e, uint32_t n) {
    for (uint32_t k = 0; k < n; ++k) {
        const kzo_body_edit* d = &e[k];
        const int b = body_of(w, d->body);
        if (b < 0) continue;
        const int dyn = w->motion[b] == KZO_DYNAMIC;
        const v3 v0 = V(d->v[0], d->v[1], d->v[2]), v1 = V(d->v[3], d->v[4], d->v[5]);
        switch (d->op) {
            case KZO_EDIT_SET_POSITION: w->pos[b] = v0; break;
            case KZO_EDIT_SET_ROTATION:
                w->rot[b] = qnormalized(Q(d->v[0], d->v[1], d->v[2], d->v[3]));
                update_world_inertia(w, b);
                break;
            case KZO_EDIT_SET_TRANSFORM:
                w->pos[b] = v0;
                w->rot[b] = Q(d->v[3], d->v[4], d->v[5], d->v[6]);
                update_world_inertia(w, b);
                break;
            case KZO_EDIT_SET_LINEAR_VELOCITY: w->lv[b] = v0; break;
            case KZO_EDIT_SET_ANGULAR_VELOCITY: w->av[b] = v0; break;
            case KZO_EDIT_ADD_FORCE:
                if (dyn) w->force[b] = vadd(w->force[b], v0);
                break;
            case KZO_EDIT_ADD_FORCE_AT_POINT:
                if (dyn) {
                    w->force[b] = vadd(w->force[b], v0);
                    w->torque[b] = vadd(w->torque[b], vcross(vsub(v1, w->pos[b]), v0));
                }
                break;
            case KZO_EDIT_ADD_TORQUE:
                if (dyn) w->torque[b] = vadd(w->torque[b], v0);
                break;
            case KZO_EDIT_ADD_IMPULSE:
                if (dyn) w->lv[b] = vadd(w->lv[b], vmul(v0, w->inv_mass[b]));
                break;
            case KZO_EDIT_ADD_IMPULSE_AT_POINT:
                if (dyn) {
                    w->lv[b] = vadd(w->lv[b], vmul(v0, w->inv_mass[b]));
                    const v3 r = vsub(v1, w->pos[b]);
                    w->av[b] = vadd(w->av[b], mmulv(&w->iiw[b], vcross(r, v0)));
                }
                break;
            case KZO_EDIT_ACTIVATE: activate_body(w, b); continue;
            case KZO_EDIT_DEACTIVATE: deactivate_body(w, b); continue;
            default: continue;
        }
        if (d->wake) activate_body(w, b);
    }
}

void kzo_get_stats(const kzo_world* w, uint32_t* o) {
    o[0] = w->npairs; o[1] = w->ncons; o[2] = w->st_points; o[3] = w->st_islands;
    o[4] = w->st_batches; o[5] = w->st_max_vl; o[6] = w->st_max_bl; o[7] = w->st_max_isl_pts; o[8] = w->st_sum_vl;
    o[9] = w->st_max_open;
    o[10] = w->st_max_iters; o[11] = w->st_pt_iters;
    memcpy(&o[12], &w->st_final_res, sizeof(float));
}

void kzo_get_mass(const kzo_world* w, float* im, float* iw) {
    for (int i = 0; i < w->nb; ++i) {
        im[i] = w->inv_mass[i];
        for (int c = 0; c < 3; ++c) { iw[9 * i + 3 * c] = w->iiw[i].c[c].x; iw[9 * i + 3 * c + 1] = w->iiw[i].c[c].y; iw[9 * i + 3 * c + 2] = w->iiw[i].c[c].z; }
    }
}

uint32_t kzo_collide_bodies(const kzo_world* w, uint32_t a, uint32_t b, float max_sep, float* out) {
    kzo_manifold m;
    uint32_t n = kzo_collide(&w->shapes[w->shape[a]], w->rot[a], w->pos[a], &w->shapes[w->shape[b]], w->rot[b],
                             w->pos[b], max_sep, 1.0e-4f, &m);
    for (uint32_t i = 0; i < m.n; ++i) {
        float* o = out + 11 * i;
        put3(o, m.pts[i].pA); put3(o + 3, m.pts[i].pB); put3(o + 6, m.pts[i].n); o[9] = m.pts[i].sep;
        memcpy(&o[10], &m.pts[i].feature, 4);
    }
    (void)n;
    return m.n;
}
