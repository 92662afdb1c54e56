// kzg_ctx.h - internal state of one kzg context (not part of the C-ABI).
//
// Device layout (slot order = BodyID index order, reference BodyManager::mBodies):
//   bodies   : float4 SoA - pos, rot, lin/ang velocity, split-impulse pseudo velocities,
//              force/torque accumulators, world/local inverse inertia as 3 float4 columns,
//              two float4 parameter packs; u32 SoA for shape, motion, flags, layer, mask,
//              world, packed id.  One float4 load per vector keeps pair gathers coalesced.
//   pairs    : uint2 (slot A, slot B) in broad-phase order, + u64 MakePairKey per pair.
//   manifold : per pair a count and 4 contact points (pA|sep, pB|feature, n).
//   rows     : per constraint 4 point rows (stride 4), SoA float4 fields.
//   cache    : open-addressing table keyed by the u64 pair key, entries never evicted
//              (the reference keeps every entry forever, PhysicsWorld.cpp:418-452).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/kzg.h"
#include "kzg_narrow.cuh"

namespace kzg {

struct DeviceBodies {
    float4 *pos, *rot, *lv, *av, *plv, *pav, *force, *torque;
    float4 *iiw, *iil;    // 3 columns per body
    float4 *prm0, *prm1;  // (linDamp, angDamp, gravityFactor, maxLin), (maxAng, friction, restitution, ccdMotionThreshold)
    float* inv_mass;
    uint32_t *shape, *motion, *flags, *layer, *mask, *world, *packed;
    float4 *aabb_mn, *aabb_mx;
    float4 *fat_mn, *fat_mx;  // broad-phase fat bounds (DynamicAABBTree leaves, BroadPhase.cpp:35-75)
    uint32_t* act;     // 1: ActivationState::Active (every body is active while sleeping is off)
    float* sleep_t;    // MotionProperties::sleepTimer
    uint32_t* isl_idx; // Body::mIslandIndex: compact island index or active-list position, stale while asleep
    uint32_t* apos;    // position in the active list (kNone while asleep)
};

struct DeviceRows {  // per point row, index = 4 * constraint + point
    float4 *pA, *pB, *n;       // pA.w = separation, pB.w = feature (bits), n.w = combinedRestitution
    float4 *t1, *t2;           // t1.w = combinedFriction
    float4 *rA, *rB;           // world offsets used by the warm start (pointOnA - posA)
    float4 *rAr, *rBr;         // Rotate(localAnchor): offsets used by the velocity/bias solves
    float4 *laA, *laB;         // local anchors (exported only)
    float4 *mass;              // normalMass, tangentMass1, tangentMass2, -
    float4 *imp;               // normalImpulse, tangentImpulse1, tangentImpulse2, biasImpulse
    float4 *bias;              // restitutionBias, positionBias, normalVelocity, -
};

struct Counters {  // device-side counters, copied back after each stage that sizes the next
    uint32_t npairs;
    uint32_t ncons;
    uint32_t nislands;
    uint32_t batches;
    uint32_t max_vlev;
    uint32_t max_blev;
    uint32_t error;
    uint32_t npoints;
    uint32_t nsmall;
    uint32_t nlarge;
    uint32_t nepa;
    uint32_t epa_next;   // next deferred pair for the EPA warps
    uint32_t max_iters;  // most velocity iterations of an island
    uint32_t pt_iters;   // sum of batched points x iterations
    uint32_t res_bits;   // largest final residual (float bits, >= 0)
    uint32_t nmiss;      // contact points without a cached warm start (learned warm start / logging)
    uint32_t njisl;      // islands holding joints
    uint32_t nx_sched_w, nx_sched_c, nx_solve_w, nx_solve_c;  // largest-first island order: next island to take
    uint32_t nroots;     // islands as the reference counts them: every dynamic body's union-find root
    uint32_t ndyn;       // active dynamic bodies (BuildIslands' compact index range)
    uint32_t nsleep_n;   // active-list length when the sleeping pass began
    uint32_t sleep_islands;  // WorldStats::numIslands as the sleeping pass counts it
    uint32_t cache_entries;  // persists across steps
    uint32_t frame;          // step counter, advanced on the device by k_begin_step
    uint32_t nact;           // active-list length (persists)
};

// Learned warm start (kzg_mlp.cu): model, optimiser state, training log and dataset.
struct MlpState {
    bool have = false, enabled = false, logging = false;
    float blend_n = 1.0f, blend_t = 1.0f;  // fractions of the normal / tangent predictions used
    float tau = 0.0f;                      // training loss: 0 squared error, else pinball of this quantile
    float* theta = nullptr;  // KZG_MLP_PARAMS fp32 parameters
    float *adam_m = nullptr, *adam_v = nullptr;
    uint32_t adam_t = 0;
    float* grad = nullptr;  // KZG_MLP_PARAMS + loss
    float* norm = nullptr;  // feature mean[24], 1/std[24]
    std::vector<float> std;
    uint32_t* log_n = nullptr;
    float* log = nullptr;  // KZG_MLP_LOG_FLOATS per sample
    uint32_t log_cap = 0;
    float* ds = nullptr;  // training samples, same layout as the log
    uint32_t ds_n = 0;
    std::vector<double> ds_valid_prefix;
    float* part = nullptr;  // per-CTA partial gradients
    uint32_t part_blocks = 0;
    float* out = nullptr;
    uint32_t out_cap = 0;
};

struct JointDev;  // kzg_joint.cuh

constexpr uint32_t kDefaultWaitLimit = 1u << 26;

struct Ctx {
    kzg_config cfg{};
    kzg_world_settings ws{};
    kzg_solver_settings ss{};
    std::string err;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;

    // host mirrors needed for launches
    uint32_t nbodies = 0, nshapes = 0, nlarge = 0;
    float cell_size = 1.0f;
    bool shapes_uploaded = false;

    // shapes
    ShapeDev* shapes = nullptr;
    float4* hull_verts = nullptr;
    uint8_t* face_sizes = nullptr;
    uint32_t* face_idx = nullptr;

    DeviceBodies b{};
    uint32_t* large_list = nullptr;  // slots of bodies that bypass the grid (planes), grouped by world
    uint32_t* large_off = nullptr;   // per world: range in large_list (nworlds + 1 entries)
    uint32_t nworlds = 0;
    uint8_t* is_large = nullptr;

    // broad phase
    unsigned long long* cell_keys = nullptr;
    unsigned long long* cell_keys_sorted = nullptr;
    uint32_t* cell_vals = nullptr;
    uint32_t* cell_vals_sorted = nullptr;
    unsigned long long* pair_keys = nullptr;
    unsigned long long* pair_keys_sorted = nullptr;
    uint2* pairs = nullptr;

    // narrow phase
    uint32_t* m_count = nullptr;
    float4* m_data = nullptr;  // 12 float4 per pair
    unsigned long long* m_key = nullptr;
    uint32_t* epa_list = nullptr;  // pairs whose narrow phase needs EPA (warp pass)
    void* epa_gjk = nullptr;       // their GJK results from the thread pass (epa_gjk_cap records)
    uint32_t epa_gjk_cap = 0;
    float4* ccd_disp = nullptr;    // continuous collision: each LinearCast body's step displacement
    uint32_t* ccd_list = nullptr;  // slots of the LinearCast bodies, ascending
    uint32_t* ccd_state = nullptr; // per body slot: CCD round that finished it (LinearCast bodies)
    uint32_t *ccd_deps = nullptr, *ccd_ndeps = nullptr;  // per LinearCast body: predecessors (8 max), count
    uint32_t nccd = 0;
    // joints (kzg_joint.cuh): records, creation staging, per-step island grouping
    JointDev* joints = nullptr;
    kzg_joint_desc* joint_stage = nullptr;
    unsigned long long *jkeys = nullptr, *jkeys_sorted = nullptr;  // island root << 32 | joint index
    uint2* jisl = nullptr;           // per joint island: range in jkeys_sorted
    uint32_t* jisl_cisl = nullptr;   // per joint island: its contact island, or ~0
    uint32_t* jflag = nullptr;       // per contact island: 1 when a joint island owns it
    uint32_t njoints = 0;

    // constraints
    uint32_t* con_flag = nullptr;    // per pair: 1 if it makes a constraint
    uint32_t* con_index = nullptr;   // per pair: exclusive scan of con_flag
    uint32_t *con_pair = nullptr, *con_a = nullptr, *con_b = nullptr, *con_np = nullptr, *con_bits = nullptr;
    float2* con_fr = nullptr;
    unsigned long long* con_key = nullptr;
    DeviceRows r{};

    // islands and schedule
    uint32_t* uf = nullptr;
    uint32_t* isl_key = nullptr;
    uint32_t* isl_key_sorted = nullptr;
    uint32_t* isl_con_in = nullptr;
    uint32_t* isl_con = nullptr;      // constraints grouped by island, ascending within each
    uint32_t* isl_head = nullptr;
    uint32_t* isl_start = nullptr;    // nislands + 1
    uint32_t* isl_pts = nullptr;      // first point slot of each island in the level lists
    uint32_t* lvl_count = nullptr;    // per island level counters (4*ncons + nislands + 1)
    uint4* brec = nullptr;            // batch records, 64 B each (4*ncons + nislands + 1)
    float4* pk = nullptr;             // packed velocity items of cluster islands (kPackArrays x pk_cap per cluster)
    uint32_t pk_cap = 0;
    uint32_t* cl_ids = nullptr;       // local-id scratch of cluster islands (cluster_id_words)
    uint32_t* last_g = nullptr;       // level tables that do not fit shared memory (3 x 2*ncons)
    uint32_t *first_w = nullptr, *first_b = nullptr;  // per sorted constraint: first warm / bias level
    uint32_t* lvl_tmp = nullptr;      // per point: velocity level (batch order)
    uint32_t* ids_tmp = nullptr;      // per point: velocity item row (batch order)
    uint32_t *wl_list = nullptr, *vl_list = nullptr, *bl_list = nullptr;   // per island point lists by level
    uint32_t *wl_off = nullptr, *vl_off = nullptr, *bl_off = nullptr;      // level offsets
    uint32_t* isl_meta = nullptr;     // per island: warm / velocity / bias level counts, dynamic bodies
    uint32_t *body_stamp = nullptr, *body_loc = nullptr;       // per body scratch
    uint32_t* isl_bodies = nullptr;                             // per island dynamic bodies
    uint32_t *con_la = nullptr, *con_lb = nullptr;             // per constraint local body indices
    uint32_t *isl_small = nullptr, *isl_large = nullptr;       // islands by solve kernel
    uint32_t* isl_order = nullptr;   // largest-first island order (KZG_ISLANDS_LARGEST_FIRST)
    // sleeping: the active list (BodyManager::mActiveBodies; the buffer keeps values past its end, as
    // the reference's swap-removal does) and per-step scratch
    uint32_t* alist = nullptr;
    uint32_t *node = nullptr, *dyn2slot = nullptr, *act_flag = nullptr, *act_scan = nullptr;
    uint32_t *suf = nullptr, *smin = nullptr, *smark = nullptr, *root_mark = nullptr;
    uint32_t* ccd_rank_keys = nullptr;  // continuous collision in active-list order
    uint32_t *ccd_sorted = nullptr, *ccd_keys_sorted = nullptr;
    uint32_t* isl_bins = nullptr;    // its 32 size bins: counts, then cursors (64 words)
    uint32_t* miss_rows = nullptr;                              // rows without a cached warm start
    float4* miss_prior = nullptr;  // per miss: nearest cached point's impulses, pair's cached normal impulse per point
    MlpState mlp;

    // manifold cache: open addressing over cache_cap slots (a power of two), doubled between steps
    // when the coming steps could take it past 0.7 load (PhysicsWorld::GetOrCreateCached grows at
    // the same load); never evicted
    unsigned long long* c_key = nullptr;
    uint32_t* c_np = nullptr;
    float4* c_pos = nullptr;
    float4* c_imp = nullptr;
    uint32_t cache_cap = 0;
    bool all_active = true;  // every body in the active list (false once a call may have deactivated one)
    bool sleep_count_pending = false;  // the last step's UpdateSleeping island count is still to be counted
    bool cache_fixed = false;  // the tuner holds a copy of the table: no growth while it runs

    // misc
    Counters* dcnt = nullptr;
    Counters* hcnt = nullptr;  // pinned
    void* cub_tmp = nullptr;
    size_t cub_tmp_bytes = 0;
    unsigned long long* hash_words = nullptr;
    cudaEvent_t ev[8] = {};
    kzg_stats stats{};
    uint32_t frame = 0;
    uint32_t launches = 0;

    // launch-shape choices (kzg_set_tuning / kzg_autotune); every choice gives identical results
    kzg_tuning tune{128u, 384u, 0.0f, KZG_ISLANDS_IN_ORDER};
    uint32_t wait_limit = kDefaultWaitLimit;  // polls of the bounded in-kernel waits (kzg_set_wait_limit)

    // CUDA graph of one canonical step (kzg_set_graph); recaptured when dt or the configuration changes
    bool use_graph = false, graph_dirty = true, capturing = false;
    float graph_dt = 0.0f;
    cudaGraphExec_t graph_exec = nullptr;
    uint32_t graph_launches = 0;
};

}  // namespace kzg
