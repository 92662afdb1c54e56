/* Oracle API (test infrastructure only).
 *
 * A plain-C restatement of the reference's per-step contact pipeline
 * (PhysicsWorld::StepFixed, src/World/PhysicsWorld.cpp:245-329) used as the checker for the
 * GPU path: tests compare the CUDA library against it, and bench.py's CPU baseline times it.
 * It is pinned against the reference itself through the traces written by ref_trace.cpp
 * (tests/golden/).  The product never links, loads or includes anything under oracle/.
 */
#ifndef KZO_H
#define KZO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kzo_world kzo_world;

/* Pair sources for the broad phase. */
enum {
    KZO_PAIRS_TREE = 0,      /* the reference's dynamic AABB tree (BroadPhase.cpp), reference order */
    KZO_PAIRS_CANONICAL = 1, /* every overlapping pair, sorted by MakePairKey (lower packed id first) */
    KZO_PAIRS_EXTERNAL = 2   /* pairs supplied with kzo_set_external_pairs */
};

#define KZO_PT_FLOATS 39   /* floats per exported contact point (see kzo_get_constraints) */
#define KZO_STATE_FLOATS 13 /* pos3 rot4 linvel3 angvel3 */

/* scene: KZSC bytes; resolved: per hull shape (u32 nv, f32[3nv], u32 nf, u8[nf] padded to 4,
 * u32 ni, u32[ni]) followed by per body (f32 invMass, f32 invInertiaLocal[9] column-major). */
kzo_world* kzo_create(const uint8_t* scene, size_t scene_len, const uint8_t* resolved, size_t resolved_len);
void kzo_destroy(kzo_world* w);
const char* kzo_error(void);

void kzo_set_threads(kzo_world* w, int threads);
void kzo_set_pair_mode(kzo_world* w, int mode);
int kzo_set_external_pairs(kzo_world* w, const uint32_t* packed_pairs, uint32_t n);
void kzo_set_schedule_stats(kzo_world* w, int enabled);
/* Residual-terminated velocity iterations (not in the reference, which always runs the fixed
 * count): tol > 0 stops an island's iterations once the relative impulse change of an iteration,
 * sum|dImpulse| / sum|impulse| over its batched points (2^-20 N s fixed-point sums), is <= tol,
 * after at most cap iterations; tol = 0 restores the fixed count. */
void kzo_set_residual(kzo_world* w, float tol, uint32_t cap);
/* Joint trigonometry: 0 (default) the C library's float sinf/cosf/acosf/atan2f, as the reference
 * calls them; 1 the double-precision functions rounded to float, as the GPU evaluates them. */
void kzo_set_trig_mode(kzo_world* w, int mode);
/* 1: the manifold cache uses a 64-bit mixed slot function instead of the reference's (pa ^ pb) & mask.
 * Results are identical (entries are found by key and never evicted); large worlds avoid the
 * reference's clustered probe runs. */
void kzo_set_cache_hash(kzo_world* w, int mixed);
/* Sleeping state: the active list in order (kzo_num_active entries), per-body activity flags and
 * sleep timers (each pointer may be NULL). */
uint32_t kzo_num_active(const kzo_world* w);
void kzo_get_activity(const kzo_world* w, uint32_t* active_list, uint8_t* active_flags, float* sleep_timers);
/* Sleeping bodies whose contacts were assigned to two different islands in the last step. */
uint32_t kzo_shared_sleepers(const kzo_world* w);
/* PhysicsWorld::SetBodyActive for each packed id in order (stale ids skipped). */
void kzo_set_bodies_active(kzo_world* w, const uint32_t* ids, uint32_t n, int active);
/* PhysicsWorld's convenience body operations in order; the layout and op numbers are those of the
 * GPU library's kzg_body_edit. */
enum {
    KZO_EDIT_SET_POSITION, KZO_EDIT_SET_ROTATION, KZO_EDIT_SET_TRANSFORM, KZO_EDIT_SET_LINEAR_VELOCITY,
    KZO_EDIT_SET_ANGULAR_VELOCITY, KZO_EDIT_ADD_FORCE, KZO_EDIT_ADD_FORCE_AT_POINT, KZO_EDIT_ADD_TORQUE,
    KZO_EDIT_ADD_IMPULSE, KZO_EDIT_ADD_IMPULSE_AT_POINT, KZO_EDIT_ACTIVATE, KZO_EDIT_DEACTIVATE
};
typedef struct {
    uint32_t op, body, wake, reserved;
    float v[8];
} kzo_body_edit;
void kzo_edit_bodies(kzo_world* w, const kzo_body_edit* edits, uint32_t n);

int kzo_step(kzo_world* w, float dt);

uint32_t kzo_num_bodies(const kzo_world* w);
void kzo_get_state(const kzo_world* w, float* out);      /* KZO_STATE_FLOATS per body, slot order */
void kzo_set_state(kzo_world* w, const float* in);
uint64_t kzo_hash(const kzo_world* w);                    /* PhysicsWorld::ComputeStateHash */

uint32_t kzo_num_pairs(const kzo_world* w);
void kzo_get_pairs(const kzo_world* w, uint32_t* out);    /* 2 packed ids per pair, step order */
uint32_t kzo_num_constraints(const kzo_world* w);
/* hdr: 3 u32 per constraint (packed A, packed B, numPoints); pts: 8*KZO_PT_FLOATS per constraint:
 * pA3 pB3 n3 sep feature(bits) rA3 rB3 localA3 localB3 t1_3 t2_3 nMass t1Mass t2Mass
 * nImp t1Imp t2Imp restitutionBias positionBias biasImpulse normalVelocity */
void kzo_get_constraints(const kzo_world* w, uint32_t* hdr, float* pts, float* fric_rest);
/* pairs, constraints, points, islands, batches, max velocity levels, max bias levels,
 * largest island points, sum of velocity levels over islands, most batches open at once,
 * most velocity iterations of an island, sum over islands of batched points x iterations,
 * largest final residual (float bits) */
void kzo_get_stats(const kzo_world* w, uint32_t* out13);
void kzo_get_mass(const kzo_world* w, float* inv_mass, float* inv_inertia_world /*9 per body*/);

/* Narrow phase between two bodies at their current poses (A = first argument). Returns the
 * number of points; out gets 11 floats per point: pA3 pB3 n3 sep feature. */
uint32_t kzo_collide_bodies(const kzo_world* w, uint32_t slot_a, uint32_t slot_b, float max_sep, float* out);

#ifdef __cplusplus
}
#endif
#endif
