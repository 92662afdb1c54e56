/* kzg.h - C-ABI of the GB300-native contact pipeline (libkzg.so).
 *
 * This is the drop-in boundary for the reference's per-step pipeline behind
 * PhysicsWorld::Step / StepFixed (reference: include/Kizuri/World/PhysicsWorld.h:82-239,
 * src/World/PhysicsWorld.cpp:245-329).  The reference has no FFI of its own; every entry point
 * below replaces one piece of its C++ API, cited beside it, and keeps that piece's argument
 * meaning.  Plain pointers and sizes only; every call returns a kzg_status and records a
 * message retrievable with kzg_last_error().  One context = one device-resident world (or a
 * batch of independent worlds), owned by one host thread, running on one CUDA stream.
 *
 * Body state (positions, quaternions, velocities, inverse mass and inertia) and the manifold
 * cache stay resident in device memory between steps.  There is no CPU fallback: when no
 * suitable GPU is present, kzg_create fails with KZG_ERR_CUDA.
 */
#ifndef KZG_H
#define KZG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kzg_ctx kzg_ctx;
typedef int kzg_status;

#define KZG_OK 0
#define KZG_ERR_INVALID (-1)     /* bad argument or call order */
#define KZG_ERR_CUDA (-2)        /* CUDA runtime failure or no usable device */
#define KZG_ERR_CAPACITY (-3)    /* a device table or buffer is full; raise the kzg_config limit */
#define KZG_ERR_UNSUPPORTED (-4) /* feature outside the accelerated path (e.g. the scalar solver) */
#define KZG_ERR_DEVICE (-5)      /* a kernel raised its error word (see kzg_stats.device_error) */

/* Shape types: numbering of ShapeType (reference include/Kizuri/Geometry/Shape.h:13-25). */
#define KZG_SHAPE_SPHERE 0
#define KZG_SHAPE_BOX 1
#define KZG_SHAPE_CAPSULE 2
#define KZG_SHAPE_HULL 4
#define KZG_SHAPE_PLANE 8

/* Motion types: MotionType (reference include/Kizuri/Body/Body.h:37-41). */
#define KZG_MOTION_STATIC 0
#define KZG_MOTION_KINEMATIC 1
#define KZG_MOTION_DYNAMIC 2

#define KZG_BODY_SENSOR 1u         /* BodySettings::isSensor */
#define KZG_BODY_ALLOW_SLEEPING 2u /* BodySettings::allowSleeping */
#define KZG_BODY_LINEAR_CAST 4u    /* BodySettings::motionQuality = MotionQuality::LinearCast (Body.h:46-67) */

/* Broad-phase pair order of kzg_step (production mode). */
#define KZG_PAIRS_CANONICAL 0 /* every overlapping pair, sorted by MakePairKey (PhysicsWorld.cpp:13-18) */

/* Solver schedules. */
#define KZG_SCHEDULE_REFERENCE 0 /* the reference's greedy 4-wide batches (PhysicsWorld.cpp:680-717): bit-exact */

/* Device capacities, fixed at creation (no reallocation while stepping). */
typedef struct {
    uint32_t max_bodies;
    uint32_t max_shapes;
    uint32_t max_hull_vertices;
    uint32_t max_hull_indices;
    uint32_t max_pairs;         /* broad-phase pairs per step */
    uint32_t max_cache_entries; /* initial manifold cache slots (power of two).  Entries are never
                                 * evicted; like PhysicsWorld::GetOrCreateCached's table, this one
                                 * doubles (entries rehashed, results unchanged) between steps once the
                                 * coming steps could take it past 0.7 load */
    int device;                 /* CUDA ordinal */
    uint32_t max_joints;        /* joints (0: none) */
} kzg_config;

/* Mirrors SolverSettings (reference include/Kizuri/Solver/ContactSolver.h:67-82). */
typedef struct {
    uint32_t velocity_iterations;
    uint32_t position_iterations;
    float baumgarte;
    float penetration_slop;
    float restitution_threshold;
    float max_bias_velocity;
    float warm_start_factor;
    int use_velocity_bias;
    int schedule; /* KZG_SCHEDULE_* */
    /* Residual-terminated velocity iterations (not in the reference, which always runs
     * velocity_iterations).  The residual of one velocity iteration of an island is its relative
     * impulse change: the sum over the island's batched contact points of |dImpulse| of the
     * friction 1, friction 2 and normal rows in that iteration, divided by the sum over the same
     * points of |normalImpulse| + |tangentImpulse1| + |tangentImpulse2| after it (both sums taken
     * in 2^-20 N s fixed point, so they do not depend on the order of the additions; dimensionless).
     * With residual_tolerance > 0 an island stops iterating once its residual is <=
     * residual_tolerance, after at most max_velocity_iterations iterations.  0 keeps the
     * reference's fixed count. */
    float residual_tolerance;
    uint32_t max_velocity_iterations;
    /* SolverSettings::useSplitImpulse (ContactSolver.h:75).  The reference declares it but reads it
     * nowhere: the split-impulse bias pass runs whenever use_velocity_bias is 0.  Both values are
     * accepted and behave the same, as in the reference. */
    int use_split_impulse;
    /* SolverSettings::useSIMDSolver (ContactSolver.h:77): 1 solves the velocity iterations over the
     * reference's 4-wide first-fit batches (PhysicsWorld.cpp:677-722) with SolveVelocityBatchSIMD's
     * lane math; 0 takes the scalar path, SolveVelocityConstraint over every constraint in island
     * order (PhysicsWorld.cpp:723-729, ContactSolver.cpp:136-188).  Both are bit-exact. */
    int use_simd_solver;
} kzg_solver_settings;

/* Mirrors the WorldSettings fields the step reads (reference PhysicsWorld.h:20-43). */
typedef struct {
    float gravity[3];
    float fixed_timestep;   /* used for the broad-phase displacement, PhysicsWorld.cpp:342 */
    int allow_sleeping;     /* WorldSettings::allowSleeping (default 1, as in the reference) */
    int warm_start;         /* 0 reproduces the reference's KZ_NOWS switch (PhysicsWorld.cpp:493) */
    int use_ccd;            /* WorldSettings::useCCD: clamp LinearCast bodies' motion (PhysicsWorld.cpp:785-852) */
    float ccd_max_penetration; /* WorldSettings::ccdMaxPenetration */
    /* WorldSettings::sleepTimeThreshold (s), sleepLinearThreshold (m/s), sleepAngularThreshold
     * (rad/s) (PhysicsWorld.h:25-27), read by the sleeping pass when allow_sleeping is set. */
    float sleep_time_threshold;
    float sleep_linear_threshold;
    float sleep_angular_threshold;
} kzg_world_settings;

/* One shape. params: sphere {r}; box {hx,hy,hz}; capsule {halfHeight, radius}
 * (CapsuleShape(halfHeight, radius), Shape.h:206); plane {nx,ny,nz,d}.  Hulls reference a
 * range of the vertex / face-size / face-index pools given to kzg_upload_shapes. */
typedef struct {
    uint32_t type;
    float params[4];
    uint32_t first_vertex, num_vertices;
    uint32_t first_face, num_faces;
    uint32_t first_index, num_indices;
} kzg_shape_desc;

/* Bodies in creation order (reference BodyManager::CreateBody, src/Body/BodyManager.cpp:15-61).
 * Arrays of n entries; vectors packed xyz / xyzw; inertia 9 floats column-major.  inv_mass and
 * inv_inertia_local are the resolved mass properties (kzg_mass_properties). world_id separates
 * independent worlds stepped together (pairs never cross worlds); 0 for a single world. */
typedef struct {
    const uint32_t* shape;
    const uint32_t* motion;
    const uint32_t* flags;
    const float* position;
    const float* rotation;
    const float* linear_velocity;
    const float* angular_velocity;
    const float* friction;
    const float* restitution;
    const float* linear_damping;
    const float* angular_damping;
    const float* gravity_factor;
    const float* max_linear_velocity;
    const float* max_angular_velocity;
    const float* inv_mass;
    const float* inv_inertia_local;
    const uint32_t* object_layer;
    const uint32_t* collision_mask;
    const uint32_t* world_id; /* may be NULL */
    /* BodySettings::ccdMotionThreshold (Body.h:70; may be NULL = 0): a LinearCast body whose step
     * displacement is shorter than a positive threshold is not clamped (PhysicsWorld.cpp:807). */
    const float* ccd_motion_threshold;
} kzg_body_soa;

/* Counters of the last step (reference WorldStats, PhysicsWorld.h:66-77, with honest stage
 * labels) plus device-side diagnostics. */
typedef struct {
    uint32_t num_bodies;
    uint32_t num_broadphase_pairs;
    uint32_t num_contact_constraints;
    uint32_t num_contact_points;
    uint32_t num_islands;
    uint32_t num_batches;
    uint32_t max_velocity_levels;
    uint32_t max_bias_levels;
    uint32_t cache_entries;
    uint32_t device_error;  /* bit mask of KZG_DEVERR_* raised by kernels */
    uint32_t kernel_launches; /* kernels launched by the last step (own kernels + CUB passes) */
    uint32_t max_velocity_iterations_used;  /* most velocity iterations any island ran */
    uint32_t point_velocity_iterations;     /* sum over islands of batched points x iterations */
    /* CUDA-event times of the last step on the context stream: broad phase; narrow-phase kernel;
     * constraint build + velocity integration; prepare + islands + batch schedule; solver kernel;
     * cache store + position integration; whole step. */
    float broadphase_ms, narrowphase_ms, constraints_ms, schedule_ms, solve_ms, integrate_ms, step_ms;
    float final_residual; /* largest residual (relative impulse change, see kzg_solver_settings) of any
                           * island's last velocity iteration */
    uint32_t num_active_bodies; /* WorldStats::numActiveBodies: the active list's length */
    uint32_t cache_capacity;    /* manifold cache slots now (kzg_config.max_cache_entries, doubled as it fills) */
    uint32_t num_epa_pairs;     /* pairs of the last step that needed EPA (overlapping convex pairs) */
} kzg_stats;

#define KZG_DEVERR_PAIRS 1u     /* pair buffer overflow */
#define KZG_DEVERR_CACHE 2u     /* cache table full */
#define KZG_DEVERR_EPA 4u       /* EPA polytope exceeded its face capacity */
#define KZG_DEVERR_MANIFOLD 8u  /* a manifold produced more than 4 points */
/* A bounded wait between the warps of a kernel gave up.  The waiting warp's work is then redone
 * by its CTA after the wait, so the step completes with the same result: the bit is reported in
 * kzg_stats.device_error and the step still returns KZG_OK. */
#define KZG_DEVERR_WAIT 16u
/* A tensor-core wait of the learned warm start gave up: the tiles it was running got no
 * prediction (their points keep the plain warm start) and the call returns KZG_ERR_DEVICE. */
#define KZG_DEVERR_MMA 32u

/* ---- lifecycle (PhysicsWorld ctor/dtor, PhysicsWorld.cpp:64-78) ----------------------------- */
kzg_status kzg_create(const kzg_config* cfg, kzg_ctx** out);
kzg_status kzg_destroy(kzg_ctx* ctx);
const char* kzg_last_error(const kzg_ctx* ctx); /* ctx may be NULL: last creation error */
/* All work is issued on this stream (cudaStream_t passed as void*; NULL = the context's own). */
kzg_status kzg_set_stream(kzg_ctx* ctx, void* stream);
kzg_status kzg_synchronize(kzg_ctx* ctx);

/* ---- settings (PhysicsWorld::GetSettings, PhysicsWorld.h:91-95) ----------------------------- */
kzg_status kzg_set_world_settings(kzg_ctx* ctx, const kzg_world_settings* s);
kzg_status kzg_set_solver_settings(kzg_ctx* ctx, const kzg_solver_settings* s);
void kzg_default_settings(kzg_world_settings* ws, kzg_solver_settings* ss);

/* ---- scene setup (PhysicsWorld::CreateBody, PhysicsWorld.cpp:83-93) ------------------------- */
kzg_status kzg_upload_shapes(kzg_ctx* ctx, const kzg_shape_desc* shapes, uint32_t num_shapes,
                             const float* hull_vertices, uint32_t num_vertices, const uint8_t* face_sizes,
                             uint32_t num_faces, const uint32_t* face_indices, uint32_t num_indices);
/* Appends bodies; *first_slot receives the slot (BodyID index) of the first one. */
kzg_status kzg_add_bodies(kzg_ctx* ctx, uint32_t n, const kzg_body_soa* bodies, uint32_t* first_slot);

/* ---- joints (Constraints.h:41-277, PhysicsWorld::AddConstraint, PhysicsWorld.cpp:210-212) --- */
#define KZG_JOINT_POINT 0u    /* PointConstraint */
#define KZG_JOINT_DISTANCE 1u /* DistanceConstraint */
#define KZG_JOINT_FIXED 2u    /* FixedConstraint */
#define KZG_JOINT_HINGE 3u    /* HingeConstraint */
#define KZG_JOINT_SLIDER 4u   /* SliderConstraint */
#define KZG_JOINT_SIXDOF 5u   /* SixDOFConstraint */
#define KZG_JOINT_DISABLED 1u      /* Constraint::SetEnabled(false) */
#define KZG_JOINT_LIMITS 2u        /* Hinge/SliderConstraint::SetLimits(lower, upper) */
#define KZG_JOINT_MOTOR 4u         /* Hinge/SliderConstraint::SetMotor(motor_target, motor_max) */
#define KZG_JOINT_LOCAL_ANCHORS 8u /* PointConstraint(a, b, localAnchorA = anchor_a, localAnchorB = anchor_b) */
/* One joint as the reference's constructors take it: anchors and axes in world space at the
 * bodies' poses when kzg_add_joints is called.  anchor_b: DistanceConstraint's second anchor;
 * axis_b: HingeConstraint's axis on B; rotation (x, y, z, w): SixDOFConstraint's world frame;
 * axis_modes: 2 bits per axis (SixDOFConstraint::AxisMode; linear x, y, z in bits 0-5, angular in
 * bits 6-11); motor_mask: bit k = SetLinearMotor(k), bit 3+k = SetAngularMotor(k), with
 * six_motor = linear targets[3], linear max[3], angular targets[3], angular max[3]. */
typedef struct {
    uint32_t type, body_a, body_b, flags;
    float anchor_a[3], anchor_b[3], axis_a[3], axis_b[3], rotation[4];
    float distance, lower, upper, motor_target, motor_max;
    uint32_t axis_modes, motor_mask;
    float six_motor[12];
} kzg_joint_desc;
/* Appends joints (slots of existing bodies); *first_index receives the first one's index. */
kzg_status kzg_add_joints(kzg_ctx* ctx, uint32_t n, const kzg_joint_desc* joints, uint32_t* first_index);

/* ---- stepping (PhysicsWorld::StepFixed, PhysicsWorld.cpp:245-329) --------------------------- */
/* nsteps fixed steps with the GPU broad phase (canonical pair order). */
kzg_status kzg_step(kzg_ctx* ctx, float dt, uint32_t nsteps);
/* One step using the caller's broad-phase pairs, in order (2 packed BodyIDs per pair, host
 * memory).  With the reference's own pair list this reproduces the reference bit for bit. */
kzg_status kzg_step_with_pairs(kzg_ctx* ctx, const uint32_t* packed_pairs, uint32_t num_pairs, float dt);
/* Step kzg_step through a CUDA graph: one step is captured once (again after dt or any setting
 * changes) and kzg_step's nsteps steps are launched back to back with one synchronisation at the
 * end; stats then describe the last step, except that the stage times are 0 and step_ms is the
 * mean over the replayed steps.  No counterpart in the reference. */
kzg_status kzg_set_graph(kzg_ctx* ctx, int enabled);

/* Launch shapes of the island work, all bit-identical in result: islands with at most
 * small_island_constraints constraints (<= 128) get one warp for their schedule, islands with at
 * most warp_island_bodies dynamic bodies (<= 384) one warp for their solve, larger ones a CTA.
 * island_order is the island-to-CTA schedule: KZG_ISLANDS_IN_ORDER hands the islands to warps and
 * CTAs in island order with a fixed stride; KZG_ISLANDS_LARGEST_FIRST hands them out from a shared
 * counter, largest first (islands binned by the power of two of their constraint count), the
 * longest-processing-time-first rule that evens out the load of worlds of very uneven size.
 * kzg_autotune saves the world on the device, steps it steps_per_candidate steps from that same
 * state with each of a small set of choices, restores it, keeps the fastest choice (by CUDA-event
 * step time) and returns it: the world is left exactly as it was.  No counterpart in the
 * reference. */
#define KZG_ISLANDS_IN_ORDER 0u
#define KZG_ISLANDS_LARGEST_FIRST 1u
typedef struct {
    uint32_t small_island_constraints;
    uint32_t warp_island_bodies;
    float step_ms; /* out: mean step time of this choice during kzg_autotune */
    uint32_t island_order; /* KZG_ISLANDS_* */
} kzg_tuning;
kzg_status kzg_set_tuning(kzg_ctx* ctx, const kzg_tuning* t);
/* Poll limit of the bounded in-kernel waits (default 2^26 polls, over 8 s): past it a wait
 * gives up and raises KZG_DEVERR_WAIT (see above).  A small limit makes the give-up path run on
 * purpose, which is how it is tested; 0 restores the default.  No counterpart in the reference. */
kzg_status kzg_set_wait_limit(kzg_ctx* ctx, uint32_t polls);
kzg_status kzg_get_tuning(kzg_ctx* ctx, kzg_tuning* t);
kzg_status kzg_autotune(kzg_ctx* ctx, float dt, uint32_t steps_per_candidate, kzg_tuning* best);

/* ---- state access (Body getters/setters, Body.h:146-178) ------------------------------------ */
/* 13 floats per body in slot order: position xyz, rotation xyzw, linear xyz, angular xyz. */
kzg_status kzg_download_state(kzg_ctx* ctx, float* out, uint32_t first, uint32_t count);
kzg_status kzg_upload_state(kzg_ctx* ctx, const float* in, uint32_t first, uint32_t count);
/* 7 floats per body: position xyz + rotation xyzw (what a renderer reads each frame). */
kzg_status kzg_download_transforms(kzg_ctx* ctx, float* out, uint32_t first, uint32_t count);
/* Force and torque accumulators for the next step (Body::ApplyForce / ApplyTorque); 6 floats per
 * body (force xyz, torque xyz); cleared after every step like Body::ClearForces. */
kzg_status kzg_upload_forces(kzg_ctx* ctx, const float* force_torque, uint32_t first, uint32_t count);
kzg_status kzg_download_mass(kzg_ctx* ctx, float* inv_mass, float* inv_inertia_world);

/* ---- sleeping (WorldSettings::allowSleeping; UpdateSleeping, PhysicsWorld.cpp:866-951) --------
 * With allow_sleeping set, islands whose dynamic bodies stayed below the sleep thresholds for
 * sleep_time_threshold seconds are deactivated (velocities zeroed, removed from the active list),
 * and a sleeping dynamic body touched by a moving one is woken (PhysicsWorld.cpp:473-490), with the
 * reference's active-list order and island numbering.  One difference, by design: the reference
 * solves concurrently two islands that both hold a contact of one sleeping body whose island index
 * is stale past the active count (a race on that body's velocity); here such islands are joined and
 * solved as one, deterministically. */
/* PhysicsWorld::SetBodyActive / ActivateBody / DeactivateBody (PhysicsWorld.cpp:108-111, 132-133)
 * for each packed BodyID in order (stale ids skipped). */
kzg_status kzg_set_bodies_active(kzg_ctx* ctx, const uint32_t* packed_ids, uint32_t n, int active);
/* BodyManager::GetActiveBodyList (packed BodyIDs in active-list order); *count receives its length,
 * at most `capacity` ids are written. */
kzg_status kzg_get_active_bodies(kzg_ctx* ctx, uint32_t* packed_ids, uint32_t capacity, uint32_t* count);

/* ---- body edits between steps (PhysicsWorld convenience operations, PhysicsWorld.cpp:109-205) --
 * Applied in array order on the device, each exactly as the reference's method does it: the
 * Body::Apply* forms change dynamic bodies only (Body.h:181-203), SetRotation normalises the
 * quaternion and updates the world inverse inertia, and with `wake` set the body is then activated
 * (BodyManager::ActivateBody: appended to the active list if it was inactive).  Forces and torques
 * accumulate until the next step, which clears them (PhysicsWorld.cpp:312). */
#define KZG_EDIT_SET_POSITION 0u          /* v[0..2]: position (SetBodyPosition) */
#define KZG_EDIT_SET_ROTATION 1u          /* v[0..3]: quaternion x, y, z, w (SetBodyRotation) */
#define KZG_EDIT_SET_TRANSFORM 2u         /* v[0..2] position, v[3..6] quaternion, used as given (SetBodyTransform) */
#define KZG_EDIT_SET_LINEAR_VELOCITY 3u   /* v[0..2] (SetLinearVelocity) */
#define KZG_EDIT_SET_ANGULAR_VELOCITY 4u  /* v[0..2] (SetAngularVelocity) */
#define KZG_EDIT_ADD_FORCE 5u             /* v[0..2] at the centre (AddForce) */
#define KZG_EDIT_ADD_FORCE_AT_POINT 6u    /* v[0..2] force, v[3..5] world point (AddForceAtPoint) */
#define KZG_EDIT_ADD_TORQUE 7u            /* v[0..2] (AddTorque) */
#define KZG_EDIT_ADD_IMPULSE 8u           /* v[0..2] at the centre (AddImpulse) */
#define KZG_EDIT_ADD_IMPULSE_AT_POINT 9u  /* v[0..2] impulse, v[3..5] world point (AddImpulseAtPoint) */
#define KZG_EDIT_ACTIVATE 10u             /* ActivateBody (wake ignored) */
#define KZG_EDIT_DEACTIVATE 11u           /* DeactivateBody: velocities zeroed, swap-removed (wake ignored) */
typedef struct {
    uint32_t op;      /* KZG_EDIT_* */
    uint32_t body;    /* packed BodyID; a stale id is skipped, as GetBody's nullptr is */
    uint32_t wake;    /* the reference's `wake` argument (default true) */
    uint32_t reserved;
    float v[8];
} kzg_body_edit;
kzg_status kzg_edit_bodies(kzg_ctx* ctx, const kzg_body_edit* edits, uint32_t n);

/* ---- diagnostics (ComputeStateHash / GetStats / GetContactConstraints / GetPairs) ----------- */
kzg_status kzg_state_hash(kzg_ctx* ctx, uint64_t* out); /* PhysicsWorld.cpp:1145-1175 */
kzg_status kzg_get_stats(kzg_ctx* ctx, kzg_stats* out);
kzg_status kzg_num_pairs(kzg_ctx* ctx, uint32_t* n);
kzg_status kzg_download_pairs(kzg_ctx* ctx, uint32_t* packed_pairs, uint32_t capacity);
kzg_status kzg_num_constraints(kzg_ctx* ctx, uint32_t* n);
/* Per constraint: hdr 3 u32 (packed A, packed B, numPoints), fr 2 floats (friction, restitution),
 * pts 8*39 floats in the layout: pA3 pB3 n3 sep feature(bits) rA3 rB3 localA3 localB3 t1_3 t2_3
 * nMass t1Mass t2Mass nImp t1Imp t2Imp restitutionBias positionBias biasImpulse normalVelocity
 * (the fields of ContactPointConstraint, reference ContactSolver.h:13-43). */
kzg_status kzg_download_constraints(kzg_ctx* ctx, uint32_t* hdr, float* fr, float* pts, uint32_t capacity);

/* ComputeStateHash (PhysicsWorld.cpp:1145-1175) of body state in the caller's own device buffers,
 * allocating nothing on the host or the device.  No counterpart in the reference: it exists for
 * callers that must not allocate in their frame loop (lockstep games that compare state hashes
 * every tick, hosts whose device memory budget is fixed after start-up).
 *   state      device pointer, n x 13 floats per body in kzg_download_state's layout
 *   packed_ids device pointer, n BodyID::Packed values (slot order)
 *   stream     cudaStream_t to run on (NULL: the legacy default stream); the call synchronises it
 *   error      optional; receives a static message on failure
 * n above KZG_NOALLOC_HASH_MAX_BODIES returns KZG_ERR_CAPACITY.  The work runs in one fixed
 * 1.75 MiB device scratch array shared by all calls on a device: the first call on a device sets it
 * up (symbol lookup, module load) and should come before any stream capture, and calls that
 * overlap on one device race on the scratch - serialise them. */
#define KZG_NOALLOC_HASH_MAX_BODIES 16384
kzg_status kzg_state_hash_noalloc(const float* state, const uint32_t* packed_ids, uint32_t n, void* stream,
                                  uint64_t* out, const char** error);

/* ---- device snapshots (no counterpart in the reference) ---------------------------------------
 * Body state (positions, rotations, velocities, pseudo velocities, force accumulators, world
 * inverse inertia) and the occupied entries of the manifold cache, so that a context built from the
 * same bodies resumes bit-exactly where the snapshot was taken.  The reference's KZP1 files
 * (kizuriphysics3d_gb300/kzp1.py) carry bodies only: warm starting restarts from zero. */
kzg_status kzg_snapshot_size(kzg_ctx* ctx, size_t* bytes);
kzg_status kzg_snapshot_save(kzg_ctx* ctx, void* out, size_t capacity);
kzg_status kzg_snapshot_load(kzg_ctx* ctx, const void* in, size_t size);

/* ---- learned warm start ------------------------------------------------------------------------
 * No counterpart in the reference, which warm-starts a contact point that misses the manifold
 * cache with zero impulses (PhysicsWorld.cpp:518-529).  With a model set and enabled, such points
 * start from the prediction of an MLP (24 features -> 64 -> 64 -> 3, ReLU; BF16 weights and
 * activations, FP32 accumulation on the tensor cores).  Parameters: KZG_MLP_PARAMS floats,
 * row-major W1[64][24], b1[64], W2[64][64], b2[64], W3[3][64], b3[3]; features are standardised
 * with the given mean / std.  An output o maps to impulse / effective mass 0.05 sinh(o) (|o|
 * limited to 6) for the normal and the two tangent rows.  Training runs on the GPU too: log
 * samples (features + converged impulse / effective mass) while stepping, load them as a dataset
 * with the targets mapped through asinh(y / 0.05), take Adam steps. */
#define KZG_MLP_FEATURES 24
#define KZG_MLP_PARAMS 5955
#define KZG_MLP_LOG_FLOATS 30 /* per sample: 24 features, 3 targets, 3 target masks */
kzg_status kzg_mlp_set_params(kzg_ctx* ctx, const float* theta, const float* mean, const float* std);
kzg_status kzg_mlp_get_params(kzg_ctx* ctx, float* theta, float* mean, float* std);
kzg_status kzg_mlp_enable(kzg_ctx* ctx, int enabled);
/* Fractions in [0, 1] of the predicted normal and tangent impulses used as the warm start
 * (default 1, 1). */
kzg_status kzg_mlp_set_blend(kzg_ctx* ctx, float normal, float tangent);
/* Log every cache-missing contact point of the following steps (features before the solve,
 * impulse / effective mass after it) into a device buffer of `capacity` samples; 0 stops. */
kzg_status kzg_mlp_log_begin(kzg_ctx* ctx, uint32_t capacity);
kzg_status kzg_mlp_log_fetch(kzg_ctx* ctx, float* out, uint32_t capacity, uint32_t* count);
kzg_status kzg_mlp_set_dataset(kzg_ctx* ctx, const float* samples, uint32_t n); /* log layout */
/* Training loss: 0 (default) the squared error, tau in (0, 1) the pinball loss of quantile tau
 * (fits the tau-quantile of the target: below-median quantiles give conservative warm starts). */
kzg_status kzg_mlp_set_quantile(kzg_ctx* ctx, float tau);
/* Loss averaged over the valid targets of samples [first, first + count): its gradient
 * (no update), or one Adam step (beta 0.9 / 0.999). */
kzg_status kzg_mlp_gradient(kzg_ctx* ctx, uint32_t first, uint32_t count, float* grad, float* loss);
kzg_status kzg_mlp_train_step(kzg_ctx* ctx, uint32_t first, uint32_t count, float lr, float* loss);
kzg_status kzg_mlp_predict(kzg_ctx* ctx, uint32_t first, uint32_t count, float* out); /* 3 per sample */

/* ---- host-side setup helpers (no device needed) ---------------------------------------------- */
/* ConvexHullShape::Create (reference src/Geometry/Shapes.cpp:331-471): builds the hull of a point
 * cloud keeping the reference's vertex order.  Returns KZG_ERR_INVALID for degenerate clouds.
 * Output capacities: vertices max_points*3 floats, sizes/indices see kzg_hull_capacity. */
kzg_status kzg_hull_build(const float* points, uint32_t num_points, uint32_t max_points, float* out_vertices,
                          uint32_t* out_num_vertices, uint8_t* out_face_sizes, uint32_t* out_num_faces,
                          uint32_t* out_face_indices, uint32_t* out_num_indices, uint32_t capacity_faces);
/* BodyManager::RecomputeMassProperties (reference BodyManager.cpp:63-99) for one body. */
kzg_status kzg_mass_properties(const kzg_shape_desc* shape, const float* hull_vertices, const uint8_t* face_sizes,
                               const uint32_t* face_indices, uint32_t motion, float density, float mass_override,
                               float* out_inv_mass, float* out_inv_inertia_local);

#ifdef __cplusplus
}
#endif
#endif
