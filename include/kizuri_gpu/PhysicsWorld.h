// kizuri_gpu/PhysicsWorld.h - C++ facade with the reference's PhysicsWorld surface, stepping on
// the GPU through the C-ABI of libkzg.so (include/kzg.h).  Header-only.
//
// Mirrors (reference paths):
//   PhysicsWorld           include/Kizuri/World/PhysicsWorld.h:82-239  (CreateBody, Step, StepFixed,
//                          GetSettings, GetStats, ComputeStateHash)
//   WorldSettings          PhysicsWorld.h:20-43     SolverSettings  include/Kizuri/Solver/ContactSolver.h:67-82
//   BodySettings / BodyID  include/Kizuri/Body/Body.h:14-30, 62-90
//   shapes                 include/Kizuri/Geometry/Shape.h (Sphere, Box, Capsule(halfHeight, radius),
//                          ConvexHull, Plane)
//   joints                 include/Kizuri/Constraint/Constraints.h:41-277 (PointConstraint ...
//                          SixDOFConstraint as descriptions, SetLimits / SetMotor, AddConstraint)
//   continuous collision   BodySettings::motionQuality = LinearCast, WorldSettings::useCCD /
//                          ccdMaxPenetration (PhysicsWorld.cpp:785-852)
// Differences, by design: shapes are registered with AddShape before the first step (the device
// shape table is uploaded once); body state is read back with GetBodyState instead of a Body*;
// errors throw kizuri_gpu::Error carrying the kzg_status and kzg_last_error() text.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <initializer_list>
#include <vector>

#include "../kzg.h"

namespace kizuri_gpu {

struct Vec3 {
    float x = 0, y = 0, z = 0;
};
struct Quat {
    float x = 0, y = 0, z = 0, w = 1;
};

enum class ShapeType : uint32_t { Sphere = KZG_SHAPE_SPHERE, Box = KZG_SHAPE_BOX, Capsule = KZG_SHAPE_CAPSULE,
                                  ConvexHull = KZG_SHAPE_HULL, Plane = KZG_SHAPE_PLANE };
enum class MotionType : uint32_t { Static = KZG_MOTION_STATIC, Kinematic = KZG_MOTION_KINEMATIC,
                                   Dynamic = KZG_MOTION_DYNAMIC };

class Error : public std::runtime_error {
public:
    Error(kzg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    kzg_status status;
};

inline void Check(kzg_status s, const kzg_ctx* ctx) {
    if (s != KZG_OK) throw Error(s, kzg_last_error(ctx));
}

struct Shape {
    ShapeType type = ShapeType::Sphere;
    float params[4] = {0, 0, 0, 0};
    std::vector<float> hullVertices;   // built hull (ConvexHullShape::Create vertex order)
    std::vector<uint8_t> faceSizes;
    std::vector<uint32_t> faceIndices;

    static Shape Sphere(float radius) { Shape s; s.type = ShapeType::Sphere; s.params[0] = radius; return s; }
    static Shape Box(const Vec3& he) {
        Shape s; s.type = ShapeType::Box; s.params[0] = he.x; s.params[1] = he.y; s.params[2] = he.z; return s;
    }
    static Shape Capsule(float halfHeight, float radius) {
        Shape s; s.type = ShapeType::Capsule; s.params[0] = halfHeight; s.params[1] = radius; return s;
    }
    static Shape Plane(const Vec3& n, float distance) {
        Shape s; s.type = ShapeType::Plane; s.params[0] = n.x; s.params[1] = n.y; s.params[2] = n.z;
        s.params[3] = distance; return s;
    }
    // ConvexHullShape::Create(points, maxPoints)
    static Shape ConvexHull(const std::vector<Vec3>& pts, uint32_t maxPoints = 256) {
        Shape s;
        s.type = ShapeType::ConvexHull;
        std::vector<float> in(3 * pts.size());
        for (size_t i = 0; i < pts.size(); ++i) { in[3 * i] = pts[i].x; in[3 * i + 1] = pts[i].y; in[3 * i + 2] = pts[i].z; }
        const uint32_t cap = 2 * (uint32_t)pts.size() + 8;
        s.hullVertices.resize(3 * pts.size());
        s.faceSizes.resize(cap);
        s.faceIndices.resize(3 * cap);
        uint32_t nv = 0, nf = 0, ni = 0;
        Check(kzg_hull_build(in.data(), (uint32_t)pts.size(), maxPoints, s.hullVertices.data(), &nv, s.faceSizes.data(),
                             &nf, s.faceIndices.data(), &ni, cap), nullptr);
        s.hullVertices.resize(3 * nv);
        s.faceSizes.resize(nf);
        s.faceIndices.resize(ni);
        return s;
    }
};

struct BodyID {
    uint32_t index = 0x00FFFFFFu;
    uint32_t sequence = 0;
    bool IsInvalid() const { return index == 0x00FFFFFFu; }
    uint32_t Packed() const { return (sequence << 24) | (index & 0x00FFFFFFu); }
};

enum class MotionQuality : uint8_t { Discrete = 0, LinearCast };  // Body.h:46-49

// BodySettings defaults (Body.h:62-90); `shape` is an index returned by AddShape.
struct BodySettings {
    Vec3 position;
    Quat rotation;
    int shape = -1;
    MotionType motionType = MotionType::Dynamic;
    Vec3 linearVelocity, angularVelocity;
    float friction = 0.5f, restitution = 0.0f, linearDamping = 0.05f, angularDamping = 0.05f;
    float gravityFactor = 1.0f, maxLinearVelocity = 500.0f, maxAngularVelocity = 50.0f;
    uint32_t objectLayer = 1, collisionMask = 0xFFFFFFFFu;
    bool allowSleeping = true, isSensor = false;
    MotionQuality motionQuality = MotionQuality::Discrete;
    float ccdMotionThreshold = 0.0f;  // Body.h:70
    float massOverride = 0.0f, density = 1000.0f;
    uint32_t worldId = 0;  // independent worlds stepped together (batched scenes)
};

struct SolverSettings {  // ContactSolver.h:67-82
    uint32_t velocityIterations = 16, positionIterations = 6;
    float baumgarte = 0.2f, penetrationSlop = 0.005f, restitutionThreshold = 1.0f, maxBiasVelocity = 3.0f;
    float warmStartFactor = 1.0f;
    bool useSplitImpulse = true;  // read nowhere by the reference; accepted with either value
    bool useSIMDSolver = true;    // false: the scalar constraint-order sweep
    bool useVelocityBias = false;
};

struct WorldSettings {  // PhysicsWorld.h:20-43 (the fields the accelerated step reads)
    Vec3 gravity{0.0f, -9.81f, 0.0f};
    SolverSettings solver;
    bool allowSleeping = true;    // the reference's default (PhysicsWorld.h:24)
    float sleepTimeThreshold = 0.5f, sleepLinearThreshold = 0.05f, sleepAngularThreshold = 0.1f;
    bool useFixedTimestep = true;
    float fixedTimestep = (float)(1.0 / 60.0);
    uint32_t maxSubSteps = 4;
    bool warmStart = true;
    bool useCCD = true;               // continuous collision for LinearCast bodies
    float ccdMaxPenetration = 0.01f;
};

// Joints (Constraints.h:41-277), built like the reference's constructors: world-space anchors and
// axes at the bodies' poses when the world next steps; pass the result to AddConstraint.
inline kzg_joint_desc JointDesc(uint32_t type, BodyID a, BodyID b, const Vec3& anchorA) {
    kzg_joint_desc d{};
    d.type = type;
    d.body_a = a.index;
    d.body_b = b.index;
    d.anchor_a[0] = anchorA.x; d.anchor_a[1] = anchorA.y; d.anchor_a[2] = anchorA.z;
    d.rotation[3] = 1.0f;
    return d;
}
inline kzg_joint_desc PointConstraint(BodyID a, BodyID b, const Vec3& worldAnchor) {
    return JointDesc(KZG_JOINT_POINT, a, b, worldAnchor);
}
inline kzg_joint_desc DistanceConstraint(BodyID a, BodyID b, const Vec3& worldAnchorA, const Vec3& worldAnchorB,
                                         float distance) {
    kzg_joint_desc d = JointDesc(KZG_JOINT_DISTANCE, a, b, worldAnchorA);
    d.anchor_b[0] = worldAnchorB.x; d.anchor_b[1] = worldAnchorB.y; d.anchor_b[2] = worldAnchorB.z;
    d.distance = distance;
    return d;
}
inline kzg_joint_desc FixedConstraint(BodyID a, BodyID b, const Vec3& worldAnchor) {
    return JointDesc(KZG_JOINT_FIXED, a, b, worldAnchor);
}
inline kzg_joint_desc HingeConstraint(BodyID a, BodyID b, const Vec3& worldAnchor, const Vec3& worldAxisA,
                                      const Vec3& worldAxisB) {
    kzg_joint_desc d = JointDesc(KZG_JOINT_HINGE, a, b, worldAnchor);
    d.axis_a[0] = worldAxisA.x; d.axis_a[1] = worldAxisA.y; d.axis_a[2] = worldAxisA.z;
    d.axis_b[0] = worldAxisB.x; d.axis_b[1] = worldAxisB.y; d.axis_b[2] = worldAxisB.z;
    return d;
}
inline kzg_joint_desc SliderConstraint(BodyID a, BodyID b, const Vec3& worldAnchor, const Vec3& worldAxis) {
    kzg_joint_desc d = JointDesc(KZG_JOINT_SLIDER, a, b, worldAnchor);
    d.axis_a[0] = worldAxis.x; d.axis_a[1] = worldAxis.y; d.axis_a[2] = worldAxis.z;
    return d;
}
inline kzg_joint_desc SixDOFConstraint(BodyID a, BodyID b, const Vec3& worldAnchor, const Quat& worldRotation) {
    kzg_joint_desc d = JointDesc(KZG_JOINT_SIXDOF, a, b, worldAnchor);
    d.rotation[0] = worldRotation.x; d.rotation[1] = worldRotation.y; d.rotation[2] = worldRotation.z;
    d.rotation[3] = worldRotation.w;
    return d;
}
// Hinge/SliderConstraint::SetLimits and SetMotor on a description.
inline kzg_joint_desc& SetLimits(kzg_joint_desc& d, float lower, float upper) {
    d.lower = lower; d.upper = upper; d.flags |= KZG_JOINT_LIMITS;
    return d;
}
inline kzg_joint_desc& SetMotor(kzg_joint_desc& d, float target, float maxImpulse) {
    d.motor_target = target; d.motor_max = maxImpulse; d.flags |= KZG_JOINT_MOTOR;
    return d;
}

struct Capacity {
    uint32_t maxBodies = 1u << 16, maxShapes = 1u << 16, maxHullVertices = 1u << 20, maxHullIndices = 1u << 22;
    uint32_t maxPairs = 1u << 20, maxCacheEntries = 1u << 21;
    int device = 0;
    uint32_t maxJoints = 1u << 16;
};

struct Transform {  // Math.h Transform: translation, then rotation
    Vec3 translation;
    Quat rotation;
};

struct BodyState {
    Vec3 position;
    Quat rotation;
    Vec3 linearVelocity, angularVelocity;
};

class PhysicsWorld {
public:
    explicit PhysicsWorld(const Capacity& cap = Capacity()) {
        kzg_config c{cap.maxBodies, cap.maxShapes, cap.maxHullVertices, cap.maxHullIndices, cap.maxPairs,
                     cap.maxCacheEntries, cap.device, cap.maxJoints};
        Check(kzg_create(&c, &ctx_), nullptr);
    }
    ~PhysicsWorld() {
        if (ctx_) kzg_destroy(ctx_);
    }
    PhysicsWorld(const PhysicsWorld&) = delete;
    PhysicsWorld& operator=(const PhysicsWorld&) = delete;

    WorldSettings& GetSettings() { return settings_; }
    void SetGravity(const Vec3& g) { settings_.gravity = g; }

    int AddShape(const Shape& s) {
        if (shapesUploaded_) throw Error(KZG_ERR_INVALID, "shapes must be added before the first step");
        shapes_.push_back(s);
        return (int)shapes_.size() - 1;
    }

    // PhysicsWorld::CreateBody: resolves mass properties like BodyManager::RecomputeMassProperties.
    BodyID CreateBody(const BodySettings& bs) {
        if (bs.shape < 0 || bs.shape >= (int)shapes_.size()) return BodyID{};
        const Shape& s = shapes_[bs.shape];
        kzg_shape_desc d = Desc(s, 0, 0, 0);
        float im = 0.0f, iil[9];
        Check(kzg_mass_properties(&d, s.hullVertices.data(), s.faceSizes.data(), s.faceIndices.data(),
                                  (uint32_t)bs.motionType, bs.density, bs.massOverride, &im, iil), ctx_);
        pending_.push_back(bs);
        invMass_.push_back(im);
        iil_.insert(iil_.end(), iil, iil + 9);
        BodyID id{numBodies_++, 0};
        return id;
    }

    // PhysicsWorld::AddConstraint: created when the world next steps, after the pending bodies, at
    // their poses then; returns the joint's index.
    uint32_t AddConstraint(const kzg_joint_desc& d) {
        pendingJoints_.push_back(d);
        return numJoints_++;
    }

    // PhysicsWorld::StepFixed
    void StepFixed(float dt) {
        Flush();
        Check(kzg_step(ctx_, dt, 1), ctx_);
    }
    // PhysicsWorld::Step: fixed-timestep accumulator with at most maxSubSteps steps (PhysicsWorld.cpp:225-243)
    void Step(float dt) {
        if (dt <= 0.0f) return;
        if (!settings_.useFixedTimestep) { StepFixed(dt); return; }
        accumulator_ += dt;
        uint32_t steps = 0;
        while (accumulator_ >= settings_.fixedTimestep && steps < settings_.maxSubSteps) {
            StepFixed(settings_.fixedTimestep);
            accumulator_ -= settings_.fixedTimestep;
            ++steps;
        }
        if (steps == settings_.maxSubSteps) accumulator_ = 0.0f;
    }

    BodyState GetBodyState(BodyID id) {
        Flush();
        float s[13];
        Check(kzg_download_state(ctx_, s, id.index, 1), ctx_);
        BodyState b;
        b.position = {s[0], s[1], s[2]};
        b.rotation = {s[3], s[4], s[5], s[6]};
        b.linearVelocity = {s[7], s[8], s[9]};
        b.angularVelocity = {s[10], s[11], s[12]};
        return b;
    }
    uint64_t ComputeStateHash() {
        Flush();
        uint64_t h = 0;
        Check(kzg_state_hash(ctx_, &h), ctx_);
        return h;
    }
    kzg_stats GetStats() {
        kzg_stats s{};
        Check(kzg_get_stats(ctx_, &s), ctx_);
        return s;
    }
    uint32_t GetNumBodies() const { return numBodies_; }
    kzg_ctx* Handle() { return ctx_; }

    // Activation and the convenience body operations (PhysicsWorld.cpp:109-205), applied on the
    // device in call order; `wake` activates the body afterwards, as in the reference.
    void SetBodyActive(BodyID id, bool active) { Edit(active ? KZG_EDIT_ACTIVATE : KZG_EDIT_DEACTIVATE, id, {}, false); }
    void ActivateBody(BodyID id) { Edit(KZG_EDIT_ACTIVATE, id, {}, false); }
    void DeactivateBody(BodyID id) { Edit(KZG_EDIT_DEACTIVATE, id, {}, false); }
    uint32_t GetNumActiveBodies() {
        Flush();
        uint32_t n = 0;
        Check(kzg_get_active_bodies(ctx_, nullptr, 0, &n), ctx_);
        return n;
    }
    void SetBodyPosition(BodyID id, const Vec3& p, bool wake = true) { Edit(KZG_EDIT_SET_POSITION, id, {p.x, p.y, p.z}, wake); }
    void SetBodyRotation(BodyID id, const Quat& q, bool wake = true) {
        Edit(KZG_EDIT_SET_ROTATION, id, {q.x, q.y, q.z, q.w}, wake);
    }
    void SetBodyTransform(BodyID id, const Transform& t, bool wake = true) {
        Edit(KZG_EDIT_SET_TRANSFORM, id,
             {t.translation.x, t.translation.y, t.translation.z, t.rotation.x, t.rotation.y, t.rotation.z, t.rotation.w},
             wake);
    }
    void SetLinearVelocity(BodyID id, const Vec3& v, bool wake = true) { Edit(KZG_EDIT_SET_LINEAR_VELOCITY, id, {v.x, v.y, v.z}, wake); }
    void SetAngularVelocity(BodyID id, const Vec3& w, bool wake = true) {
        Edit(KZG_EDIT_SET_ANGULAR_VELOCITY, id, {w.x, w.y, w.z}, wake);
    }
    void AddForce(BodyID id, const Vec3& f, bool wake = true) { Edit(KZG_EDIT_ADD_FORCE, id, {f.x, f.y, f.z}, wake); }
    void AddForceAtPoint(BodyID id, const Vec3& f, const Vec3& p, bool wake = true) {
        Edit(KZG_EDIT_ADD_FORCE_AT_POINT, id, {f.x, f.y, f.z, p.x, p.y, p.z}, wake);
    }
    void AddTorque(BodyID id, const Vec3& t, bool wake = true) { Edit(KZG_EDIT_ADD_TORQUE, id, {t.x, t.y, t.z}, wake); }
    void AddImpulse(BodyID id, const Vec3& i, bool wake = true) { Edit(KZG_EDIT_ADD_IMPULSE, id, {i.x, i.y, i.z}, wake); }
    void AddImpulseAtPoint(BodyID id, const Vec3& i, const Vec3& p, bool wake = true) {
        Edit(KZG_EDIT_ADD_IMPULSE_AT_POINT, id, {i.x, i.y, i.z, p.x, p.y, p.z}, wake);
    }

private:
    static kzg_shape_desc Desc(const Shape& s, uint32_t fv, uint32_t ff, uint32_t fi) {
        kzg_shape_desc d{};
        d.type = (uint32_t)s.type;
        for (int k = 0; k < 4; ++k) d.params[k] = s.params[k];
        d.first_vertex = fv; d.num_vertices = (uint32_t)s.hullVertices.size() / 3;
        d.first_face = ff; d.num_faces = (uint32_t)s.faceSizes.size();
        d.first_index = fi; d.num_indices = (uint32_t)s.faceIndices.size();
        return d;
    }

    void Edit(uint32_t op, BodyID id, std::initializer_list<float> v, bool wake) {
        Flush();
        kzg_body_edit e{};
        e.op = op;
        e.body = id.Packed();
        e.wake = wake ? 1u : 0u;
        int k = 0;
        for (float x : v) e.v[k++] = x;
        Check(kzg_edit_bodies(ctx_, &e, 1), ctx_);
    }

    void Flush() {
        if (!shapesUploaded_) {
            std::vector<kzg_shape_desc> d;
            std::vector<float> v;
            std::vector<uint8_t> f;
            std::vector<uint32_t> ix;
            for (const Shape& s : shapes_) {
                d.push_back(Desc(s, (uint32_t)v.size() / 3, (uint32_t)f.size(), (uint32_t)ix.size()));
                v.insert(v.end(), s.hullVertices.begin(), s.hullVertices.end());
                f.insert(f.end(), s.faceSizes.begin(), s.faceSizes.end());
                ix.insert(ix.end(), s.faceIndices.begin(), s.faceIndices.end());
            }
            Check(kzg_upload_shapes(ctx_, d.data(), (uint32_t)d.size(), v.data(), (uint32_t)v.size() / 3, f.data(),
                                    (uint32_t)f.size(), ix.data(), (uint32_t)ix.size()), ctx_);
            shapesUploaded_ = true;
        }
        kzg_world_settings ws;
        kzg_solver_settings ss;
        kzg_default_settings(&ws, &ss);
        ws.gravity[0] = settings_.gravity.x; ws.gravity[1] = settings_.gravity.y; ws.gravity[2] = settings_.gravity.z;
        ws.fixed_timestep = settings_.fixedTimestep;
        ws.allow_sleeping = settings_.allowSleeping ? 1 : 0;
        ws.warm_start = settings_.warmStart ? 1 : 0;
        ws.use_ccd = settings_.useCCD ? 1 : 0;
        ws.ccd_max_penetration = settings_.ccdMaxPenetration;
        ws.sleep_time_threshold = settings_.sleepTimeThreshold;
        ws.sleep_linear_threshold = settings_.sleepLinearThreshold;
        ws.sleep_angular_threshold = settings_.sleepAngularThreshold;
        ss.velocity_iterations = settings_.solver.velocityIterations;
        ss.position_iterations = settings_.solver.positionIterations;
        ss.baumgarte = settings_.solver.baumgarte;
        ss.penetration_slop = settings_.solver.penetrationSlop;
        ss.restitution_threshold = settings_.solver.restitutionThreshold;
        ss.max_bias_velocity = settings_.solver.maxBiasVelocity;
        ss.warm_start_factor = settings_.solver.warmStartFactor;
        ss.use_velocity_bias = settings_.solver.useVelocityBias ? 1 : 0;
        ss.use_split_impulse = settings_.solver.useSplitImpulse ? 1 : 0;
        ss.use_simd_solver = settings_.solver.useSIMDSolver ? 1 : 0;
        Check(kzg_set_world_settings(ctx_, &ws), ctx_);
        Check(kzg_set_solver_settings(ctx_, &ss), ctx_);
        if (!pending_.empty()) FlushBodies();
        if (!pendingJoints_.empty()) {
            uint32_t first = 0;
            Check(kzg_add_joints(ctx_, (uint32_t)pendingJoints_.size(), pendingJoints_.data(), &first), ctx_);
            pendingJoints_.clear();
        }
    }

    void FlushBodies() {
        const size_t n = pending_.size();
        std::vector<uint32_t> shape(n), motion(n), flags(n), layer(n), mask(n), world(n);
        std::vector<float> pos(3 * n), rot(4 * n), lv(3 * n), av(3 * n), fr(n), rs(n), ld(n), ad(n), gf(n), ml(n), ma(n),
            ccd(n);
        for (size_t i = 0; i < n; ++i) {
            const BodySettings& b = pending_[i];
            shape[i] = (uint32_t)b.shape; motion[i] = (uint32_t)b.motionType;
            flags[i] = (b.isSensor ? KZG_BODY_SENSOR : 0u) | (b.allowSleeping ? KZG_BODY_ALLOW_SLEEPING : 0u) |
                       (b.motionQuality == MotionQuality::LinearCast ? KZG_BODY_LINEAR_CAST : 0u);
            layer[i] = b.objectLayer; mask[i] = b.collisionMask; world[i] = b.worldId;
            pos[3 * i] = b.position.x; pos[3 * i + 1] = b.position.y; pos[3 * i + 2] = b.position.z;
            rot[4 * i] = b.rotation.x; rot[4 * i + 1] = b.rotation.y; rot[4 * i + 2] = b.rotation.z; rot[4 * i + 3] = b.rotation.w;
            lv[3 * i] = b.linearVelocity.x; lv[3 * i + 1] = b.linearVelocity.y; lv[3 * i + 2] = b.linearVelocity.z;
            av[3 * i] = b.angularVelocity.x; av[3 * i + 1] = b.angularVelocity.y; av[3 * i + 2] = b.angularVelocity.z;
            fr[i] = b.friction; rs[i] = b.restitution; ld[i] = b.linearDamping; ad[i] = b.angularDamping;
            gf[i] = b.gravityFactor; ml[i] = b.maxLinearVelocity; ma[i] = b.maxAngularVelocity;
            ccd[i] = b.ccdMotionThreshold;
        }
        kzg_body_soa soa{shape.data(), motion.data(), flags.data(), pos.data(), rot.data(), lv.data(), av.data(),
                         fr.data(), rs.data(), ld.data(), ad.data(), gf.data(), ml.data(), ma.data(), invMass_.data(),
                         iil_.data(), layer.data(), mask.data(), world.data(), ccd.data()};
        uint32_t first = 0;
        Check(kzg_add_bodies(ctx_, (uint32_t)n, &soa, &first), ctx_);
        pending_.clear();
        invMass_.clear();
        iil_.clear();
    }

    kzg_ctx* ctx_ = nullptr;
    WorldSettings settings_;
    std::vector<Shape> shapes_;
    std::vector<BodySettings> pending_;
    std::vector<kzg_joint_desc> pendingJoints_;
    uint32_t numJoints_ = 0;
    std::vector<float> invMass_, iil_;
    bool shapesUploaded_ = false;
    uint32_t numBodies_ = 0;
    float accumulator_ = 0.0f;
};

}  // namespace kizuri_gpu
