// Trace exporter for the reference engine (test infrastructure, never shipped).
//
// Drives the UNMODIFIED reference through its public API only:
//   PhysicsWorld::CreateBody / StepFixed / GetBody / GetBroadPhase().GetPairs() /
//   GetContactConstraints() / ComputeStateHash()   (include/Kizuri/World/PhysicsWorld.h:82-239)
// and writes a binary trace that the oracle and the GPU parity tests are pinned to.
//
// Built only by oracle/Makefile.ref, from the reference's own sources, into oracle/_ref/.
//
// usage: ref_trace <scene.kzsc> <out.kztr> <steps> [detail_steps] [--st] [--kzp1 <path>]
//   detail_steps : number of leading steps that also dump pairs and contact constraints
//   --st         : WorldSettings::useMultithreading = false
//   --kzp1 path  : write the world after the last step with SaveWorldToFile (a KZP1 file)
//   --edits path : body operations applied before given steps through PhysicsWorld's own methods
//                  (SetBodyPosition ... DeactivateBody, PhysicsWorld.cpp:109-205); the file holds
//                  a u32 count, then per edit u32 step, op, slot (bit 31: use a stale BodyID of
//                  that slot), wake and 8 floats (op numbers and operands as kzg_body_edit's)
#include "Kizuri/Kizuri.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <chrono>
#include <memory>
#include <vector>

using namespace kizuri;

namespace {

struct Reader {
    std::vector<uint8_t> buf;
    size_t off = 0;
    template <typename T> T get() {
        T v;
        std::memcpy(&v, buf.data() + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
};

struct Writer {
    FILE* f;
    template <typename T> void put(const T& v) { std::fwrite(&v, sizeof(T), 1, f); }
    void putv(const Vec3& v) { put(v.x); put(v.y); put(v.z); }
};

struct Edit {
    uint32_t step, op, slot, wake;
    float v[8];
};

void apply_edit(PhysicsWorld& world, const std::vector<BodyID>& ids, const Edit& e) {
    const uint32_t slot = e.slot & 0x7FFFFFFFu;
    BodyID id = ids[slot];
    if (e.slot & 0x80000000u) id = BodyID::Unpack(id.Packed() ^ (1u << 24));  // stale: another sequence
    const Vec3 a(e.v[0], e.v[1], e.v[2]), b(e.v[3], e.v[4], e.v[5]);
    const bool wake = e.wake != 0;
    switch (e.op) {
        case 0: world.SetBodyPosition(id, a, wake); break;
        case 1: world.SetBodyRotation(id, Quat(e.v[0], e.v[1], e.v[2], e.v[3]), wake); break;
        case 2: world.SetBodyTransform(id, Transform(Quat(e.v[3], e.v[4], e.v[5], e.v[6]), a), wake); break;
        case 3: world.SetLinearVelocity(id, a, wake); break;
        case 4: world.SetAngularVelocity(id, a, wake); break;
        case 5: world.AddForce(id, a, wake); break;
        case 6: world.AddForceAtPoint(id, a, b, wake); break;
        case 7: world.AddTorque(id, a, wake); break;
        case 8: world.AddImpulse(id, a, wake); break;
        case 9: world.AddImpulseAtPoint(id, a, b, wake); break;
        case 10: world.ActivateBody(id); break;
        case 11: world.DeactivateBody(id); break;
        default: std::fprintf(stderr, "edit op %u unknown\n", e.op); std::exit(1);
    }
}

struct SceneShape {
    uint32_t type;
    float p[4];
    std::vector<Vec3> pts;
};

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s scene out steps [detail_steps] [--st]\n", argv[0]);
        return 2;
    }
    const char* scenePath = argv[1];
    const char* outPath = argv[2];
    int steps = std::atoi(argv[3]);
    int detail = argc > 4 ? std::atoi(argv[4]) : 0;
    bool singleThread = false;
    const char* kzp1Path = nullptr;  // --kzp1 <path>: SaveWorldToFile after the last step
    for (int i = 1; i < argc; ++i) {
        if (std::strcmp(argv[i], "--st") == 0) singleThread = true;
        if (std::strcmp(argv[i], "--kzp1") == 0 && i + 1 < argc) kzp1Path = argv[i + 1];
    }
    std::vector<Edit> edits;
    for (int i = 1; i + 1 < argc; ++i) {
        if (std::strcmp(argv[i], "--edits") != 0) continue;
        FILE* ef = std::fopen(argv[i + 1], "rb");
        if (!ef) { std::perror("edits"); return 1; }
        uint32_t n = 0;
        if (std::fread(&n, 4, 1, ef) != 1) { std::fprintf(stderr, "edits: short file\n"); return 1; }
        edits.resize(n);
        if (n && std::fread(edits.data(), sizeof(Edit), n, ef) != n) { std::fprintf(stderr, "edits: short file\n"); return 1; }
        std::fclose(ef);
    }

    Reader rd;
    {
        FILE* f = std::fopen(scenePath, "rb");
        if (!f) { std::perror("scene"); return 1; }
        std::fseek(f, 0, SEEK_END);
        long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        rd.buf.resize(size_t(n));
        if (std::fread(rd.buf.data(), 1, size_t(n), f) != size_t(n)) return 1;
        std::fclose(f);
    }
    if (rd.get<uint32_t>() != 0x43535A4Bu) {
        std::fprintf(stderr, "bad scene\n");
        return 1;
    }
    const uint32_t version = rd.get<uint32_t>();
    if (version != 1u && version != 2u) {
        std::fprintf(stderr, "bad scene version\n");
        return 1;
    }

    PhysicsWorld world;
    WorldSettings& ws = world.GetSettings();
    ws.gravity.x = rd.get<float>(); ws.gravity.y = rd.get<float>(); ws.gravity.z = rd.get<float>();
    float dt = rd.get<float>();
    ws.solver.velocityIterations = rd.get<uint32_t>();
    ws.solver.positionIterations = rd.get<uint32_t>();
    uint32_t wflags = rd.get<uint32_t>();
    ws.solver.baumgarte = rd.get<float>();
    ws.solver.penetrationSlop = rd.get<float>();
    ws.solver.restitutionThreshold = rd.get<float>();
    ws.solver.maxBiasVelocity = rd.get<float>();
    ws.solver.warmStartFactor = rd.get<float>();
    if (version >= 2u) {
        ws.sleepTimeThreshold = rd.get<float>();
        ws.sleepLinearThreshold = rd.get<float>();
        ws.sleepAngularThreshold = rd.get<float>();
    }
    ws.allowSleeping = (wflags & 1u) != 0;
    ws.solver.useVelocityBias = (wflags & 2u) != 0;
    ws.useMultithreading = !singleThread;
    if (wflags & 4u) setenv("KZ_NOWS", "1", 1);
    ws.solver.useSIMDSolver = (wflags & 8u) == 0;

    uint32_t ns = rd.get<uint32_t>();
    std::vector<ShapeRef> shapes(ns);
    std::vector<SceneShape> sdesc(ns);
    for (uint32_t i = 0; i < ns; ++i) {
        SceneShape& s = sdesc[i];
        s.type = rd.get<uint32_t>();
        for (float& p : s.p) p = rd.get<float>();
        uint32_t np = rd.get<uint32_t>();
        for (uint32_t k = 0; k < np; ++k) {
            float x = rd.get<float>(), y = rd.get<float>(), z = rd.get<float>();
            s.pts.push_back(Vec3(x, y, z));
        }
        switch (s.type) {
            case 0: shapes[i] = ShapeRef(new SphereShape(s.p[0])); break;
            case 1: shapes[i] = ShapeRef(new BoxShape(Vec3(s.p[0], s.p[1], s.p[2]))); break;
            case 2: shapes[i] = ShapeRef(new CapsuleShape(s.p[0], s.p[1])); break;
            case 4: {
                Ref<ConvexHullShape> h = ConvexHullShape::Create(ArrayView<const Vec3>(s.pts.data(), s.pts.size()));
                if (!h) { std::fprintf(stderr, "hull %u degenerate\n", i); return 1; }
                shapes[i] = ShapeRef(h.Get());
                break;
            }
            case 8: shapes[i] = ShapeRef(new PlaneShape(Plane(Vec3(s.p[0], s.p[1], s.p[2]), s.p[3]))); break;
            default: std::fprintf(stderr, "shape type %u unsupported\n", s.type); return 1;
        }
    }

    uint32_t nb = rd.get<uint32_t>();
    std::vector<BodyID> ids(nb);
    for (uint32_t i = 0; i < nb; ++i) {
        BodySettings bs;
        uint32_t shape = rd.get<uint32_t>();
        uint32_t motion = rd.get<uint32_t>();
        float v[13];
        for (float& x : v) x = rd.get<float>();
        float m[9];
        for (float& x : m) x = rd.get<float>();
        uint32_t layer = rd.get<uint32_t>(), mask = rd.get<uint32_t>(), flags = rd.get<uint32_t>();
        if (version >= 2u) bs.ccdMotionThreshold = rd.get<float>();
        bs.shape = shapes[shape];
        bs.motionType = MotionType(motion);
        bs.position = Vec3(v[0], v[1], v[2]);
        bs.rotation = Quat(v[3], v[4], v[5], v[6]);
        bs.linearVelocity = Vec3(v[7], v[8], v[9]);
        bs.angularVelocity = Vec3(v[10], v[11], v[12]);
        bs.friction = m[0]; bs.restitution = m[1]; bs.linearDamping = m[2]; bs.angularDamping = m[3];
        bs.gravityFactor = m[4]; bs.maxLinearVelocity = m[5]; bs.maxAngularVelocity = m[6];
        bs.density = m[7]; bs.massOverride = m[8];
        bs.objectLayer = layer; bs.collisionMask = mask;
        bs.isSensor = (flags & 1u) != 0;
        bs.allowSleeping = (flags & 2u) != 0;
        if (flags & 4u) bs.motionQuality = MotionQuality::LinearCast;
        ids[i] = world.CreateBody(bs);
        if (ids[i].IsInvalid()) { std::fprintf(stderr, "body %u invalid\n", i); return 1; }
    }

    // Optional joint section: count, then per joint {type, body A, body B, flags, anchor A/B,
    // axis A/B, rotation, distance, limits, motor, axis modes, motor mask, six-dof motors}, created
    // through the reference's constructors and PhysicsWorld::AddConstraint.
    uint32_t nj = rd.off < rd.buf.size() ? rd.get<uint32_t>() : 0u;
    for (uint32_t j = 0; j < nj; ++j) {
        uint32_t type = rd.get<uint32_t>(), ia = rd.get<uint32_t>(), ib = rd.get<uint32_t>(), fl = rd.get<uint32_t>();
        float f[21];
        for (float& x : f) x = rd.get<float>();
        uint32_t modes = rd.get<uint32_t>(), motors = rd.get<uint32_t>();
        float sm[12];
        for (float& x : sm) x = rd.get<float>();
        Body* a = world.GetBody(ids[ia]);
        Body* b = world.GetBody(ids[ib]);
        const Vec3 anA(f[0], f[1], f[2]), anB(f[3], f[4], f[5]), axA(f[6], f[7], f[8]), axB(f[9], f[10], f[11]);
        const Quat rot(f[12], f[13], f[14], f[15]);
        std::unique_ptr<Constraint> c;
        switch (type) {
            case 0:
                if (fl & 8u) c = std::make_unique<PointConstraint>(a, b, anA, anB);
                else c = std::make_unique<PointConstraint>(a, b, anA);
                break;
            case 1: c = std::make_unique<DistanceConstraint>(a, b, anA, anB, f[16]); break;
            case 2: c = std::make_unique<FixedConstraint>(a, b, anA); break;
            case 3: {
                auto h = std::make_unique<HingeConstraint>(a, b, anA, axA, axB);
                if (fl & 2u) h->SetLimits(f[17], f[18]);
                if (fl & 4u) h->SetMotor(f[19], f[20]);
                c = std::move(h);
                break;
            }
            case 4: {
                auto sl = std::make_unique<SliderConstraint>(a, b, anA, axA);
                if (fl & 2u) sl->SetLimits(f[17], f[18]);
                if (fl & 4u) sl->SetMotor(f[19], f[20]);
                c = std::move(sl);
                break;
            }
            case 5: {
                auto d = std::make_unique<SixDOFConstraint>(a, b, anA, rot);
                for (uint32_t k = 0; k < 3; ++k) {
                    d->SetLinearAxisMode(k, SixDOFConstraint::AxisMode((modes >> (2 * k)) & 3u));
                    d->SetAngularAxisMode(k, SixDOFConstraint::AxisMode((modes >> (2 * k + 6)) & 3u));
                    if (motors & (1u << k)) d->SetLinearMotor(k, sm[k], sm[3 + k]);
                    if (motors & (8u << k)) d->SetAngularMotor(k, sm[6 + k], sm[9 + k]);
                }
                c = std::move(d);
                break;
            }
            default: std::fprintf(stderr, "joint type %u unsupported\n", type); return 1;
        }
        if (fl & 1u) c->SetEnabled(false);
        world.AddConstraint(std::move(c));
    }

    FILE* f = std::fopen(outPath, "wb");
    if (!f) { std::perror("out"); return 1; }
    Writer w{f};
    w.put(uint32_t(0x52545A4Bu));  // 'KZTR'
    w.put(uint32_t(1));
    w.put(nb);
    w.put(uint32_t(steps));
    w.put(uint32_t(detail));

    // Setup: packed ids and mass properties exactly as the reference computed them.
    for (uint32_t i = 0; i < nb; ++i) {
        const Body* b = world.GetBody(ids[i]);
        const MotionProperties& mp = b->GetMotionProperties();
        w.put(uint32_t(ids[i].Packed()));
        w.put(mp.inverseMass);
        for (int c = 0; c < 3; ++c) w.putv(mp.inverseInertiaLocal.col[c]);
        for (int c = 0; c < 3; ++c) w.putv(mp.inverseInertiaWorld.col[c]);
    }
    // Hulls as built by ConvexHullShape::Create.
    uint32_t nh = 0;
    for (uint32_t i = 0; i < ns; ++i) nh += sdesc[i].type == 4 ? 1u : 0u;
    w.put(nh);
    for (uint32_t i = 0; i < ns; ++i) {
        if (sdesc[i].type != 4) continue;
        const ConvexHullShape* h = static_cast<const ConvexHullShape*>(shapes[i].Get());
        w.put(i);
        auto pts = h->GetPoints();
        auto sizes = h->GetFaceSizes();
        auto idx = h->GetFaceIndices();
        w.put(uint32_t(pts.Size()));
        for (usize k = 0; k < pts.Size(); ++k) w.putv(pts[k]);
        w.put(uint32_t(sizes.Size()));
        for (usize k = 0; k < sizes.Size(); ++k) w.put(uint8_t(sizes[k]));
        w.put(uint32_t(idx.Size()));
        for (usize k = 0; k < idx.Size(); ++k) w.put(uint32_t(idx[k]));
        w.put(h->GetVolume());
    }

    auto dumpState = [&]() {
        for (uint32_t i = 0; i < nb; ++i) {
            const Body* b = world.GetBody(ids[i]);
            w.putv(b->GetPosition());
            const Quat& q = b->GetRotation();
            w.put(q.x); w.put(q.y); w.put(q.z); w.put(q.w);
            w.putv(b->GetLinearVelocity());
            w.putv(b->GetAngularVelocity());
        }
    };
    dumpState();

    double totalMs = 0;
    for (int s = 0; s < steps; ++s) {
        for (const Edit& e : edits)
            if (e.step == uint32_t(s)) {
                if ((e.slot & 0x7FFFFFFFu) >= nb) { std::fprintf(stderr, "edit slot out of range\n"); return 1; }
                apply_edit(world, ids, e);
            }
        auto t0 = std::chrono::steady_clock::now();
        world.StepFixed(dt);
        auto t1 = std::chrono::steady_clock::now();
        totalMs += std::chrono::duration<double, std::milli>(t1 - t0).count();
        w.put(uint32_t(s));
        w.put(uint64_t(world.ComputeStateHash()));
        const WorldStats& st = world.GetStats();
        w.put(st.numBroadPhasePairs); w.put(st.numContactConstraints);
        w.put(st.numContactPoints); w.put(st.numIslands);
        dumpState();
        if (s < detail) {
            auto pairs = world.GetBroadPhase().GetPairs();
            w.put(uint32_t(pairs.Size()));
            for (usize k = 0; k < pairs.Size(); ++k) {
                w.put(uint32_t(world.GetBroadPhase().GetUserData(pairs[k].proxyA)));
                w.put(uint32_t(world.GetBroadPhase().GetUserData(pairs[k].proxyB)));
            }
            auto cons = world.GetContactConstraints();
            w.put(uint32_t(cons.Size()));
            for (usize k = 0; k < cons.Size(); ++k) {
                const ContactConstraint& c = cons[k];
                w.put(uint32_t(c.bodyA->GetID().Packed()));
                w.put(uint32_t(c.bodyB->GetID().Packed()));
                w.put(uint32_t(c.numPoints));
                w.put(c.friction); w.put(c.restitution);
                for (u32 p = 0; p < c.numPoints; ++p) {
                    const ContactPointConstraint& q = c.points[p];
                    w.putv(q.pointOnA); w.putv(q.pointOnB); w.putv(q.normal);
                    w.put(q.separation); w.put(uint32_t(q.featureId));
                    w.putv(q.rA); w.putv(q.rB); w.putv(q.localAnchorA); w.putv(q.localAnchorB);
                    w.putv(q.tangent1); w.putv(q.tangent2);
                    w.put(q.normalMass); w.put(q.tangentMass1); w.put(q.tangentMass2);
                    w.put(q.normalImpulse); w.put(q.tangentImpulse1); w.put(q.tangentImpulse2);
                    w.put(q.restitutionBias); w.put(q.positionBias); w.put(q.biasImpulse);
                    w.put(q.normalVelocity);
                }
            }
        }
    }
    w.put(totalMs);
    std::fclose(f);
    if (kzp1Path && !SaveWorldToFile(world, kzp1Path)) {
        std::fprintf(stderr, "SaveWorldToFile failed\n");
        return 1;
    }
    std::fprintf(stderr, "ref_trace: %u bodies, %d steps, %.3f ms/step, hash %016llx\n", nb, steps,
                 steps ? totalMs / steps : 0.0, (unsigned long long)world.ComputeStateHash());
    return 0;
}
