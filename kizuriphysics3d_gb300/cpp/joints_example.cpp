// C++ usage of joints and continuous collision through kizuri_gpu::PhysicsWorld: nx x nz chains of
// `links` boxes hanging from static hooks (point joints, every third a hinge about z limited to
// +-0.8 rad), pushed sideways, and one LinearCast ball fired through the field; stepped `steps`
// times, then the state hash is printed.
//
//   joints_example [nx=3] [nz=3] [links=6] [steps=60]
#include <cstdio>
#include <cstdlib>

#include "kizuri_gpu/PhysicsWorld.h"

using namespace kizuri_gpu;

int main(int argc, char** argv) {
    const int nx = argc > 1 ? std::atoi(argv[1]) : 3;
    const int nz = argc > 2 ? std::atoi(argv[2]) : 3;
    const int links = argc > 3 ? std::atoi(argv[3]) : 6;
    const int steps = argc > 4 ? std::atoi(argv[4]) : 60;
    try {
        PhysicsWorld world;
        WorldSettings& ws = world.GetSettings();
        ws.solver.velocityIterations = 10;
        ws.solver.positionIterations = 2;
        ws.allowSleeping = false;  // as the Python API's scenes it is compared with
        const int plane = world.AddShape(Shape::Plane({0, 1, 0}, 0.0f));
        const int hook = world.AddShape(Shape::Box({0.1f, 0.1f, 0.1f}));
        const int link = world.AddShape(Shape::Box({0.1f, 0.25f, 0.1f}));
        const int ball = world.AddShape(Shape::Sphere(0.1f));
        BodySettings ground;
        ground.shape = plane;
        ground.motionType = MotionType::Static;
        ground.friction = 0.6f;
        world.CreateBody(ground);
        for (int ix = 0; ix < nx; ++ix) {
            for (int iz = 0; iz < nz; ++iz) {
                const int c = ix * nz + iz;
                const float x = (float)((ix - (nx - 1) * 0.5) * 1.5), z = (float)((iz - (nz - 1) * 0.5) * 1.5);
                BodySettings h;
                h.shape = hook;
                h.motionType = MotionType::Static;
                h.position = {x, 6.1f, z};
                BodyID prev = world.CreateBody(h);
                Vec3 anchor{x, 6.0f, z};
                for (int k = 0; k < links; ++k) {
                    const float y = (float)(6.0 - 0.5 * k - 0.25);
                    BodySettings b;
                    b.shape = link;
                    b.position = {x, y, z};
                    b.linearVelocity = {(float)(((c % 5) - 2) * 0.5 * (k + 1) / links), 0.0f,
                                        (float)(((c % 3) - 1) * 0.7 * (k + 1) / links)};
                    const BodyID id = world.CreateBody(b);
                    if (k % 3 == 2) {
                        kzg_joint_desc d = HingeConstraint(prev, id, anchor, {0, 0, 1}, {0, 0, 1});
                        world.AddConstraint(SetLimits(d, -0.8f, 0.8f));
                    } else {
                        world.AddConstraint(PointConstraint(prev, id, anchor));
                    }
                    prev = id;
                    anchor = {x, (float)(y - 0.25), z};
                }
            }
        }
        BodySettings shot;
        shot.shape = ball;
        shot.position = {-5.0f, 5.75f, 0.0f};
        shot.linearVelocity = {80.0f, 0.0f, 0.0f};
        shot.motionQuality = MotionQuality::LinearCast;
        world.CreateBody(shot);
        for (int s = 0; s < steps; ++s) world.StepFixed((float)(1.0 / 60.0));
        const kzg_stats st = world.GetStats();
        std::printf("bodies %u constraints %u points %u hash %016llx\n", world.GetNumBodies(),
                    st.num_contact_constraints, st.num_contact_points,
                    (unsigned long long)world.ComputeStateHash());
    } catch (const Error& e) {
        std::fprintf(stderr, "kizuri_gpu error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
