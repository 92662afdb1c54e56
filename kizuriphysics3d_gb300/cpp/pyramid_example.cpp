// C++ usage of the GPU contact pipeline through kizuri_gpu::PhysicsWorld (reference-style API):
// the World_PyramidRest layout (reference tests/TestWorld.cpp:103-128) scaled to `rows` rows,
// stepped `steps` times, then the state hash is printed.  With `poke` = 1, halfway through the
// run the top box gets an off-centre impulse, a bottom box a new velocity and an upward force,
// another box a new rotation, and one box is put to sleep, through the reference's own calls
// (AddImpulseAtPoint, SetLinearVelocity, AddForce, SetBodyRotation, SetBodyActive).
//
//   pyramid_example [rows=20] [steps=60] [poke=0]
#include <cstdio>
#include <cstdlib>

#include "kizuri_gpu/PhysicsWorld.h"

using namespace kizuri_gpu;

int main(int argc, char** argv) {
    const int rows = argc > 1 ? std::atoi(argv[1]) : 20;
    const int steps = argc > 2 ? std::atoi(argv[2]) : 60;
    const bool poke = argc > 3 && std::atoi(argv[3]) != 0;
    try {
        PhysicsWorld world;
        WorldSettings& ws = world.GetSettings();
        ws.solver.velocityIterations = 10;
        ws.solver.positionIterations = 2;
        ws.allowSleeping = false;  // as the Python API's scenes it is compared with
        const int plane = world.AddShape(Shape::Plane({0, 1, 0}, 0.0f));
        const int box = world.AddShape(Shape::Box({0.5f, 0.5f, 0.5f}));
        BodySettings ground;
        ground.shape = plane;
        ground.motionType = MotionType::Static;
        ground.friction = 0.6f;
        world.CreateBody(ground);
        BodyID first, top;
        for (int row = 0; row < rows; ++row) {
            const int n = rows - row;
            for (int i = 0; i < n; ++i) {
                BodySettings b;
                b.shape = box;
                b.friction = 0.6f;
                b.position = {(float)((i - (n - 1) * 0.5) * 1.02), (float)(0.5 + row * 1.02), 0.0f};
                top = world.CreateBody(b);
                if (row == 0 && i == 0) first = top;
            }
        }
        for (int s = 0; s < steps; ++s) {
            if (poke && s == steps / 2) {
                const BodyState t = world.GetBodyState(top);
                world.AddImpulseAtPoint(top, {3.0f, 0.0f, 0.0f}, {t.position.x, t.position.y + 0.5f, t.position.z + 0.3f});
                world.SetLinearVelocity(first, {0.0f, 2.0f, 0.0f});
                world.AddForce(first, {0.0f, 150.0f, 0.0f});
                world.SetBodyRotation(BodyID{first.index + 1, 0}, Quat{0.0f, 0.2f, 0.0f, 1.0f});
                world.SetBodyActive(BodyID{first.index + 2, 0}, false);
            }
            world.StepFixed((float)(1.0 / 60.0));
        }
        const kzg_stats st = world.GetStats();
        std::printf("bodies %u active %u constraints %u points %u hash %016llx\n", world.GetNumBodies(),
                    world.GetNumActiveBodies(), st.num_contact_constraints, st.num_contact_points,
                    (unsigned long long)world.ComputeStateHash());
    } catch (const Error& e) {
        std::fprintf(stderr, "kizuri_gpu error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
