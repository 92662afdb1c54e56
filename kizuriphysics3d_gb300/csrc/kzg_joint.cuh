// Joints (Constraints.cpp:1-597, Constraints.h:41-277): point, distance, fixed, hinge (limits,
// motor), slider (limits, motor) and six-dof, with the reference's creation, Prepare, WarmStart,
// SolveVelocity and SolvePosition arithmetic, operation for operation.
//
// A joint lives in one JointDev record.  Joints join islands (PhysicsWorld.cpp:625-633); an island
// that holds joints is solved by one CTA of k_solve_big in the reference's order (contact warm
// start, joint warm starts, contact velocity sweeps, joint velocity iterations, contact bias
// sweeps; PhysicsWorld.cpp:666-743), the joint parts by one thread in joint order.  After the
// positions are integrated, k_joint_positions runs each island's joints' position correction
// (PhysicsWorld.cpp:293-306, 745-752).
//
// sin, cos, acos and atan2 are evaluated in double precision and rounded to float; the reference
// calls the C library's float functions, so a result can differ from the reference's in the last
// bit.  The oracle's matching mode (kzo_set_trig_mode 1) does the same with the C library's double
// functions: the two agree wherever CUDA's and the C library's double results round to the same
// float, which the joint parity tests check rather than assume.
#pragma once
#include "kzg_ctx.h"
#include "kzg_math.cuh"

namespace kzg {

constexpr uint32_t kJointDisabled = 1u, kJointLimits = 2u, kJointMotor = 4u, kJointLocalAnchors = 8u;
enum : uint32_t { kJointPoint = 0, kJointDistance = 1, kJointFixed = 2, kJointHinge = 3, kJointSlider = 4,
                  kJointSixDof = 5 };

struct JointDev {
    uint32_t type, a, b, flags, modes, motors, pad0, pad1;
    Vec3 la, lb, lax, lbx, lpa[2], lpb[2];
    Quat relrot;
    Mat3 crot;
    float target, lower, upper, motor_target, motor_max;
    float six[12];  // six-dof motors: linear targets, linear max, angular targets, angular max
    // prepared state and accumulated impulses
    Vec3 r0, r1, axis, imp1, imp2;
    Mat3 m1, m2;
    float sm[2], simp[2], limit_mass, limit_imp, motor_imp, axial_mass, axial_imp, dmass, dimp;
    Vec3 lin_imp[3], ang_imp[3], axes[3];
};

__device__ __forceinline__ float jsin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float jcos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float jacos(float x) { return (float)acos((double)x); }
__device__ __forceinline__ float jatan2(float y, float x) { return (float)atan2((double)y, (double)x); }

__device__ __forceinline__ Mat3 m_diag(float s) {
    return Mat3{Vec3(1.0f * s, 0.0f * s, 0.0f * s), Vec3(0.0f * s, 1.0f * s, 0.0f * s), Vec3(0.0f * s, 0.0f * s, 1.0f * s)};
}
// Mat3::Skew (Math.h:193-197)
__device__ __forceinline__ Mat3 m_skew(const Vec3& v) {
    return Mat3{Vec3(0.0f, v.z, -v.y), Vec3(-v.z, 0.0f, v.x), Vec3(v.y, -v.x, 0.0f)};
}
__device__ __forceinline__ Mat3 m_add(const Mat3& a, const Mat3& b) { return Mat3{a.c0 + b.c0, a.c1 + b.c1, a.c2 + b.c2}; }
__device__ __forceinline__ Mat3 m_sub(const Mat3& a, const Mat3& b) { return Mat3{a.c0 - b.c0, a.c1 - b.c1, a.c2 - b.c2}; }
// Mat3::Inversed (Math.cpp:27-43): adjugate over determinant, zero for a singular matrix
__device__ __forceinline__ Mat3 m_inverse(const Mat3& m) {
    const Vec3 r0 = m.c1.cross(m.c2), r1 = m.c2.cross(m.c0), r2 = m.c0.cross(m.c1);
    const float det = m.c0.dot(r0);
    const float inv = det != 0.0f ? 1.0f / det : 0.0f;
    return Mat3{Vec3(r0.x, r1.x, r2.x) * inv, Vec3(r0.y, r1.y, r2.y) * inv, Vec3(r0.z, r1.z, r2.z) * inv};
}
// Vec3::GetBasis (Math.cpp:9-22)
__device__ __forceinline__ void v_basis(const Vec3& n, Vec3& b, Vec3& c) {
    if (n.z < -0.9999999f) {
        b = Vec3(0.0f, -1.0f, 0.0f);
        c = Vec3(-1.0f, 0.0f, 0.0f);
    } else {
        const float a = 1.0f / (1.0f + n.z);
        const float bb = -n.x * n.y * a;
        b = Vec3(1.0f - n.x * n.x * a, bb, -n.x);
        c = Vec3(bb, 1.0f - n.y * n.y * a, -n.y);
    }
}
__device__ __forceinline__ Quat q_conj(const Quat& q) { return Quat(-q.x, -q.y, -q.z, q.w); }

// Body access for the joint routines: velocities, pose and inverse mass / world inertia.
struct JBodies {
    const DeviceBodies& b;
    __device__ Vec3 pos(uint32_t i) const { return V3(b.pos[i]); }
    __device__ Quat rot(uint32_t i) const { return Q4(b.rot[i]); }
    __device__ Vec3 lv(uint32_t i) const { return V3(b.lv[i]); }
    __device__ Vec3 av(uint32_t i) const { return V3(b.av[i]); }
    __device__ Mat3 iiw(uint32_t i) const { return M3(&b.iiw[3 * i]); }
    __device__ float im(uint32_t i) const { return b.inv_mass[i]; }
};

// PointEffectiveMass, AngularEffectiveMass, LinearEffectiveMass (Constraints.cpp:23-52)
__device__ inline Mat3 point_mass(const JBodies& B, uint32_t a, uint32_t b, const Vec3& ra, const Vec3& rb) {
    Mat3 K = m_diag(B.im(a) + B.im(b));
    const Mat3 sa = m_skew(ra), sb = m_skew(rb);
    K = m_sub(K, sa * (B.iiw(a) * sa));
    return m_sub(K, sb * (B.iiw(b) * sb));
}
__device__ inline float angular_mass(const JBodies& B, uint32_t a, uint32_t b, const Vec3& axis) {
    const float k = axis.dot(B.iiw(a) * axis) + axis.dot(B.iiw(b) * axis);
    return k > kEps ? 1.0f / k : 0.0f;
}
__device__ inline float linear_mass(const JBodies& B, uint32_t a, uint32_t b, const Vec3& ra, const Vec3& rb,
                                    const Vec3& axis) {
    const Vec3 ca = ra.cross(axis), cb = rb.cross(axis);
    float k = B.im(a) + B.im(b);
    k += ca.dot(B.iiw(a) * ca);
    k += cb.dot(B.iiw(b) * cb);
    return k > kEps ? 1.0f / k : 0.0f;
}
// ApplyImpulse / ApplyAngularImpulse (Constraints.cpp:8-20)
__device__ inline void apply_impulse(const JBodies& B, uint32_t a, uint32_t b, const Vec3& ra, const Vec3& rb,
                                     const Vec3& imp) {
    B.b.lv[a] = F4(B.lv(a) + imp * B.im(a), 0.0f);
    B.b.av[a] = F4(B.av(a) + B.iiw(a) * ra.cross(imp), 0.0f);
    B.b.lv[b] = F4(B.lv(b) - imp * B.im(b), 0.0f);
    B.b.av[b] = F4(B.av(b) - B.iiw(b) * rb.cross(imp), 0.0f);
}
__device__ inline void apply_angular(const JBodies& B, uint32_t a, uint32_t b, const Vec3& ang) {
    B.b.av[a] = F4(B.av(a) + B.iiw(a) * ang, 0.0f);
    B.b.av[b] = F4(B.av(b) - B.iiw(b) * ang, 0.0f);
}
// IntegrateRotation(q, dw) (Constraints.cpp:54-59) with Quat::AxisAngle (Math.cpp:78-83)
__device__ inline Quat rotate_by(const Quat& q, const Vec3& dw) {
    const float a2 = dw.len2();
    if (a2 < 1.0e-12f) return q;
    const float a = sqrtf(a2);
    const Vec3 ax = (dw / a).normalized();
    const float half = a * 0.5f;
    const float s = jsin(half);
    return (Quat(ax.x * s, ax.y * s, ax.z * s, jcos(half)) * q).normalized();
}
// ApplyPositionalImpulse (Constraints.cpp:62-71)
__device__ inline void apply_positional(const JBodies& B, uint32_t a, uint32_t b, const Vec3& lin, const Vec3& ang) {
    B.b.pos[a] = F4(B.pos(a) + lin * B.im(a), 0.0f);
    B.b.rot[a] = F4q(rotate_by(B.rot(a), B.iiw(a) * ang));
    B.b.pos[b] = F4(B.pos(b) - lin * B.im(b), 0.0f);
    B.b.rot[b] = F4q(rotate_by(B.rot(b), -(B.iiw(b) * ang)));
}
__device__ __forceinline__ Vec3 rel_vel(const JBodies& B, const JointDev& j) {
    return (B.lv(j.a) + B.av(j.a).cross(j.r0)) - (B.lv(j.b) + B.av(j.b).cross(j.r1));
}
// HingeConstraint::GetAngle (Constraints.cpp:361-368)
__device__ inline float hinge_angle(const JBodies& B, const JointDev& j) {
    const Quat qa = B.rot(j.a);
    const Vec3 axis = qa.rotate(j.lax), pa = qa.rotate(j.lpa[0]), pb = B.rot(j.b).rotate(j.lpb[0]);
    return jatan2(axis.dot(pa.cross(pb)), pa.dot(pb));
}

// The constructors: world anchors and axes at the bodies' current poses.
__device__ inline void joint_create(const JBodies& B, JointDev& j, const kzg_joint_desc& d) {
    j = JointDev{};
    j.type = d.type;
    j.a = d.body_a;
    j.b = d.body_b;
    j.flags = d.flags;
    j.modes = d.axis_modes;
    j.motors = d.motor_mask;
    j.target = d.distance;
    j.lower = d.lower;
    j.upper = d.upper;
    j.motor_target = d.motor_target;
    j.motor_max = d.motor_max;
    for (int k = 0; k < 12; ++k) j.six[k] = d.six_motor[k];
    const Vec3 anA(d.anchor_a[0], d.anchor_a[1], d.anchor_a[2]), anB(d.anchor_b[0], d.anchor_b[1], d.anchor_b[2]);
    const Vec3 axA(d.axis_a[0], d.axis_a[1], d.axis_a[2]), axB(d.axis_b[0], d.axis_b[1], d.axis_b[2]);
    const Quat qa = B.rot(j.a), qb = B.rot(j.b);
    const Vec3 pa = B.pos(j.a), pb = B.pos(j.b);
    if (j.type == kJointPoint && (j.flags & kJointLocalAnchors)) {
        j.la = anA;
        j.lb = anB;
    } else {
        j.la = qa.inv_rotate(anA - pa);
        j.lb = qb.inv_rotate((j.type == kJointDistance ? anB : anA) - pb);
    }
    if (j.type == kJointFixed) j.relrot = q_conj(qa) * qb;
    if (j.type == kJointHinge) {
        j.lax = qa.inv_rotate(axA.normalized());
        j.lbx = qb.inv_rotate(axB.normalized());
        v_basis(j.lax, j.lpa[0], j.lpa[1]);
        v_basis(j.lbx, j.lpb[0], j.lpb[1]);
    }
    if (j.type == kJointSlider) {
        j.lax = qa.inv_rotate(axA.normalized());
        j.lbx = qb.inv_rotate(axA.normalized());
    }
    if (j.type == kJointSixDof) j.crot = Quat(d.rotation[0], d.rotation[1], d.rotation[2], d.rotation[3]).to_mat3();
}

__device__ inline void joint_prepare(const JBodies& B, JointDev& j) {
    const uint32_t a = j.a, b = j.b;
    const Quat qa = B.rot(a), qb = B.rot(b);
    j.r0 = qa.rotate(j.la);
    j.r1 = qb.rotate(j.lb);
    switch (j.type) {
        case kJointPoint: j.m1 = m_inverse(point_mass(B, a, b, j.r0, j.r1)); break;
        case kJointDistance: {
            const Vec3 d = (B.pos(b) + j.r1) - (B.pos(a) + j.r0);
            const float dist = d.len();
            j.axis = dist > kEps ? d / dist : Vec3(0.0f, 1.0f, 0.0f);
            j.dmass = linear_mass(B, a, b, j.r0, j.r1, j.axis);
            break;
        }
        case kJointFixed:
            j.m1 = m_inverse(point_mass(B, a, b, j.r0, j.r1));
            j.m2 = m_inverse(m_add(B.iiw(a), B.iiw(b)));
            break;
        case kJointHinge: {
            j.m1 = m_inverse(point_mass(B, a, b, j.r0, j.r1));
            const Vec3 pa[2] = {qa.rotate(j.lpa[0]), qa.rotate(j.lpa[1])};
            const Vec3 pb[2] = {qb.rotate(j.lpb[0]), qb.rotate(j.lpb[1])};
            for (int i = 0; i < 2; ++i) {
                const Vec3 axis = (pa[i] + pb[i]).normalized_or(pa[i]);
                j.sm[i] = angular_mass(B, a, b, axis);
                j.lpa[i] = qa.inv_rotate(axis);
            }
            j.limit_mass = angular_mass(B, a, b, qa.rotate(j.lax));
            break;
        }
        case kJointSlider: {
            const Vec3 axis = qa.rotate(j.lax);
            Vec3 p0, p1;
            v_basis(axis, p0, p1);
            j.axial_mass = linear_mass(B, a, b, j.r0, j.r1, axis);
            const Mat3 K = point_mass(B, a, b, j.r0, j.r1);
            const float k00 = p0.dot(K * p0), k01 = p0.dot(K * p1), k11 = p1.dot(K * p1);
            const float det = k00 * k11 - k01 * k01;
            if (rabs(det) > 1.0e-12f) {
                const float inv = 1.0f / det;
                j.m1 = Mat3{p0 * (k11 * inv) + p1 * (-k01 * inv), p0 * (-k01 * inv) + p1 * (k00 * inv), Vec3()};
            } else {
                j.m1 = Mat3{Vec3(), Vec3(), Vec3()};
            }
            j.m2 = m_inverse(m_add(B.iiw(a), B.iiw(b)));
            break;
        }
        case kJointSixDof: {
            const Mat3 r = qa.to_mat3() * j.crot;
            j.axes[0] = r.c0;
            j.axes[1] = r.c1;
            j.axes[2] = r.c2;
            break;
        }
        default: break;
    }
}

__device__ inline void joint_warm(const JBodies& B, JointDev& j) {
    const uint32_t a = j.a, b = j.b;
    switch (j.type) {
        case kJointPoint: apply_impulse(B, a, b, j.r0, j.r1, j.imp1); break;
        case kJointDistance: apply_impulse(B, a, b, j.r0, j.r1, j.axis * j.dimp); break;
        case kJointFixed:
            apply_impulse(B, a, b, j.r0, j.r1, j.imp1);
            apply_angular(B, a, b, j.imp2);
            break;
        case kJointHinge:
            apply_impulse(B, a, b, j.r0, j.r1, j.imp1);
            for (int i = 0; i < 2; ++i) apply_angular(B, a, b, B.rot(a).rotate(j.lpa[i]) * j.simp[i]);
            apply_angular(B, a, b, B.rot(a).rotate(j.lax) * (j.limit_imp + j.motor_imp));
            break;
        case kJointSlider:
            apply_impulse(B, a, b, j.r0, j.r1, j.imp1);
            apply_angular(B, a, b, j.imp2);
            apply_impulse(B, a, b, j.r0, j.r1, B.rot(a).rotate(j.lax) * j.axial_imp);
            break;
        case kJointSixDof:
            for (int i = 0; i < 3; ++i) {
                apply_impulse(B, a, b, j.r0, j.r1, j.lin_imp[i]);
                apply_angular(B, a, b, j.ang_imp[i]);
            }
            break;
        default: break;
    }
}

__device__ inline void joint_velocity(const JBodies& B, JointDev& j) {
    const uint32_t a = j.a, b = j.b;
    switch (j.type) {
        case kJointPoint: {
            const Vec3 imp = j.m1 * (-rel_vel(B, j));
            j.imp1 = j.imp1 + imp;
            apply_impulse(B, a, b, j.r0, j.r1, imp);
            break;
        }
        case kJointDistance: {
            const float lambda = -j.dmass * rel_vel(B, j).dot(j.axis);
            j.dimp += lambda;
            apply_impulse(B, a, b, j.r0, j.r1, j.axis * lambda);
            break;
        }
        case kJointFixed: {
            const Vec3 li = j.m1 * (-rel_vel(B, j));
            j.imp1 = j.imp1 + li;
            apply_impulse(B, a, b, j.r0, j.r1, li);
            const Vec3 ai = j.m2 * (-(B.av(a) - B.av(b)));
            j.imp2 = j.imp2 + ai;
            apply_angular(B, a, b, ai);
            break;
        }
        case kJointHinge: {
            const Vec3 li = j.m1 * (-rel_vel(B, j));
            j.imp1 = j.imp1 + li;
            apply_impulse(B, a, b, j.r0, j.r1, li);
            const Vec3 wrel = B.av(a) - B.av(b);
            for (int i = 0; i < 2; ++i) {
                const Vec3 axis = B.rot(a).rotate(j.lpa[i]);
                const float lambda = -j.sm[i] * wrel.dot(axis);
                j.simp[i] += lambda;
                apply_angular(B, a, b, axis * lambda);
            }
            if (j.flags & kJointMotor) {
                const Vec3 ha = B.rot(a).rotate(j.lax);
                const float rv = (B.av(a) - B.av(b)).dot(ha);
                float lambda = j.limit_mass * (j.motor_target - rv);
                const float ni = rclamp(j.motor_imp + lambda, -j.motor_max, j.motor_max);
                lambda = ni - j.motor_imp;
                j.motor_imp = ni;
                apply_angular(B, a, b, ha * lambda);
            }
            if (j.flags & kJointLimits) {
                const Vec3 ha = B.rot(a).rotate(j.lax);
                const float angle = hinge_angle(B, j);
                const float rv = (B.av(a) - B.av(b)).dot(ha);
                float lambda = 0.0f;
                if (angle <= j.lower) {
                    lambda = j.limit_mass * (-rv);
                    j.limit_imp = rmax(j.limit_imp + lambda, 0.0f);
                    lambda = j.limit_imp;
                } else if (angle >= j.upper) {
                    lambda = j.limit_mass * (-rv);
                    j.limit_imp = rmin(j.limit_imp + lambda, 0.0f);
                    lambda = j.limit_imp;
                } else {
                    j.limit_imp = 0.0f;
                    lambda = 0.0f;
                }
                if (lambda != 0.0f) apply_angular(B, a, b, ha * lambda);
            }
            break;
        }
        case kJointSlider: {
            const Vec3 axis = B.rot(a).rotate(j.lax);
            const Vec3 vr = rel_vel(B, j);
            const Vec3 vp = vr - axis * vr.dot(axis);
            const Vec3 pi = -(j.m1 * vp);
            j.imp1 = j.imp1 + pi;
            apply_impulse(B, a, b, j.r0, j.r1, pi);
            const Vec3 ai = j.m2 * (-(B.av(a) - B.av(b)));
            j.imp2 = j.imp2 + ai;
            apply_angular(B, a, b, ai);
            const float rel = (B.lv(a) - B.lv(b)).dot(axis);
            if (j.flags & kJointMotor) {
                float lambda = j.axial_mass * (j.motor_target - rel);
                const float ni = rclamp(j.motor_imp + lambda, -j.motor_max, j.motor_max);
                lambda = ni - j.motor_imp;
                j.motor_imp = ni;
                apply_impulse(B, a, b, j.r0, j.r1, axis * lambda);
            } else if (j.flags & kJointLimits) {
                const Quat qa = B.rot(a);
                const Vec3 ra = qa.rotate(j.la), rb = B.rot(b).rotate(j.lb);
                const float pos = ((B.pos(b) + rb) - (B.pos(a) + ra)).dot(axis);
                float lambda = 0.0f;
                if (pos <= j.lower) {
                    lambda = j.axial_mass * (-rel);
                    j.axial_imp = rmax(j.axial_imp + lambda, 0.0f);
                    lambda = j.axial_imp;
                } else if (pos >= j.upper) {
                    lambda = j.axial_mass * (-rel);
                    j.axial_imp = rmin(j.axial_imp + lambda, 0.0f);
                    lambda = j.axial_imp;
                } else {
                    j.axial_imp = 0.0f;
                }
                if (lambda != 0.0f) apply_impulse(B, a, b, j.r0, j.r1, axis * lambda);
            }
            break;
        }
        case kJointSixDof: {
            for (int k = 0; k < 3; ++k) {  // SolveLinearAxis (Constraints.cpp:503-536)
                const uint32_t mode = (j.modes >> (2 * k)) & 3u;
                const bool motor = (j.motors >> k) & 1u;
                if (mode == 0u && !motor) continue;
                const Vec3 dir = j.axes[k];
                const float rel = rel_vel(B, j).dot(dir);
                const float mass = linear_mass(B, a, b, j.r0, j.r1, dir);
                float target = 0.0f;
                float lambda = mass * (target - rel);
                if (motor) {
                    target = j.six[k];
                    lambda = mass * (target - rel);
                    const float mx = j.six[3 + k];
                    const float acc = j.lin_imp[k].dot(dir);
                    const float na = rclamp(acc + lambda, -mx, mx);
                    lambda = na - acc;
                } else if (mode == 2u) {
                    lambda = mass * (-rel);
                }
                const Vec3 imp = dir * lambda;
                j.lin_imp[k] = j.lin_imp[k] + imp;
                apply_impulse(B, a, b, j.r0, j.r1, imp);
            }
            for (int k = 0; k < 3; ++k) {  // SolveAngularAxis (Constraints.cpp:538-557)
                const uint32_t mode = (j.modes >> (2 * k + 6)) & 3u;
                const bool motor = (j.motors >> (3 + k)) & 1u;
                if (mode == 0u && !motor) continue;
                const Vec3 dir = j.axes[k];
                const float rel = (B.av(a) - B.av(b)).dot(dir);
                const float mass = angular_mass(B, a, b, dir);
                float lambda;
                if (motor) {
                    lambda = mass * (j.six[6 + k] - rel);
                    const float acc = j.ang_imp[k].dot(dir);
                    const float na = rclamp(acc + lambda, -j.six[9 + k], j.six[9 + k]);
                    lambda = na - acc;
                } else {
                    lambda = mass * (-rel);
                }
                const Vec3 imp = dir * lambda;
                j.ang_imp[k] = j.ang_imp[k] + imp;
                apply_angular(B, a, b, imp);
            }
            break;
        }
        default: break;
    }
}

__device__ inline void joint_position(const JBodies& B, JointDev& j) {
    const uint32_t a = j.a, b = j.b;
    const Vec3 ra = B.rot(a).rotate(j.la), rb = B.rot(b).rotate(j.lb);
    switch (j.type) {
        case kJointPoint: {
            const Vec3 err = (B.pos(a) + ra) - (B.pos(b) + rb);
            const float slop = 0.001f;
            if (err.len2() < slop * slop) return;
            const Vec3 imp = m_inverse(point_mass(B, a, b, ra, rb)) * (-err);
            apply_positional(B, a, b, imp, ra.cross(imp));
            break;
        }
        case kJointDistance: {
            const Vec3 d = (B.pos(b) + rb) - (B.pos(a) + ra);
            const float dist = d.len();
            if (dist < kEps) return;
            const Vec3 axis = d / dist;
            const float err = dist - j.target;
            const float k = linear_mass(B, a, b, ra, rb, axis);
            const float lambda = -k * err * 0.2f;
            apply_positional(B, a, b, axis * lambda, Vec3());
            break;
        }
        case kJointFixed:
        case kJointHinge: {
            const Vec3 err = (B.pos(a) + ra) - (B.pos(b) + rb);
            if (err.len2() > 1.0e-8f) {
                const Vec3 imp = (m_inverse(point_mass(B, a, b, ra, rb)) * (-err)) * 0.2f;
                apply_positional(B, a, b, imp, ra.cross(imp));
            }
            if (j.type == kJointHinge) break;
            const Quat cur = q_conj(B.rot(a)) * B.rot(b);
            Quat diff = cur * q_conj(j.relrot);
            if (diff.w < 0.0f) diff = Quat(-diff.x, -diff.y, -diff.z, -diff.w);
            const float s = sqrtf(rmax(0.0f, 1.0f - diff.w * diff.w));
            const Vec3 axis = s >= kEps ? Vec3(diff.x, diff.y, diff.z) / s : Vec3(1.0f, 0.0f, 0.0f);
            const float angle = 2.0f * jacos(rclamp(diff.w, -1.0f, 1.0f));
            if (rabs(angle) > 1.0e-4f) {
                const Vec3 imp = (m_inverse(m_add(B.iiw(a), B.iiw(b))) * (-(axis * angle))) * 0.2f;
                apply_positional(B, a, b, Vec3(), imp);
            }
            break;
        }
        case kJointSlider: {
            const Vec3 axis = B.rot(a).rotate(j.lax);
            Vec3 err = (B.pos(a) + ra) - (B.pos(b) + rb);
            err = err - axis * err.dot(axis);
            if (err.len2() > 1.0e-8f) {
                Vec3 imp = (m_inverse(point_mass(B, a, b, ra, rb)) * (-err)) * 0.2f;
                imp = imp - axis * imp.dot(axis);
                apply_positional(B, a, b, imp, ra.cross(imp));
            }
            break;
        }
        case kJointSixDof: {
            const Vec3 err = (B.pos(a) + ra) - (B.pos(b) + rb);
            for (int k = 0; k < 3; ++k) {
                if (((j.modes >> (2 * k)) & 3u) != 2u) continue;
                const Vec3 dir = j.axes[k];
                const float e = err.dot(dir);
                if (rabs(e) < 1.0e-4f) continue;
                const float mass = linear_mass(B, a, b, ra, rb, dir);
                const Vec3 imp = dir * (-mass * e * 0.2f);
                apply_positional(B, a, b, imp, ra.cross(imp));
            }
            break;
        }
        default: break;
    }
}

}  // namespace kzg
