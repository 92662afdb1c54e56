// kzg_math.cuh - float vector math with the reference's rounding points.
//
// Every operation reproduces the evaluation order of the reference's Math.h / Math.cpp
// (include/Kizuri/Core/Math.h, src/Core/Math.cpp; Real = float, Types.h:18-22).  The library is
// compiled with --fmad=false (device) and -ffp-contract=off (host) and IEEE division / square
// root, so results are bit-identical to the reference's x86 SSE build.  Comparisons use the
// reference's ternary forms (math::Min/Max/Clamp, Types.h:52-55), not fminf/fmaxf, whose
// signed-zero and NaN behaviour differs.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define KZG_HD __host__ __device__ __forceinline__
#else
#define KZG_HD inline
#endif

namespace kzg {

constexpr float kEps = 1.1920928955078125e-7f;  // math::kEpsilon

KZG_HD float rmin(float a, float b) { return a < b ? a : b; }
KZG_HD float rmax(float a, float b) { return a > b ? a : b; }
KZG_HD float rclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
KZG_HD float rabs(float v) { return v < 0.0f ? -v : v; }
KZG_HD float rsqrt_ieee(float v) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(v);
#else
    return std::sqrt(v);
#endif
}
KZG_HD bool rfinite(float v) {
#ifdef __CUDA_ARCH__
    return isfinite(v);
#else
    return std::isfinite(v);
#endif
}
KZG_HD float rdiv(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

struct Vec3 {
    float x, y, z;
    KZG_HD Vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    KZG_HD Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    KZG_HD float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    KZG_HD void set(int i, float v) {
        if (i == 0) x = v; else if (i == 1) y = v; else z = v;
    }
    KZG_HD Vec3 operator-() const { return Vec3(-x, -y, -z); }
    KZG_HD Vec3 operator+(const Vec3& o) const { return Vec3(x + o.x, y + o.y, z + o.z); }
    KZG_HD Vec3 operator-(const Vec3& o) const { return Vec3(x - o.x, y - o.y, z - o.z); }
    KZG_HD Vec3 operator*(float s) const { return Vec3(x * s, y * s, z * s); }
    KZG_HD Vec3 mul(const Vec3& o) const { return Vec3(x * o.x, y * o.y, z * o.z); }
    // Vec3::operator/(Real): one reciprocal, three products (Math.h:39).
    KZG_HD Vec3 operator/(float s) const {
        float inv = rdiv(1.0f, s);
        return Vec3(x * inv, y * inv, z * inv);
    }
    KZG_HD float dot(const Vec3& o) const { return x * o.x + y * o.y + z * o.z; }
    KZG_HD float len2() const { return x * x + y * y + z * z; }
    KZG_HD float len() const { return rsqrt_ieee(len2()); }
    KZG_HD Vec3 cross(const Vec3& o) const {
        return Vec3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    KZG_HD Vec3 abs() const { return Vec3(rabs(x), rabs(y), rabs(z)); }
    KZG_HD Vec3 vmin(const Vec3& o) const { return Vec3(rmin(x, o.x), rmin(y, o.y), rmin(z, o.z)); }
    KZG_HD Vec3 vmax(const Vec3& o) const { return Vec3(rmax(x, o.x), rmax(y, o.y), rmax(z, o.z)); }
    KZG_HD int max_comp_index() const { return x >= y ? (x >= z ? 0 : 2) : (y >= z ? 1 : 2); }
    KZG_HD Vec3 normalized() const {
        float l = len();
        return l >= kEps ? *this / l : Vec3();
    }
    KZG_HD Vec3 normalized_or(const Vec3& fb) const {
        float l = len();
        return l >= kEps ? *this / l : fb;
    }
    KZG_HD bool finite() const { return rfinite(x) && rfinite(y) && rfinite(z); }
    // GetNormalizedPerpendicular (Math.h:102-110)
    KZG_HD Vec3 perp_normalized() const {
        if (rabs(x) > rabs(y)) {
            float l = rsqrt_ieee(x * x + z * z);
            return Vec3(rdiv(-z, l), 0.0f, rdiv(x, l));
        }
        float l = rsqrt_ieee(y * y + z * z);
        return Vec3(0.0f, rdiv(z, l), rdiv(-y, l));
    }
};

KZG_HD Vec3 lerp(const Vec3& a, const Vec3& b, float t) { return a + (b - a) * t; }
// ClampLength (Math.h:130-133)
KZG_HD Vec3 clamp_length(const Vec3& v, float m) {
    float l = v.len();
    return (l > m && l >= kEps) ? v * rdiv(m, l) : v;
}

// Column-major 3x3 (Math.h:167-242).
struct Mat3 {
    Vec3 c0, c1, c2;
    KZG_HD Vec3 operator*(const Vec3& v) const { return (c0 * v.x + c1 * v.y) + c2 * v.z; }
    KZG_HD Mat3 operator*(const Mat3& o) const { return Mat3{(*this) * o.c0, (*this) * o.c1, (*this) * o.c2}; }
    KZG_HD Mat3 transposed() const {
        return Mat3{Vec3(c0.x, c1.x, c2.x), Vec3(c0.y, c1.y, c2.y), Vec3(c0.z, c1.z, c2.z)};
    }
};

struct Quat {
    float x, y, z, w;
    KZG_HD Quat() : x(0.0f), y(0.0f), z(0.0f), w(1.0f) {}
    KZG_HD Quat(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    // Quat::operator*(Quat), Math.h:271-277
    KZG_HD Quat operator*(const Quat& q) const {
        return Quat(w * q.x + x * q.w + y * q.z - z * q.y, w * q.y - x * q.z + y * q.w + z * q.x,
                    w * q.z + x * q.y - y * q.x + z * q.w, w * q.w - x * q.x - y * q.y - z * q.z);
    }
    KZG_HD Quat operator+(const Quat& q) const { return Quat(x + q.x, y + q.y, z + q.z, w + q.w); }
    KZG_HD Quat scaled(float s) const { return Quat(x * s, y * s, z * s, w * s); }
    KZG_HD Quat normalized() const {
        float l = rsqrt_ieee(x * x + y * y + z * z + w * w);
        return l >= kEps ? scaled(rdiv(1.0f, l)) : Quat();
    }
    // Rotate / InverseRotate (Math.h:296-307): t = 2 (q x v); v + w t + q x t
    KZG_HD Vec3 rotate(const Vec3& v) const {
        Vec3 qv(x, y, z);
        Vec3 t = qv.cross(v) * 2.0f;
        return (v + t * w) + qv.cross(t);
    }
    KZG_HD Vec3 inv_rotate(const Vec3& v) const {
        Vec3 qv(-x, -y, -z);
        Vec3 t = qv.cross(v) * 2.0f;
        return (v + t * w) + qv.cross(t);
    }
    // ToMat3 (Math.h:314-322)
    KZG_HD Mat3 to_mat3() const {
        float xx = x * x, yy = y * y, zz = z * z;
        float xy = x * y, xz = x * z, yz = y * z;
        float wx = w * x, wy = w * y, wz = w * z;
        return Mat3{Vec3(1.0f - 2.0f * (yy + zz), 2.0f * (xy + wz), 2.0f * (xz - wy)),
                    Vec3(2.0f * (xy - wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz + wx)),
                    Vec3(2.0f * (xz + wy), 2.0f * (yz - wx), 1.0f - 2.0f * (xx + yy))};
    }
};

// q' = normalize(q + (0.5 dt w, 0) q)  (PhysicsWorld.cpp:31-35)
KZG_HD Quat integrate_rotation(const Quat& q, const Vec3& w, float dt) {
    Quat dq(0.5f * dt * w.x, 0.5f * dt * w.y, 0.5f * dt * w.z, 0.0f);
    return (q + dq * q).normalized();
}

// Transform * point (Math.h:363)
KZG_HD Vec3 xform(const Quat& q, const Vec3& t, const Vec3& p) { return q.rotate(p) + t; }

struct AABB {
    Vec3 mn, mx;
};
KZG_HD AABB aabb_merge(const AABB& a, const AABB& b) { return AABB{a.mn.vmin(b.mn), a.mx.vmax(b.mx)}; }
KZG_HD bool aabb_overlaps(const AABB& a, const AABB& o) {
    return a.mn.x <= o.mx.x && a.mx.x >= o.mn.x && a.mn.y <= o.mx.y && a.mx.y >= o.mn.y && a.mn.z <= o.mx.z &&
           a.mx.z >= o.mn.z;
}
// AABB::Transformed(Transform) (Math.cpp:176-189)
KZG_HD AABB aabb_transformed(const AABB& b, const Quat& q, const Vec3& t) {
    Vec3 c = (b.mn + b.mx) * 0.5f;
    Vec3 e = (b.mx - b.mn) * 0.5f;
    Mat3 m = q.to_mat3();
    Vec3 nc = xform(q, t, c);
    Vec3 ne(rabs(m.c0.x) * e.x + rabs(m.c1.x) * e.y + rabs(m.c2.x) * e.z,
            rabs(m.c0.y) * e.x + rabs(m.c1.y) * e.y + rabs(m.c2.y) * e.z,
            rabs(m.c0.z) * e.x + rabs(m.c1.z) * e.y + rabs(m.c2.z) * e.z);
    return AABB{nc - ne, nc + ne};
}

// float4 storage <-> math types (device buffers keep vectors as float4)
__device__ __forceinline__ Vec3 V3(float4 a) { return Vec3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 F4(const Vec3& v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ Quat Q4(float4 a) { return Quat(a.x, a.y, a.z, a.w); }
__device__ __forceinline__ float4 F4q(const Quat& q) { return make_float4(q.x, q.y, q.z, q.w); }
__device__ __forceinline__ Mat3 M3(const float4* c) { return Mat3{V3(c[0]), V3(c[1]), V3(c[2])}; }

}  // namespace kzg
