/* Oracle (test infrastructure only): float vector math restated op-for-op from the
 * reference's include/Kizuri/Core/Math.h and src/Core/Math.cpp.
 *
 * Every expression keeps the reference's evaluation order and float rounding points
 * (Real = float, Types.h:18-22).  Build with -ffp-contract=off so no a*b+c is fused.
 * Nothing in the product links or includes this file.
 */
#ifndef KZO_MATH_H
#define KZO_MATH_H

#include <math.h>
#include <stdint.h>

#define KZO_EPS 1.1920928955078125e-7f /* math::kEpsilon, Types.h:43 */

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } qt;
typedef struct { v3 c[3]; } m3; /* column-major (Math.h:167-169) */
typedef struct { v3 mn, mx; } aabb;

static inline float fmin_r(float a, float b) { return a < b ? a : b; }   /* math::Min, Types.h:53 */
static inline float fmax_r(float a, float b) { return a > b ? a : b; }   /* math::Max, Types.h:54 */
static inline float fclamp_r(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline float fabs_r(float v) { return v < 0.0f ? -v : v; }        /* math::Abs, Types.h:52 */

static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline v3 vmul(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vmulv(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
/* Vec3::operator/(Real): multiply by the reciprocal (Math.h:39). */
static inline v3 vdiv(v3 a, float s) { float inv = 1.0f / s; return V(a.x * inv, a.y * inv, a.z * inv); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float vlen2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline float vlen(v3 a) { return sqrtf(vlen2(a)); }
static inline v3 vcross(v3 a, v3 b) {
    return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 vabs(v3 a) { return V(fabs_r(a.x), fabs_r(a.y), fabs_r(a.z)); }
static inline v3 vmin(v3 a, v3 b) { return V(fmin_r(a.x, b.x), fmin_r(a.y, b.y), fmin_r(a.z, b.z)); }
static inline v3 vmax(v3 a, v3 b) { return V(fmax_r(a.x, b.x), fmax_r(a.y, b.y), fmax_r(a.z, b.z)); }
static inline float vget(v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline void vset(v3* a, int i, float s) { if (i == 0) a->x = s; else if (i == 1) a->y = s; else a->z = s; }
/* Normalized / NormalizedOr (Math.h:58-72). */
static inline v3 vnormalized(v3 a) { float l = vlen(a); return l >= KZO_EPS ? vdiv(a, l) : V(0, 0, 0); }
static inline v3 vnormalized_or(v3 a, v3 fb) { float l = vlen(a); return l >= KZO_EPS ? vdiv(a, l) : fb; }
static inline int vmax_comp_index(v3 a) { return a.x >= a.y ? (a.x >= a.z ? 0 : 2) : (a.y >= a.z ? 1 : 2); }
static inline v3 vlerp(v3 a, v3 b, float t) { return vadd(a, vmul(vsub(b, a), t)); }
static inline int visfinite(v3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
/* ClampLength, Math.h:130-133 */
static inline v3 vclamp_len(v3 v, float maxl) {
    float l = vlen(v);
    return (l > maxl && l >= KZO_EPS) ? vmul(v, maxl / l) : v;
}
/* GetNormalizedPerpendicular, Math.h:102-110 */
static inline v3 vperp_normalized(v3 a) {
    if (fabs_r(a.x) > fabs_r(a.y)) {
        float len = sqrtf(a.x * a.x + a.z * a.z);
        return V(-a.z / len, 0.0f, a.x / len);
    } else {
        float len = sqrtf(a.y * a.y + a.z * a.z);
        return V(0.0f, a.z / len, -a.y / len);
    }
}

/* Mat3 * Vec3 = col0*v.x + col1*v.y + col2*v.z (Math.h:216). */
static inline v3 mmulv(const m3* m, v3 v) {
    return vadd(vadd(vmul(m->c[0], v.x), vmul(m->c[1], v.y)), vmul(m->c[2], v.z));
}
static inline m3 mmul(const m3* a, const m3* b) {
    m3 r; r.c[0] = mmulv(a, b->c[0]); r.c[1] = mmulv(a, b->c[1]); r.c[2] = mmulv(a, b->c[2]); return r;
}
static inline m3 mtranspose(const m3* m) {
    m3 r;
    r.c[0] = V(m->c[0].x, m->c[1].x, m->c[2].x);
    r.c[1] = V(m->c[0].y, m->c[1].y, m->c[2].y);
    r.c[2] = V(m->c[0].z, m->c[1].z, m->c[2].z);
    return r;
}

static inline qt Q(float x, float y, float z, float w) { qt q = {x, y, z, w}; return q; }
/* Quat::operator*(Quat), Math.h:271-277 */
static inline qt qmul(qt a, qt q) {
    return Q(a.w * q.x + a.x * q.w + a.y * q.z - a.z * q.y,
             a.w * q.y - a.x * q.z + a.y * q.w + a.z * q.x,
             a.w * q.z + a.x * q.y - a.y * q.x + a.z * q.w,
             a.w * q.w - a.x * q.x - a.y * q.y - a.z * q.z);
}
static inline qt qscale(qt a, float s) { return Q(a.x * s, a.y * s, a.z * s, a.w * s); }
static inline qt qadd(qt a, qt b) { return Q(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
/* Quat::Normalized, Math.h:290-293 */
static inline qt qnormalized(qt a) {
    float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w);
    return l >= KZO_EPS ? qscale(a, 1.0f / l) : Q(0, 0, 0, 1);
}
/* Quat::Rotate / InverseRotate, Math.h:296-307 */
static inline v3 qrotate(qt q, v3 v) {
    v3 qv = V(q.x, q.y, q.z);
    v3 t = vmul(vcross(qv, v), 2.0f);
    return vadd(vadd(v, vmul(t, q.w)), vcross(qv, t));
}
static inline v3 qinv_rotate(qt q, v3 v) {
    v3 qv = V(-q.x, -q.y, -q.z);
    v3 t = vmul(vcross(qv, v), 2.0f);
    return vadd(vadd(v, vmul(t, q.w)), vcross(qv, t));
}
/* Quat::ToMat3, Math.h:314-322 */
static inline m3 qtomat(qt q) {
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    m3 m;
    m.c[0] = V(1.0f - 2.0f * (yy + zz), 2.0f * (xy + wz), 2.0f * (xz - wy));
    m.c[1] = V(2.0f * (xy - wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz + wx));
    m.c[2] = V(2.0f * (xz + wy), 2.0f * (yz - wx), 1.0f - 2.0f * (xx + yy));
    return m;
}
/* IntegrateRotation, PhysicsWorld.cpp:31-35 */
static inline qt q_integrate(qt q, v3 w, float dt) {
    qt dq = Q(0.5f * dt * w.x, 0.5f * dt * w.y, 0.5f * dt * w.z, 0.0f);
    return qnormalized(qadd(q, qmul(dq, q)));
}

/* Transform * point = rotation.Rotate(p) + translation (Math.h:363). */
static inline v3 xform(qt q, v3 t, v3 p) { return vadd(qrotate(q, p), t); }

/* AABB helpers (Math.h:390-449, Math.cpp:176-189). */
static inline aabb AB(v3 mn, v3 mx) { aabb r = {mn, mx}; return r; }
static inline aabb aabb_empty(void) { return AB(V(INFINITY, INFINITY, INFINITY), V(-INFINITY, -INFINITY, -INFINITY)); }
static inline aabb aabb_merge(aabb a, aabb b) { return AB(vmin(a.mn, b.mn), vmax(a.mx, b.mx)); }
static inline int aabb_overlaps(aabb a, aabb o) {
    return a.mn.x <= o.mx.x && a.mx.x >= o.mn.x && a.mn.y <= o.mx.y && a.mx.y >= o.mn.y &&
           a.mn.z <= o.mx.z && a.mx.z >= o.mn.z;
}
static inline int aabb_contains(aabb a, aabb o) {
    return a.mn.x <= o.mn.x && a.mx.x >= o.mx.x && a.mn.y <= o.mn.y && a.mx.y >= o.mx.y &&
           a.mn.z <= o.mn.z && a.mx.z >= o.mx.z;
}
static inline float aabb_area(aabb a) {
    v3 d = vsub(a.mx, a.mn);
    return 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
}
static inline aabb aabb_transformed(aabb b, qt q, v3 t) {
    v3 c = vmul(vadd(b.mn, b.mx), 0.5f);
    v3 e = vmul(vsub(b.mx, b.mn), 0.5f);
    m3 m = qtomat(q);
    v3 nc = xform(q, t, c);
    v3 ne = V(fabs_r(m.c[0].x) * e.x + fabs_r(m.c[1].x) * e.y + fabs_r(m.c[2].x) * e.z,
              fabs_r(m.c[0].y) * e.x + fabs_r(m.c[1].y) * e.y + fabs_r(m.c[2].y) * e.z,
              fabs_r(m.c[0].z) * e.x + fabs_r(m.c[1].z) * e.y + fabs_r(m.c[2].z) * e.z);
    return AB(vsub(nc, ne), vadd(nc, ne));
}

#endif
