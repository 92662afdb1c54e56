// kzg_narrow.cuh - device narrow phase: one thread computes one pair's manifold.
//
// Follows the reference's NarrowPhase::Collide routing and numerics
// (src/Collision/CollideShape.cpp:30-430, 480-592; GJK src/Collision/GJK.cpp:11-244;
// EPA src/Collision/EPA.cpp:16-296; support functions include/Kizuri/Geometry/Shape.h:152-226
// and src/Geometry/Shapes.cpp:538-547).  Iteration caps, tolerances, tie-breaks (first maximum /
// first minimum wins) and polytope face order are the reference's, so manifolds match it bit
// for bit.  Shapes supported on the device: sphere, box, capsule, convex hull, plane.
#pragma once

#include "kzg_math.cuh"

namespace kzg {

enum : uint32_t { kSphere = 0, kBox = 1, kCapsule = 2, kHull = 4, kPlane = 8 };

// Device shape record: 64 bytes.
struct ShapeDev {
    uint32_t type, vfirst, vnum, ffirst, fnum, ifirst, inum, pad0;
    float p[4];
    float lmn[3], lmx[3];
    float pad1[2];
};

// Read-only view of the shape tables.
struct ShapeTables {
    const ShapeDev* shapes;
    const float4* hull_verts;
    const uint8_t* face_sizes;
    const uint32_t* face_idx;
};

constexpr uint32_t kMaxManifold = 4;  // every routine here reduces to at most 4 points

struct ContactPt {
    Vec3 pA, pB, n;
    float sep;
    uint32_t feature;
};

struct Manifold {
    ContactPt pts[kMaxManifold];
    uint32_t n;
};

struct SP {  // SupportPoint (GJK.h:108-118)
    Vec3 pA, pB, p;
};

struct Body {  // pose + shape of one side of a pair
    const ShapeDev* s;
    Quat q;
    Vec3 t;
};

__device__ __forceinline__ Vec3 hv(const ShapeTables& T, uint32_t i) {
    float4 v = __ldg(&T.hull_verts[i]);
    return Vec3(v.x, v.y, v.z);
}

__device__ inline Vec3 support_local(const ShapeTables& T, const ShapeDev* s, const Vec3& d) {
    switch (s->type) {
        case kSphere: return d.normalized_or(Vec3(0.0f, 1.0f, 0.0f)) * s->p[0];
        case kBox:
            return Vec3(d.x >= 0.0f ? s->p[0] : -s->p[0], d.y >= 0.0f ? s->p[1] : -s->p[1],
                        d.z >= 0.0f ? s->p[2] : -s->p[2]);
        case kCapsule: {
            float sg = d.y >= 0.0f ? s->p[0] : -s->p[0];
            return Vec3(0.0f, sg, 0.0f) + d.normalized_or(Vec3(0.0f, 1.0f, 0.0f)) * s->p[1];
        }
        case kHull: {
            float best_dot = -INFINITY;
            Vec3 best = hv(T, s->vfirst);
            for (uint32_t i = 0; i < s->vnum; ++i) {
                Vec3 v = hv(T, s->vfirst + i);
                float dd = v.dot(d);
                if (dd > best_dot) { best_dot = dd; best = v; }
            }
            return best;
        }
        case kPlane: return Vec3(s->p[0], s->p[1], s->p[2]) * s->p[3] + d * 1.0e6f;
        default: return Vec3();
    }
}

struct SupportMap {
    const ShapeTables* T;
    Body a, b;
    __device__ SP operator()(const Vec3& d) const {
        Vec3 la = a.q.inv_rotate(d);
        Vec3 lb = b.q.inv_rotate(-d);
        SP sp;
        sp.pA = xform(a.q, a.t, support_local(*T, a.s, la));
        sp.pB = xform(b.q, b.t, support_local(*T, b.s, lb));
        sp.p = sp.pA - sp.pB;
        return sp;
    }
};

// ---------------------------------------------------------------------------------------------
// GJK (GJK.cpp:11-244)
// ---------------------------------------------------------------------------------------------
__device__ inline Vec3 closest_on_triangle(const Vec3& p, const Vec3& a, const Vec3& b, const Vec3& c, float& u,
                                           float& v, float& w) {
    Vec3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = ab.dot(ap), d2 = ac.dot(ap);
    if (d1 <= 0.0f && d2 <= 0.0f) { u = 1.0f; v = 0.0f; w = 0.0f; return a; }
    Vec3 bp = p - b;
    float d3 = ab.dot(bp), d4 = ac.dot(bp);
    if (d3 >= 0.0f && d4 <= d3) { u = 0.0f; v = 1.0f; w = 0.0f; return b; }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float t = rdiv(d1, d1 - d3);
        u = 1.0f - t; v = t; w = 0.0f;
        return a + ab * t;
    }
    Vec3 cp = p - c;
    float d5 = ab.dot(cp), d6 = ac.dot(cp);
    if (d6 >= 0.0f && d5 <= d6) { u = 0.0f; v = 0.0f; w = 1.0f; return c; }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float t = rdiv(d2, d2 - d6);
        u = 1.0f - t; v = 0.0f; w = t;
        return a + ac * t;
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float t = rdiv(d4 - d3, (d4 - d3) + (d5 - d6));
        u = 0.0f; v = 1.0f - t; w = t;
        return b + (c - b) * t;
    }
    float denom = rdiv(1.0f, va + vb + vc);
    v = vb * denom;
    w = vc * denom;
    u = 1.0f - v - w;
    return (a + ab * v) + ac * w;
}

__device__ __forceinline__ bool gjk_outside(const Vec3& p0, const Vec3& p1, const Vec3& p2, const Vec3& opp) {
    Vec3 n = (p1 - p0).cross(p2 - p0);
    if (n.dot(opp - p0) > 0.0f) n = -n;
    return n.dot(Vec3() - p0) > 0.0f;
}

__device__ inline bool reduce_simplex(SP* s, uint32_t& count, Vec3& closest) {
    if (count == 1) {
        closest = s[0].p;
    } else if (count == 2) {
        Vec3 a = s[0].p, b = s[1].p, ab = b - a;
        float t = -a.dot(ab);
        if (t <= 0.0f) { closest = a; count = 1; }
        else if (t >= ab.len2()) { s[0] = s[1]; closest = b; count = 1; }
        else { closest = a + ab * rdiv(t, ab.len2()); }
    } else if (count == 3) {
        float u, v, w;
        closest = closest_on_triangle(Vec3(), s[0].p, s[1].p, s[2].p, u, v, w);
        SP k[3] = {SP{}, SP{}, SP{}};
        uint32_t n = 0;
        if (u > 0.0f) k[n++] = s[0];
        if (v > 0.0f) k[n++] = s[1];
        if (w > 0.0f) k[n++] = s[2];
        if (n == 0) n = 1;
        for (uint32_t i = 0; i < n; ++i) s[i] = k[i];
        count = n;
    } else if (count == 4) {
        Vec3 a = s[0].p, b = s[1].p, c = s[2].p, d = s[3].p;
        bool o[4] = {gjk_outside(a, b, c, d), gjk_outside(a, c, d, b), gjk_outside(a, d, b, c),
                     gjk_outside(b, d, c, a)};
        if (!o[0] && !o[1] && !o[2] && !o[3]) return true;
        const uint8_t F[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
        float best = INFINITY;
        SP bt[3] = {SP{}, SP{}, SP{}};
        uint32_t bc = 0;
        for (int f = 0; f < 4; ++f) {
            if (!o[f]) continue;
            float u, v, w;
            Vec3 p = closest_on_triangle(Vec3(), s[F[f][0]].p, s[F[f][1]].p, s[F[f][2]].p, u, v, w);
            float d2 = p.len2();
            if (d2 < best) {
                best = d2;
                uint32_t n = 0;
                if (u > 0.0f) bt[n++] = s[F[f][0]];
                if (v > 0.0f) bt[n++] = s[F[f][1]];
                if (w > 0.0f) bt[n++] = s[F[f][2]];
                bc = n;
                closest = p;
            }
        }
        for (uint32_t i = 0; i < bc; ++i) s[i] = bt[i];
        count = bc;
    }
    return false;
}

struct GjkOut {
    bool intersect;
    float distance;
    Vec3 pA, pB, normal;
    uint32_t ns;
    SP simplex[4];
};

static __device__ __noinline__ void gjk(const SupportMap& map, float tol, uint32_t max_iter, GjkOut& r) {
    r.intersect = false;
    r.distance = 0.0f;
    r.pA = r.pB = r.normal = Vec3();
    SP s[4];
    uint32_t count = 0;
    s[count++] = map(Vec3(1.0f, 0.0f, 0.0f));
    Vec3 closest = s[0].p;
    const float tol2 = tol * tol;
    for (uint32_t it = 0; it < max_iter; ++it) {
        if (closest.len2() <= tol2) { r.intersect = true; r.distance = 0.0f; break; }
        Vec3 d = -closest;
        SP w = map(d);
        float progress = closest.len2() - closest.dot(w.p);
        if (progress <= tol * closest.len2()) break;
        bool dup = false;
        for (uint32_t i = 0; i < count; ++i)
            if ((s[i].p - w.p).len2() < tol2) { dup = true; break; }
        if (dup) break;
        s[count++] = w;
        if (reduce_simplex(s, count, closest)) { r.intersect = true; r.distance = 0.0f; break; }
    }
    r.ns = count;
    for (uint32_t i = 0; i < count; ++i) r.simplex[i] = s[i];
    if (!r.intersect) {
        float dist = closest.len();
        r.distance = dist;
        if (dist < kEps) r.intersect = true;
        else r.normal = (-closest) / dist;
        if (count == 1) {
            r.pA = s[0].pA; r.pB = s[0].pB;
        } else if (count == 2) {
            Vec3 a = s[0].p, b = s[1].p, ab = b - a;
            float t = rclamp(rdiv(-a.dot(ab), rmax(ab.len2(), kEps)), 0.0f, 1.0f);
            r.pA = lerp(s[0].pA, s[1].pA, t);
            r.pB = lerp(s[0].pB, s[1].pB, t);
        } else if (count == 3) {
            float u, v, w;
            closest_on_triangle(Vec3(), s[0].p, s[1].p, s[2].p, u, v, w);
            r.pA = (s[0].pA * u + s[1].pA * v) + s[2].pA * w;
            r.pB = (s[0].pB * u + s[1].pB * v) + s[2].pB * w;
        } else {
            r.pA = s[0].pA; r.pB = s[0].pB;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// EPA (EPA.cpp:16-296).  Polytope capacities are the reference's (256 vertices are never
// reached: 4 + 64 iterations; 512 faces; 256 horizon edges).
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kEpaVerts = 68;  // the initial tetrahedron + one vertex per iteration (64)
constexpr uint32_t kEpaFaces = 512;
constexpr uint32_t kEpaHorizon = 256;

struct EpaOut {
    bool valid;
    float depth;
    Vec3 normal, pA, pB;
};

__device__ __forceinline__ Vec3 epa_perp(const Vec3& v) {
    if (rabs(v.x) <= rabs(v.y) && rabs(v.x) <= rabs(v.z)) return Vec3(0.0f, -v.z, v.y);
    if (rabs(v.y) <= rabs(v.z)) return Vec3(-v.z, 0.0f, v.x);
    return Vec3(-v.y, v.x, 0.0f);
}

__device__ __forceinline__ bool tet_face_ok(const Vec3& a, const Vec3& b, const Vec3& c, const Vec3& d) {
    Vec3 n = (b - a).cross(c - a);
    if (n.dot(d - a) > 0.0f) n = -n;
    return n.dot(Vec3() - a) < -1.0e-9f;
}
__device__ __forceinline__ bool origin_in_tetra(const SP* v) {
    return tet_face_ok(v[0].p, v[1].p, v[2].p, v[3].p) && tet_face_ok(v[0].p, v[2].p, v[3].p, v[1].p) &&
           tet_face_ok(v[0].p, v[3].p, v[1].p, v[2].p) && tet_face_ok(v[1].p, v[3].p, v[2].p, v[0].p);
}

// Polytope of one EPA run, in shared memory, owned by one warp.
struct EpaWarpSmem {
    float vp[kEpaVerts][3], va[kEpaVerts][3], vb[kEpaVerts][3];  // SupportPoint p, pointA, pointB
    float fnx[kEpaFaces], fny[kEpaFaces], fnz[kEpaFaces], fd[kEpaFaces];
    uint8_t fa[kEpaFaces], fb[kEpaFaces], fc[kEpaFaces];
    uint32_t dead[kEpaFaces / 32];  // visible faces of the current iteration, one bit each
    uint32_t ebits[(kEpaVerts * kEpaVerts + 31) / 32];  // directed edges (u, v) of the visible faces
    uint16_t vis[kEpaFaces];
    uint8_t hu[kEpaHorizon], hv[kEpaHorizon];
};

__device__ __forceinline__ Vec3 sm_vp(const EpaWarpSmem& S, uint32_t i) { return Vec3(S.vp[i][0], S.vp[i][1], S.vp[i][2]); }

// BuildInitialTetra (EPA.cpp:58-147) for the warp EPA, every lane holding the same result.  The
// simplex-based attempts run on every lane; the fallback - the first tetrahedron, in the order of
// the reference's four nested loops, of up to 16 distinct candidate points (the simplex and 14
// support points) that has volume and holds the origin - is searched 32 combinations at a time,
// each lane testing one (its indices from the combination's rank in that order) and the smallest
// rank that passes winning.  On touching polyhedra (a box resting on a box) the simplex is
// degenerate and this search, up to 1,820 tetrahedra, is most of the pair's work.
struct TetraSmem {
    float p[18][3], pa[18][3], pb[18][3];  // the 14 support points, then the candidate list
    float cp[16][3], cpa[16][3], cpb[16][3];
};
static_assert(sizeof(TetraSmem) <= sizeof(EpaWarpSmem), "tetrahedron scratch overlays the EPA scratch");

__device__ __forceinline__ uint32_t choose3(uint32_t m) { return m < 3u ? 0u : m * (m - 1u) * (m - 2u) / 6u; }
__device__ __forceinline__ uint32_t choose2(uint32_t m) { return m < 2u ? 0u : m * (m - 1u) / 2u; }

static __device__ __noinline__ bool epa_initial_tetra_warp(const SupportMap& map, const GjkOut& g, SP* out,
                                                          EpaWarpSmem& scratch, uint32_t lane) {
    uint32_t n = 0;
    for (uint32_t i = 0; i < g.ns && n < 4; ++i) {
        bool dup = false;
        for (uint32_t j = 0; j < n; ++j)
            if ((out[j].p - g.simplex[i].p).len2() < 1.0e-12f) dup = true;
        if (!dup) out[n++] = g.simplex[i];
    }
    if (n == 0) out[n++] = map(Vec3(1.0f, 0.0f, 0.0f));
    if (n == 4 && !origin_in_tetra(out)) n = 3;
    if (n == 1) {
        out[n] = map(-out[0].p);
        if ((out[1].p - out[0].p).len2() > 1.0e-12f) ++n;
    }
    if (n == 2) {
        Vec3 ab = out[1].p - out[0].p;
        if (ab.len2() > 1.0e-12f) {
            Vec3 d1 = epa_perp(ab).normalized();
            Vec3 d2 = ab.cross(d1).normalized();
            SP k0 = out[0], k1 = out[1];
            out[0] = map(d1);
            out[1] = map(-d1);
            out[2] = map(d2);
            out[3] = map(-d2);
            if (origin_in_tetra(out)) return true;
            out[0] = k0;
            out[1] = k1;
        }
        SP s = map(epa_perp(ab));
        if ((s.p - out[0].p).len2() > 1.0e-12f && (s.p - out[1].p).len2() > 1.0e-12f) out[n++] = s;
    }
    if (n == 3) {
        Vec3 tn = (out[1].p - out[0].p).cross(out[2].p - out[0].p);
        float len = tn.len();
        if (len > 1.0e-12f) {
            tn = tn / len;
            float sd = tn.dot(Vec3() - out[0].p);
            SP a = map(sd > 0.0f ? -tn : tn);
            SP b = map(sd > 0.0f ? tn : -tn);
            out[3] = a;
            if (!origin_in_tetra(out)) out[3] = b;
            if (origin_in_tetra(out)) return true;
        }
        n = 3;
    }
    if (n == 4 && origin_in_tetra(out)) return true;

    TetraSmem& X = *reinterpret_cast<TetraSmem*>(&scratch);
    const float s = 0.5773502692f;
    const float D[14][3] = {{1, 0, 0},   {-1, 0, 0},  {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1}, {s, s, s},
                            {s, s, -s},  {s, -s, s},  {-s, s, s}, {-s, -s, s}, {-s, s, -s}, {s, -s, -s}, {-s, -s, -s}};
    __syncwarp();
    if (lane < 14u) {
        const SP sp = map(Vec3(D[lane][0], D[lane][1], D[lane][2]));
        X.p[lane][0] = sp.p.x; X.p[lane][1] = sp.p.y; X.p[lane][2] = sp.p.z;
        X.pa[lane][0] = sp.pA.x; X.pa[lane][1] = sp.pA.y; X.pa[lane][2] = sp.pA.z;
        X.pb[lane][0] = sp.pB.x; X.pb[lane][1] = sp.pB.y; X.pb[lane][2] = sp.pB.z;
    }
    __syncwarp();
    uint32_t nc = 0;
    if (lane == 0) {  // the candidate list in the reference's order, duplicates dropped
        auto add = [&](const Vec3& p, const Vec3& pa, const Vec3& pb) {
            for (uint32_t i = 0; i < nc; ++i)
                if ((Vec3(X.cp[i][0], X.cp[i][1], X.cp[i][2]) - p).len2() < 1.0e-12f) return;
            if (nc < 16) {
                X.cp[nc][0] = p.x; X.cp[nc][1] = p.y; X.cp[nc][2] = p.z;
                X.cpa[nc][0] = pa.x; X.cpa[nc][1] = pa.y; X.cpa[nc][2] = pa.z;
                X.cpb[nc][0] = pb.x; X.cpb[nc][1] = pb.y; X.cpb[nc][2] = pb.z;
                ++nc;
            }
        };
        for (uint32_t i = 0; i < g.ns && i < 4; ++i) add(g.simplex[i].p, g.simplex[i].pA, g.simplex[i].pB);
        for (uint32_t i = 0; i < 14; ++i)
            add(Vec3(X.p[i][0], X.p[i][1], X.p[i][2]), Vec3(X.pa[i][0], X.pa[i][1], X.pa[i][2]),
                Vec3(X.pb[i][0], X.pb[i][1], X.pb[i][2]));
    }
    nc = __shfl_sync(0xffffffffu, nc, 0);
    __syncwarp();
    auto cand = [&](uint32_t i) {
        SP r;
        r.p = Vec3(X.cp[i][0], X.cp[i][1], X.cp[i][2]);
        r.pA = Vec3(X.cpa[i][0], X.cpa[i][1], X.cpa[i][2]);
        r.pB = Vec3(X.cpb[i][0], X.cpb[i][1], X.cpb[i][2]);
        return r;
    };
    const uint32_t total = nc >= 4u ? nc * (nc - 1u) * (nc - 2u) * (nc - 3u) / 24u : 0u;
    for (uint32_t base = 0; base < total; base += 32u) {
        const uint32_t rank = base + lane;
        uint32_t i = 0, j = 0, k = 0, l = 0;
        bool ok = false;
        if (rank < total) {  // the rank-th (i < j < k < l) in the loops' order
            uint32_t r = rank;
            for (;; ++i) { const uint32_t c = choose3(nc - 1u - i); if (r < c) break; r -= c; }
            for (j = i + 1u;; ++j) { const uint32_t c = choose2(nc - 1u - j); if (r < c) break; r -= c; }
            for (k = j + 1u;; ++k) { const uint32_t c = nc - 1u - k; if (r < c) break; r -= c; }
            l = k + 1u + r;
            SP t[4] = {cand(i), cand(j), cand(k), cand(l)};
            float vol = (t[1].p - t[0].p).cross(t[2].p - t[0].p).dot(t[3].p - t[0].p);
            ok = !(rabs(vol) < 1.0e-12f) && origin_in_tetra(t);
        }
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (m) {
            const uint32_t w = (uint32_t)(__ffs(m) - 1);
            const uint32_t idx = __shfl_sync(0xffffffffu, i | (j << 8) | (k << 16) | (l << 24), w);
            out[0] = cand(idx & 0xFFu);
            out[1] = cand((idx >> 8) & 0xFFu);
            out[2] = cand((idx >> 16) & 0xFFu);
            out[3] = cand(idx >> 24);
            __syncwarp();
            return true;
        }
    }
    __syncwarp();
    return false;
}

// BuildFace (EPA.cpp:16-31) on vertices held in shared memory.
__device__ __forceinline__ bool epa_build_face_sm(uint32_t& fa, uint32_t& fb, uint32_t& fc, Vec3& n_out, float& d_out,
                                                  const EpaWarpSmem& S) {
    Vec3 A = sm_vp(S, fa), B = sm_vp(S, fb), C = sm_vp(S, fc);
    Vec3 n = (B - A).cross(C - A);
    float len = n.len();
    if (len < 1.0e-12f) return false;
    n = n / len;
    float d = n.dot(A);
    if (d < 0.0f) {
        n = -n;
        d = -d;
        uint32_t t = fb; fb = fc; fc = t;
    }
    n_out = n;
    d_out = d;
    return true;
}

__device__ __forceinline__ void sm_put_face(EpaWarpSmem& S, uint32_t k, uint32_t a, uint32_t b, uint32_t c, const Vec3& n,
                                            float d) {
    S.fa[k] = (uint8_t)a; S.fb[k] = (uint8_t)b; S.fc[k] = (uint8_t)c;
    S.fnx[k] = n.x; S.fny[k] = n.y; S.fnz[k] = n.z; S.fd[k] = d;
}

// FinishFace (EPA.cpp:163-172) for face k of the shared polytope.
__device__ inline void epa_finish_sm(const EpaWarpSmem& S, uint32_t k, EpaOut& r) {
    const Vec3 n(S.fnx[k], S.fny[k], S.fnz[k]);
    const float dist = S.fd[k];
    const uint32_t ia = S.fa[k], ib = S.fb[k], ic = S.fc[k];
    Vec3 proj = n * dist;
    Vec3 a = sm_vp(S, ia), b = sm_vp(S, ib), c = sm_vp(S, ic);
    Vec3 v0 = b - a, v1 = c - a, v2 = proj - a;
    float d00 = v0.dot(v0), d01 = v0.dot(v1), d11 = v1.dot(v1);
    float d20 = v2.dot(v0), d21 = v2.dot(v1);
    float denom = d00 * d11 - d01 * d01;
    float u, v, w;
    if (rabs(denom) < 1.0e-18f) { u = 1.0f; v = 0.0f; w = 0.0f; }
    else {
        v = rdiv(d11 * d20 - d01 * d21, denom);
        w = rdiv(d00 * d21 - d01 * d20, denom);
        u = 1.0f - v - w;
    }
    r.valid = true;
    r.depth = dist;
    r.normal = -n;
    const Vec3 Aa(S.va[ia][0], S.va[ia][1], S.va[ia][2]), Ba(S.va[ib][0], S.va[ib][1], S.va[ib][2]),
        Ca(S.va[ic][0], S.va[ic][1], S.va[ic][2]);
    const Vec3 Ab(S.vb[ia][0], S.vb[ia][1], S.vb[ia][2]), Bb(S.vb[ib][0], S.vb[ib][1], S.vb[ib][2]),
        Cb(S.vb[ic][0], S.vb[ic][1], S.vb[ic][2]);
    r.pA = (Aa * u + Ba * v) + Ca * w;
    r.pB = (Ab * u + Bb * v) + Cb * w;
}

// First face with the smallest distance (EPA.cpp:212-219), reduced over the warp.
__device__ __forceinline__ uint32_t epa_best_face(const EpaWarpSmem& S, uint32_t nf, uint32_t lane) {
    float bd = INFINITY;
    uint32_t bf = 0xFFFFFFFFu;
    for (uint32_t i = lane; i < nf; i += 32)
        if (S.fd[i] < bd) { bd = S.fd[i]; bf = i; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float od = __shfl_xor_sync(0xffffffffu, bd, o);
        const uint32_t of = __shfl_xor_sync(0xffffffffu, bf, o);
        if (of != 0xFFFFFFFFu && (bf == 0xFFFFFFFFu || od < bd || (od == bd && of < bf))) { bd = od; bf = of; }
    }
    return bf;
}

// EPA::Compute (EPA.cpp:176-296) by one warp.  Every per-face float operation runs on one lane in
// the reference's order; selections use the reference's tie rules and ordered ballot compaction
// keeps the visible list, horizon edges and face array in the reference's order.
static __device__ __noinline__ void epa_warp(const SupportMap& map, const GjkOut& g, float tol, uint32_t max_iter, EpaWarpSmem& S,
                         EpaOut& r, uint32_t lane, uint32_t* err) {
    const unsigned full = 0xffffffffu;
    const unsigned lt = (1u << lane) - 1u;
    r.valid = false;
    r.depth = 0.0f;
    r.normal = Vec3(0.0f, 1.0f, 0.0f);
    r.pA = r.pB = Vec3();
    SP tet[4];
    if (!epa_initial_tetra_warp(map, g, tet, S, lane)) return;  // identical on every lane
    if (lane < 4) {
        const SP& t = tet[lane];
        S.vp[lane][0] = t.p.x; S.vp[lane][1] = t.p.y; S.vp[lane][2] = t.p.z;
        S.va[lane][0] = t.pA.x; S.va[lane][1] = t.pA.y; S.va[lane][2] = t.pA.z;
        S.vb[lane][0] = t.pB.x; S.vb[lane][1] = t.pB.y; S.vb[lane][2] = t.pB.z;
    }
    __syncwarp();
    uint32_t nf = 0;
    const uint8_t T4[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
    for (int i = 0; i < 4; ++i) {
        uint32_t fa = T4[i][0], fb = T4[i][1], fc = T4[i][2];
        Vec3 n;
        float d;
        if (epa_build_face_sm(fa, fb, fc, n, d, S)) {
            if (lane == 0) sm_put_face(S, nf, fa, fb, fc, n, d);
            ++nf;
        }
    }
    __syncwarp();
    if (nf < 4) return;
    const float eps = tol;
    uint32_t nv = 4;
    for (uint32_t it = 0; it < max_iter; ++it) {
        const uint32_t bf = epa_best_face(S, nf, lane);
        if (bf == 0xFFFFFFFFu) break;
        const Vec3 fn(S.fnx[bf], S.fny[bf], S.fnz[bf]);
        const float fdist = S.fd[bf];
        const SP w = map(fn);
        const float d = w.p.dot(fn);
        if (d - fdist < eps || nv >= 256) {
            epa_finish_sm(S, bf, r);
            return;
        }
        if (nv >= kEpaVerts) {  // unreachable with max_iter <= 64
            if (lane == 0) atomicOr(err, 4u);
            epa_finish_sm(S, bf, r);
            return;
        }
        const uint32_t ni = nv;
        __syncwarp();
        if (lane == 0) {
            S.vp[ni][0] = w.p.x; S.vp[ni][1] = w.p.y; S.vp[ni][2] = w.p.z;
            S.va[ni][0] = w.pA.x; S.va[ni][1] = w.pA.y; S.va[ni][2] = w.pA.z;
            S.vb[ni][0] = w.pB.x; S.vb[ni][1] = w.pB.y; S.vb[ni][2] = w.pB.z;
        }
        ++nv;
        // faces visible from w, in index order
        uint32_t nvis = 0;
        for (uint32_t base = 0; base < nf; base += 32) {
            const uint32_t i = base + lane;
            bool v = false;
            if (i < nf) {
                const Vec3 n(S.fnx[i], S.fny[i], S.fnz[i]);
                v = n.dot(w.p) - S.fd[i] > eps;
            }
            const unsigned m = __ballot_sync(full, v);
            if (lane == 0) S.dead[base >> 5] = m;
            if (v) S.vis[nvis + __popc(m & lt)] = (uint16_t)i;
            nvis += __popc(m);
        }
        __syncwarp();
        // horizon: edges of visible faces without a reverse edge in another visible face.  The
        // visible faces' directed edges go into a bit table first (a face never holds both (u, v)
        // and (v, u): its three vertices differ), so each edge's test is one lookup.
        uint32_t nh = 0;
        const uint32_t items = 3 * nvis;
        constexpr uint32_t kEdgeWords = (kEpaVerts * kEpaVerts + 31) / 32;
        for (uint32_t k = lane; k < kEdgeWords; k += 32) S.ebits[k] = 0u;
        __syncwarp();
        for (uint32_t item = lane; item < items; item += 32) {
            const uint32_t fi = S.vis[item / 3], e = item % 3;
            const uint32_t A = S.fa[fi], B = S.fb[fi], C = S.fc[fi];
            const uint32_t u = e == 0 ? A : (e == 1 ? B : C), v = e == 0 ? B : (e == 1 ? C : A);
            const uint32_t key = u * kEpaVerts + v;
            atomicOr(&S.ebits[key >> 5], 1u << (key & 31u));
        }
        __syncwarp();
        for (uint32_t base = 0; base < items; base += 32) {
            const uint32_t item = base + lane;
            bool keep = false;
            uint32_t eu = 0, ev = 0;
            if (item < items) {
                const uint32_t fi = S.vis[item / 3], e = item % 3;
                const uint32_t A = S.fa[fi], B = S.fb[fi], C = S.fc[fi];
                eu = e == 0 ? A : (e == 1 ? B : C);
                ev = e == 0 ? B : (e == 1 ? C : A);
                const uint32_t rkey = ev * kEpaVerts + eu;
                keep = !((S.ebits[rkey >> 5] >> (rkey & 31u)) & 1u);
            }
            const unsigned m = __ballot_sync(full, keep);
            const uint32_t pos = nh + __popc(m & lt);
            if (keep && pos < kEpaHorizon) { S.hu[pos] = (uint8_t)eu; S.hv[pos] = (uint8_t)ev; }
            nh = min(kEpaHorizon, nh + (uint32_t)__popc(m));
        }
        __syncwarp();
        // drop the visible faces, keeping order
        uint32_t wi = 0;
        for (uint32_t base = 0; base < nf; base += 32) {
            const uint32_t i = base + lane;
            const bool alive = i < nf && !((S.dead[i >> 5] >> (i & 31u)) & 1u);
            uint32_t a = 0, b = 0, c = 0;
            float nx = 0.0f, ny = 0.0f, nz = 0.0f, dd = 0.0f;
            if (alive) { a = S.fa[i]; b = S.fb[i]; c = S.fc[i]; nx = S.fnx[i]; ny = S.fny[i]; nz = S.fnz[i]; dd = S.fd[i]; }
            const unsigned m = __ballot_sync(full, alive);
            __syncwarp();
            if (alive) sm_put_face(S, wi + __popc(m & lt), a, b, c, Vec3(nx, ny, nz), dd);
            wi += __popc(m);
            __syncwarp();
        }
        nf = wi;
        // new faces (horizon.v, horizon.u, new vertex) in horizon order, up to the face capacity
        for (uint32_t base = 0; base < nh; base += 32) {
            const uint32_t k = base + lane;
            bool okf = false;
            uint32_t fa = 0, fb = 0, fc = ni;
            Vec3 n;
            float dd = 0.0f;
            if (k < nh) {
                fa = S.hv[k];
                fb = S.hu[k];
                okf = epa_build_face_sm(fa, fb, fc, n, dd, S);
            }
            const unsigned m = __ballot_sync(full, okf);
            const uint32_t pos = nf + __popc(m & lt);
            if (okf && pos < kEpaFaces) sm_put_face(S, pos, fa, fb, fc, n, dd);
            nf = min(kEpaFaces, nf + (uint32_t)__popc(m));
            __syncwarp();
        }
    }
    const uint32_t bf = epa_best_face(S, nf, lane);
    if (bf != 0xFFFFFFFFu) epa_finish_sm(S, bf, r);
}

// How the pair routines obtain EPA results: the thread-per-pair pass defers pairs that need EPA
// to a worklist; the warp-per-pair pass runs them cooperatively.
struct EpaDefer {
    static constexpr bool kWarp = false;
    uint32_t* nepa;     // worklist length
    uint32_t* list;     // worklist of pair indices
    GjkOut* kept;       // per worklist slot: the GJK result the EPA starts from (first `cap` slots)
    uint32_t cap;
    uint32_t pair;
    bool deferred = false;
    __device__ bool solo() const { return true; }
    __device__ void operator()(const SupportMap&, const GjkOut& g, float, uint32_t, EpaOut& e) {
        const uint32_t slot = atomicAdd(nepa, 1u);
        list[slot] = pair;
        if (slot < cap) kept[slot] = g;
        deferred = true;
        e.valid = false;
    }
};
struct EpaCoop {
    static constexpr bool kWarp = true;
    EpaWarpSmem* S;
    uint32_t lane;
    uint32_t* err;
    const GjkOut* pre;  // the thread pass's GJK result for this pair (same inputs, same result), or null
    bool deferred = false;
    __device__ bool solo() const { return lane == 0; }  // the lane that stores the manifold
    __device__ void operator()(const SupportMap& m, const GjkOut& g, float tol, uint32_t it, EpaOut& e) {
        epa_warp(m, g, tol, it, *S, e, lane, err);
    }
};

// GJK of a pair: in the warp pass the thread pass's result when it was kept (the same call on the
// same inputs), else computed.
template <typename Epa>
__device__ __forceinline__ void run_gjk(const SupportMap& map, float tol, GjkOut& g, const Epa& epa) {
    if constexpr (Epa::kWarp) {
        if (epa.pre) {
            g = *epa.pre;
            return;
        }
    }
    gjk(map, tol, 32, g);
}

// ---------------------------------------------------------------------------------------------
// Face clipping (CollideShape.cpp:30-228)
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kMaxFaceVerts = 16;

static __device__ __noinline__ bool shape_face(const ShapeTables& T, const Body& b, const Vec3& wdir, Vec3* out, uint32_t& cnt,
                                  Vec3& nworld) {
    const ShapeDev* s = b.s;
    if (s->type == kBox) {
        Vec3 ld = b.q.inv_rotate(wdir);
        int axis = ld.abs().max_comp_index();
        float sg = ld[axis] >= 0.0f ? 1.0f : -1.0f;
        Vec3 he(s->p[0], s->p[1], s->p[2]);
        Vec3 n;
        n.set(axis, sg);
        Vec3 c(he.x * n.x, he.y * n.y, he.z * n.z);
        int a0 = (axis + 1) % 3, a1 = (axis + 2) % 3;
        float s0 = he[a0], s1 = he[a1];
        Vec3 cr[4] = {c, c, c, c};
        cr[0].set(a0, s0); cr[0].set(a1, s1);
        cr[1].set(a0, -s0); cr[1].set(a1, s1);
        cr[2].set(a0, -s0); cr[2].set(a1, -s1);
        cr[3].set(a0, s0); cr[3].set(a1, -s1);
        for (int i = 0; i < 4; ++i) out[i] = xform(b.q, b.t, cr[i]);
        cnt = 4;
        nworld = b.q.rotate(n);
        return true;
    }
    if (s->type == kHull) {
        Vec3 ld = b.q.inv_rotate(wdir);
        float bd = -INFINITY;
        uint32_t bf = 0xFFFFFFFFu, boff = 0;
        uint32_t off = s->ifirst;
        for (uint32_t fi = 0; fi < s->fnum; ++fi) {
            uint32_t n = T.face_sizes[s->ffirst + fi];
            Vec3 a = hv(T, s->vfirst + T.face_idx[off]), bb = hv(T, s->vfirst + T.face_idx[off + 1]),
                 c = hv(T, s->vfirst + T.face_idx[off + 2]);
            Vec3 fn = (bb - a).cross(c - a).normalized_or(Vec3(0.0f, 1.0f, 0.0f));
            float d = fn.dot(ld);
            if (d > bd) { bd = d; bf = fi; boff = off; }
            off += n;
        }
        if (bf == 0xFFFFFFFFu) return false;
        uint32_t n = T.face_sizes[s->ffirst + bf];
        if (n > kMaxFaceVerts) n = kMaxFaceVerts;
        for (uint32_t i = 0; i < n; ++i) out[i] = xform(b.q, b.t, hv(T, s->vfirst + T.face_idx[boff + i]));
        cnt = n;
        Vec3 a = hv(T, s->vfirst + T.face_idx[boff]), bb = hv(T, s->vfirst + T.face_idx[boff + 1]),
             c = hv(T, s->vfirst + T.face_idx[boff + 2]);
        nworld = b.q.rotate((bb - a).cross(c - a).normalized_or(Vec3(0.0f, 1.0f, 0.0f)));
        return true;
    }
    return false;
}

struct ClipPoly {
    Vec3 v[kMaxFaceVerts * 2];
    uint32_t n;
    __device__ void add(const Vec3& p) {
        if (n < kMaxFaceVerts * 2) v[n++] = p;
    }
};

__device__ inline void clip_plane(const ClipPoly& in, const Vec3& pn, float pd, ClipPoly& out) {
    out.n = 0;
    if (in.n == 0) return;
    for (uint32_t i = 0; i < in.n; ++i) {
        Vec3 cur = in.v[i], nxt = in.v[(i + 1) % in.n];
        float dc = pn.dot(cur) - pd, dn = pn.dot(nxt) - pd;
        if (dc <= 0.0f) out.add(cur);
        if ((dc <= 0.0f) != (dn <= 0.0f)) {
            float t = rdiv(dc, dc - dn);
            out.add(lerp(cur, nxt, t));
        }
    }
}

__device__ inline bool is_poly(const ShapeDev* s) { return s->type == kBox || s->type == kHull; }

// Writes at most kMaxFaceVerts*2 candidate points before reduction; keeps the reference's
// (i*(n-1)/3) reduction of more than four points.
static __device__ __noinline__ uint32_t collide_polyhedral(const ShapeTables& T, const Body& A, const Body& B, float max_sep,
                                              Manifold& m, const Vec3& normal) {
    Vec3 fa[kMaxFaceVerts], fb[kMaxFaceVerts], na, nb;
    uint32_t ca = 0, cb = 0;
    bool ha = shape_face(T, A, -normal, fa, ca, na);
    bool hb = shape_face(T, B, normal, fb, cb, nb);
    if (!ha || !hb) return 0;
    float ala = na.dot(-normal), alb = nb.dot(normal);
    const bool ref_a = ala >= alb;
    const Vec3* rv = ref_a ? fa : fb;
    const Vec3* iv = ref_a ? fb : fa;
    const uint32_t rc = ref_a ? ca : cb, ic = ref_a ? cb : ca;
    Vec3 rn = ref_a ? na : nb;
    float rd = rn.dot(rv[0]);
    ClipPoly poly, tmp;
    poly.n = 0;
    for (uint32_t i = 0; i < ic; ++i) poly.add(iv[i]);
    Vec3 cen;
    for (uint32_t i = 0; i < rc; ++i) cen = cen + rv[i];
    cen = cen / (float)rc;
    for (uint32_t i = 0; i < rc; ++i) {
        Vec3 v0 = rv[i], v1 = rv[(i + 1) % rc];
        Vec3 sn = (v1 - v0).cross(rn);
        float len = sn.len();
        if (len < 1.0e-9f) continue;
        sn = sn / len;
        if (sn.dot(v0 - cen) < 0.0f) sn = -sn;
        float sd = sn.dot(v0);
        clip_plane(poly, sn, sd, tmp);
        poly = tmp;
        if (poly.n == 0) break;
    }
    // Keep-list of up to 8 candidates (kMaxManifoldPoints), then reduce to 4.
    ContactPt cand[8];
    uint32_t nc = 0;
    for (uint32_t i = 0; i < poly.n && nc < 8; ++i) {
        Vec3 p = poly.v[i];
        float sep = rn.dot(p) - rd;
        if (sep > max_sep) continue;
        Vec3 proj = p - rn * sep;
        cand[nc].pA = ref_a ? proj : p;
        cand[nc].pB = ref_a ? p : proj;
        cand[nc].n = normal;
        cand[nc].sep = sep;
        cand[nc].feature = i;
        ++nc;
    }
    if (nc > 4) {
        for (uint32_t i = 0; i < 4; ++i) m.pts[i] = cand[i * (nc - 1) / 3];
        nc = 4;
    } else {
        for (uint32_t i = 0; i < nc; ++i) m.pts[i] = cand[i];
    }
    m.n = nc;
    return nc;
}

// ---- the same face clipping on one warp, for the EPA pass (every lane calls it; the result is on
// every lane).  The float operations are the ones above, vertex by vertex; what is spread over the
// lanes is the independent work: a hull's face normals (first largest wins, as in the loop), each
// clip pass (one input vertex per lane; its kept vertex and crossing written at its place in the
// sequential output order, found by a warp scan, past the 32-vertex cap dropped as add() drops them)
// and the candidate filter (the first eight kept, in order).  Polygons live in the warp's EPA
// scratch, free once the EPA result is taken.
struct ClipWarpSmem {
    float fa[kMaxFaceVerts][3], fb[kMaxFaceVerts][3];
    float p0[kMaxFaceVerts * 2][3], p1[kMaxFaceVerts * 2][3];
    ContactPt cand[8];
};
static_assert(sizeof(ClipWarpSmem) <= sizeof(EpaWarpSmem), "clip scratch overlays the EPA scratch");

__device__ __forceinline__ Vec3 ld3(const float (*a)[3], uint32_t i) { return Vec3(a[i][0], a[i][1], a[i][2]); }
__device__ __forceinline__ void st3(float (*a)[3], uint32_t i, const Vec3& v) { a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; }

__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, uint32_t lane, uint32_t* total) {
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    *total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// shape_face with the hull's face search spread over the lanes; the face's vertices go to `out`.
static __device__ bool shape_face_warp(const ShapeTables& T, const Body& b, const Vec3& wdir, float (*out)[3], uint32_t& cnt,
                                Vec3& nworld, uint32_t lane) {
    const ShapeDev* s = b.s;
    if (s->type == kBox) {
        Vec3 ld = b.q.inv_rotate(wdir);
        int axis = ld.abs().max_comp_index();
        float sg = ld[axis] >= 0.0f ? 1.0f : -1.0f;
        Vec3 he(s->p[0], s->p[1], s->p[2]);
        Vec3 n;
        n.set(axis, sg);
        Vec3 c(he.x * n.x, he.y * n.y, he.z * n.z);
        int a0 = (axis + 1) % 3, a1 = (axis + 2) % 3;
        float s0 = he[a0], s1 = he[a1];
        if (lane < 4) {
            Vec3 cr = c;
            cr.set(a0, (lane == 0 || lane == 3) ? s0 : -s0);
            cr.set(a1, lane < 2 ? s1 : -s1);
            st3(out, lane, xform(b.q, b.t, cr));
        }
        cnt = 4;
        nworld = b.q.rotate(n);
        return true;
    }
    if (s->type == kHull) {
        const Vec3 ld = b.q.inv_rotate(wdir);
        float bd = -INFINITY;
        uint32_t bf = 0xFFFFFFFFu, boff = 0, off = s->ifirst;
        for (uint32_t base = 0; base < s->fnum; base += 32) {
            const uint32_t fi = base + lane;
            const uint32_t n = fi < s->fnum ? T.face_sizes[s->ffirst + fi] : 0u;
            uint32_t tot;
            const uint32_t o = off + warp_excl_scan(n, lane, &tot);
            float d = -INFINITY;
            if (fi < s->fnum) {
                Vec3 a = hv(T, s->vfirst + T.face_idx[o]), bb = hv(T, s->vfirst + T.face_idx[o + 1]),
                     c = hv(T, s->vfirst + T.face_idx[o + 2]);
                Vec3 fn = (bb - a).cross(c - a).normalized_or(Vec3(0.0f, 1.0f, 0.0f));
                d = fn.dot(ld);
            }
            float md = (d > -INFINITY) ? d : -INFINITY;  // a NaN never wins, as `d > bd` never holds for it
            uint32_t mf = (d > -INFINITY) ? fi : 0xFFFFFFFFu, mo = o;
#pragma unroll
            for (int k = 16; k > 0; k >>= 1) {
                const float od = __shfl_xor_sync(0xffffffffu, md, k);
                const uint32_t of = __shfl_xor_sync(0xffffffffu, mf, k), oo = __shfl_xor_sync(0xffffffffu, mo, k);
                if (of != 0xFFFFFFFFu && (mf == 0xFFFFFFFFu || od > md || (od == md && of < mf))) { md = od; mf = of; mo = oo; }
            }
            if (mf != 0xFFFFFFFFu && md > bd) { bd = md; bf = mf; boff = mo; }  // earlier chunks win ties
            off += tot;
        }
        if (bf == 0xFFFFFFFFu) return false;
        uint32_t n = T.face_sizes[s->ffirst + bf];
        if (n > kMaxFaceVerts) n = kMaxFaceVerts;
        if (lane < n) st3(out, lane, xform(b.q, b.t, hv(T, s->vfirst + T.face_idx[boff + lane])));
        cnt = n;
        Vec3 a = hv(T, s->vfirst + T.face_idx[boff]), bb = hv(T, s->vfirst + T.face_idx[boff + 1]),
             c = hv(T, s->vfirst + T.face_idx[boff + 2]);
        nworld = b.q.rotate((bb - a).cross(c - a).normalized_or(Vec3(0.0f, 1.0f, 0.0f)));
        return true;
    }
    return false;
}

static __device__ __noinline__ uint32_t collide_polyhedral_warp(const ShapeTables& T, const Body& A, const Body& B, float max_sep,
                                            Manifold& m, const Vec3& normal, EpaWarpSmem& scratch, uint32_t lane) {
    __syncwarp();  // the EPA result has been read from the scratch by every lane
    ClipWarpSmem& C = *reinterpret_cast<ClipWarpSmem*>(&scratch);
    Vec3 na, nb;
    uint32_t ca = 0, cb = 0;
    const bool ha = shape_face_warp(T, A, -normal, C.fa, ca, na, lane);
    const bool hb = shape_face_warp(T, B, normal, C.fb, cb, nb, lane);
    __syncwarp();
    if (!ha || !hb) return 0;
    float ala = na.dot(-normal), alb = nb.dot(normal);
    const bool ref_a = ala >= alb;
    const float (*rv)[3] = ref_a ? C.fa : C.fb;
    const float (*iv)[3] = ref_a ? C.fb : C.fa;
    const uint32_t rc = ref_a ? ca : cb, ic = ref_a ? cb : ca;
    const Vec3 rn = ref_a ? na : nb;
    const float rd = rn.dot(ld3(rv, 0));
    float (*src)[3] = C.p0;
    float (*dst)[3] = C.p1;
    if (lane < ic) st3(src, lane, ld3(iv, lane));
    uint32_t count = ic;
    Vec3 cen;
    for (uint32_t i = 0; i < rc; ++i) cen = cen + ld3(rv, i);
    cen = cen / (float)rc;
    __syncwarp();
    for (uint32_t i = 0; i < rc; ++i) {
        const Vec3 v0 = ld3(rv, i), v1 = ld3(rv, i + 1 == rc ? 0 : i + 1);
        Vec3 sn = (v1 - v0).cross(rn);
        const float len = sn.len();
        if (len < 1.0e-9f) continue;
        sn = sn / len;
        if (sn.dot(v0 - cen) < 0.0f) sn = -sn;
        const float sd = sn.dot(v0);
        bool keep = false, cross = false;
        Vec3 cur, ip;
        if (lane < count) {
            cur = ld3(src, lane);
            const Vec3 nxt = ld3(src, lane + 1 == count ? 0 : lane + 1);
            const float dc = sn.dot(cur) - sd, dn = sn.dot(nxt) - sd;
            keep = dc <= 0.0f;
            cross = (dc <= 0.0f) != (dn <= 0.0f);
            if (cross) ip = lerp(cur, nxt, rdiv(dc, dc - dn));
        }
        uint32_t tot;
        const uint32_t pos = warp_excl_scan((keep ? 1u : 0u) + (cross ? 1u : 0u), lane, &tot);
        if (keep && pos < kMaxFaceVerts * 2) st3(dst, pos, cur);
        if (cross && pos + (keep ? 1u : 0u) < kMaxFaceVerts * 2) st3(dst, pos + (keep ? 1u : 0u), ip);
        count = min(tot, kMaxFaceVerts * 2);
        __syncwarp();
        float (*t)[3] = src;
        src = dst;
        dst = t;
        if (count == 0) break;
    }
    // the first eight vertices within max_sep of the reference face, in order
    bool keep = false;
    Vec3 p;
    float sep = 0.0f;
    if (lane < count) {
        p = ld3(src, lane);
        sep = rn.dot(p) - rd;
        keep = !(sep > max_sep);
    }
    uint32_t nkeep;
    const uint32_t pos = warp_excl_scan(keep ? 1u : 0u, lane, &nkeep);
    if (keep && pos < 8u) {
        const Vec3 proj = p - rn * sep;
        ContactPt& c = C.cand[pos];
        c.pA = ref_a ? proj : p;
        c.pB = ref_a ? p : proj;
        c.n = normal;
        c.sep = sep;
        c.feature = lane;
    }
    __syncwarp();
    uint32_t nc = min(nkeep, 8u);
    if (nc > 4) {
        for (uint32_t i = 0; i < 4; ++i) m.pts[i] = C.cand[i * (nc - 1) / 3];
        nc = 4;
    } else {
        for (uint32_t i = 0; i < nc; ++i) m.pts[i] = C.cand[i];
    }
    m.n = nc;
    __syncwarp();
    return nc;
}

__device__ __forceinline__ void add_point(Manifold& m, const Vec3& pA, const Vec3& pB, const Vec3& n, float sep) {
    if (m.n < kMaxManifold) {
        ContactPt& c = m.pts[m.n++];
        c.pA = pA; c.pB = pB; c.n = n; c.sep = sep; c.feature = 0;
    }
}

__device__ __forceinline__ void swap_manifold(Manifold& m) {
    for (uint32_t i = 0; i < m.n; ++i) {
        Vec3 t = m.pts[i].pA;
        m.pts[i].pA = m.pts[i].pB;
        m.pts[i].pB = t;
        m.pts[i].n = -m.pts[i].n;
    }
}

template <typename Epa>
__device__ inline uint32_t collide_generic(const ShapeTables& T, const Body& A, const Body& B, float max_sep, float tol,
                                           Manifold& m, Epa& epa) {
    SupportMap map{&T, A, B};
    GjkOut g;
    run_gjk(map, tol, g, epa);
    const bool poly = is_poly(A.s) && is_poly(B.s);
    if (!g.intersect) {
        if (g.distance > max_sep) return 0;
        if (poly && g.normal.len2() > 0.0f) {
            if (collide_polyhedral(T, A, B, max_sep, m, g.normal) > 0) return m.n;
        }
        add_point(m, g.pA, g.pB, g.normal, g.distance);
        return m.n;
    }
    EpaOut e;
    if (poly) {
        epa(map, g, tol, 64, e);
        if (epa.deferred) return 0;
        if (!e.valid) {  // the reference computes the same EPA once more below: same inputs, same result
            add_point(m, g.pA, g.pB, g.normal.len2() > 0.0f ? g.normal : Vec3(0.0f, 1.0f, 0.0f), 0.0f);
            return m.n;
        }
        if (e.valid) {
            if constexpr (Epa::kWarp) {  // a cooperative EPA: the warp clips the faces too
                if (collide_polyhedral_warp(T, A, B, max_sep, m, e.normal, *epa.S, epa.lane) > 0) return m.n;
            } else {
                if (collide_polyhedral(T, A, B, max_sep, m, e.normal) > 0) return m.n;
            }
            add_point(m, e.pA, e.pB, e.normal, -e.depth);
            return m.n;
        }
    }
    epa(map, g, tol, 64, e);
    if (epa.deferred) return 0;
    if (e.valid) {
        add_point(m, e.pA, e.pB, e.normal, -e.depth);
        return m.n;
    }
    add_point(m, g.pA, g.pB, g.normal.len2() > 0.0f ? g.normal : Vec3(0.0f, 1.0f, 0.0f), 0.0f);
    return m.n;
}

template <typename Epa>
__device__ inline uint32_t collide_sphere_convex(const ShapeTables& T, const Body& S_, const Body& B, float max_sep,
                                                 float tol, Manifold& m, Epa& epa) {
    ShapeDev point{};
    point.type = kSphere;
    point.p[0] = 1.0e-4f;
    Body P{&point, S_.q, S_.t};
    SupportMap map{&T, P, B};
    GjkOut g;
    run_gjk(map, tol, g, epa);
    const float radius = S_.s->p[0];
    const Vec3 center = S_.t;
    if (g.intersect) {
        EpaOut e;
        epa(map, g, tol, 64, e);
        if (epa.deferred) return 0;
        if (e.valid) {
            Vec3 n = -e.normal;
            add_point(m, center + n * radius, e.pB, n, -(e.depth + radius));
            return m.n;
        }
        return 0;
    }
    float dist = g.distance;
    float sep = dist - radius;
    if (sep > max_sep) return 0;
    Vec3 n = (dist > kEps) ? (center - g.pB) / dist : Vec3(0.0f, 1.0f, 0.0f);
    add_point(m, center - n * radius, g.pB, n, sep);
    return m.n;
}

__device__ inline uint32_t collide_sphere_sphere(const Body& A, const Body& B, float max_sep, Manifold& m) {
    Vec3 d = A.t - B.t;
    float dist = d.len();
    float sep = dist - (A.s->p[0] + B.s->p[0]);
    if (sep > max_sep) return 0;
    Vec3 n = dist > kEps ? d / dist : Vec3(0.0f, 1.0f, 0.0f);
    add_point(m, A.t - n * A.s->p[0], B.t + n * B.s->p[0], n, sep);
    return m.n;
}

static __device__ __noinline__ uint32_t collide_plane_convex(const ShapeTables& T, const Body& P, const Body& B, float max_sep,
                                                Manifold& m) {
    Vec3 pn = P.q.rotate(Vec3(P.s->p[0], P.s->p[1], P.s->p[2]));
    float pd = P.s->p[3] + pn.dot(P.t);
    if (is_poly(B.s)) {
        ContactPt cand[8];
        uint32_t count = 0;
        const uint32_t nverts = B.s->type == kBox ? 8u : (B.s->vnum < kMaxFaceVerts ? B.s->vnum : kMaxFaceVerts);
        for (uint32_t i = 0; i < nverts && count < 8; ++i) {
            Vec3 v;
            if (B.s->type == kBox) {
                Vec3 he(B.s->p[0], B.s->p[1], B.s->p[2]);
                v = xform(B.q, B.t, Vec3((i & 1) ? he.x : -he.x, (i & 2) ? he.y : -he.y, (i & 4) ? he.z : -he.z));
            } else {
                v = xform(B.q, B.t, hv(T, B.s->vfirst + i));
            }
            float d = pn.dot(v) - pd;
            if (d > max_sep) continue;
            cand[count].n = pn;
            cand[count].pA = v;
            cand[count].pB = v - pn * d;
            cand[count].sep = d;
            cand[count].feature = 0;
            ++count;
        }
        if (count > 4) {
            for (uint32_t i = 0; i < 4; ++i) m.pts[i] = cand[i * (count - 1) / 3];
            count = 4;
        } else {
            for (uint32_t i = 0; i < count; ++i) m.pts[i] = cand[i];
        }
        m.n = count;
        return count;
    }
    Vec3 ld = B.q.inv_rotate(-pn);
    Vec3 deep = xform(B.q, B.t, support_local(T, B.s, ld));
    float d = pn.dot(deep) - pd;
    if (d > max_sep) return 0;
    add_point(m, deep, deep - pn * d, pn, d);
    return m.n;
}

// NarrowPhase::Collide dispatch (CollideShape.cpp:480-592) for the device shape set.  With
// EpaDefer the result is incomplete when epa.deferred is set afterwards.
template <typename Epa>
__device__ inline uint32_t collide(const ShapeTables& T, const Body& A, const Body& B, float max_sep, float tol,
                                   Manifold& m, Epa& epa) {
    m.n = 0;
    const uint32_t ta = A.s->type, tb = B.s->type;
    if (ta == kPlane) {
        uint32_t n = collide_plane_convex(T, A, B, max_sep, m);
        if (n > 0) swap_manifold(m);
        return n;
    }
    if (tb == kPlane) return collide_plane_convex(T, B, A, max_sep, m);
    if (ta == kSphere && tb == kSphere) return collide_sphere_sphere(A, B, max_sep, m);
    if (ta == kSphere) return collide_sphere_convex(T, A, B, max_sep, tol, m, epa);
    if (tb == kSphere) {
        uint32_t n = collide_sphere_convex(T, B, A, max_sep, tol, m, epa);
        if (n > 0) swap_manifold(m);
        return n;
    }
    return collide_generic(T, A, B, max_sep, tol, m, epa);
}

// NarrowPhase::CastShape (CollideShape.cpp:607-661): the first fraction of `max_distance` along `direction` at
// which A, moving without rotation, touches B, and B's surface normal there.  A plane B is solved
// in closed form (A's deepest point against the plane); every other pair by conservative
// advancement: GJK distance at the current translation (tolerance 1e-4, 32 iterations), advance by
// distance - tolerance, at most 64 steps.
//
// `cut` (optional, the bits of a non-negative float that only decreases): the caller keeps only
// fractions below it, so the advancement stops once t / max_distance exceeds it (t never
// decreases, so the fraction could only be larger); a kept result is the same as without it.
__device__ inline bool cast_shape(const ShapeTables& T, const Body& A, const Vec3& direction, float max_distance,
                                  const Body& B, float& fraction, Vec3& normal,
                                  const volatile int* cut = nullptr) {
    const float dir_len = direction.len();
    if (dir_len < kEps) return false;
    const Vec3 dir = direction / dir_len;
    if (B.s->type == kPlane) {
        if (A.s->type == kPlane) return false;
        const Vec3 pn(B.s->p[0], B.s->p[1], B.s->p[2]);
        const Vec3 nw = B.q.rotate(pn).normalized();
        const float plane_dist = nw.dot(xform(B.q, B.t, pn * B.s->p[3]));
        const Vec3 deepest = xform(A.q, A.t, support_local(T, A.s, A.q.inv_rotate(-nw)));
        const float sd = nw.dot(deepest) - plane_dist;
        if (sd <= 1.0e-4f) {
            fraction = 0.0f;
            normal = nw;
            return true;
        }
        const float rate = nw.dot(dir);
        if (rate >= -kEps) return false;  // parallel or moving away
        const float t_hit = sd / (-rate);
        if (t_hit > max_distance) return false;
        fraction = t_hit / max_distance;
        normal = nw;
        return true;
    }
    const float tol = 1.0e-4f;
    float t = 0.0f;
    for (uint32_t it = 0; it < 64; ++it) {
        if (cut && t / max_distance > __int_as_float(*cut)) return false;
        SupportMap map{&T, Body{A.s, A.q, A.t + dir * t}, B};
        GjkOut g;
        gjk(map, tol, 32, g);
        if (g.intersect || g.distance <= tol) {
            fraction = t / max_distance;
            normal = g.normal;
            return true;
        }
        if (t >= max_distance) return false;
        float advance = g.distance - tol;
        if (advance <= 0.0f) advance = tol;
        t += advance;
        if (t > max_distance) return false;
    }
    return false;
}

}  // namespace kzg
