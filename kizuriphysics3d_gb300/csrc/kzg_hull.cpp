// kzg_hull.cpp - host-side scene setup: convex hull construction and mass properties.
//
// Runs once per shape/body when a scene is created, never per step.  The hull vertex order and
// the float rounding of every mass property must match the reference, because the narrow phase's
// tie-breaks (first vertex / face wins) and the solver's effective masses depend on them:
//   ConvexHullShape::Create          reference src/Geometry/Shapes.cpp:305-471
//   ComputeDerivedData (bounds)      Shapes.cpp:488-536
//   GetMassProperties                Shapes.cpp:27-33 (sphere), 53-65 (box), 108-141 (capsule),
//                                    549-608 (hull); Shape.h:518 (plane)
//   RecomputeMassProperties          reference src/Body/BodyManager.cpp:63-99
// Compiled with -ffp-contract=off so no product is fused into a sum.
#include <cmath>
#include <cstring>
#include <vector>

#include "kzg_internal.h"
#include "kzg_math.cuh"

namespace kzg {

namespace {

constexpr float kPi = 3.14159265358979323846f;

Mat3 mat_zero() { return Mat3{Vec3(), Vec3(), Vec3()}; }
Mat3 mat_diag(float x, float y, float z) { return Mat3{Vec3(x, 0.0f, 0.0f), Vec3(0.0f, y, 0.0f), Vec3(0.0f, 0.0f, z)}; }
Mat3 mat_identity_times(float s) {  // Mat3::Identity() * s (Math.h:208)
    return Mat3{Vec3(1.0f * s, 0.0f * s, 0.0f * s), Vec3(0.0f * s, 1.0f * s, 0.0f * s), Vec3(0.0f * s, 0.0f * s, 1.0f * s)};
}
Mat3 mat_scale(const Mat3& m, float s) { return Mat3{m.c0 * s, m.c1 * s, m.c2 * s}; }
Mat3 mat_add(const Mat3& a, const Mat3& b) { return Mat3{a.c0 + b.c0, a.c1 + b.c1, a.c2 + b.c2}; }
Mat3 mat_sub(const Mat3& a, const Mat3& b) { return Mat3{a.c0 - b.c0, a.c1 - b.c1, a.c2 - b.c2}; }
Mat3 outer(const Vec3& a, const Vec3& b) { return Mat3{a * b.x, a * b.y, a * b.z}; }
float determinant(const Mat3& m) { return m.c0.dot(m.c1.cross(m.c2)); }
Mat3 inversed(const Mat3& m) {  // Mat3::Inversed, Math.cpp:27-43
    Vec3 r0 = m.c1.cross(m.c2), r1 = m.c2.cross(m.c0), r2 = m.c0.cross(m.c1);
    float det = m.c0.dot(r0);
    float inv = det != 0.0f ? 1.0f / det : 0.0f;
    return Mat3{Vec3(r0.x, r1.x, r2.x) * inv, Vec3(r0.y, r1.y, r2.y) * inv, Vec3(r0.z, r1.z, r2.z) * inv};
}

struct HFace {
    uint32_t a, b, c;
    Vec3 n;
    float dist;
    bool alive;
};

void make_face(HFace& f, const std::vector<Vec3>& pts, const Vec3& interior) {
    Vec3 A = pts[f.a], B = pts[f.b], C = pts[f.c];
    Vec3 n = (B - A).cross(C - A);
    float len = n.len();
    if (len < 1.0e-12f) { f.alive = false; return; }
    n = n / len;
    if (n.dot(A - interior) < 0.0f) {
        uint32_t t = f.b; f.b = f.c; f.c = t;
        n = -n;
    }
    f.n = n;
    f.dist = n.dot(A);
}

struct MassProps {
    float mass = 0.0f;
    Mat3 inertia = mat_zero();
    Vec3 com;
};

MassProps hull_mass(const float* v, const uint8_t* sizes, uint32_t nfaces, const uint32_t* idx, float density) {
    MassProps mp;
    if (nfaces == 0) return mp;
    float total = 0.0f;
    Vec3 cacc;
    Mat3 iacc = mat_zero();
    uint32_t off = 0;
    auto P = [&](uint32_t k) { return Vec3(v[3 * k], v[3 * k + 1], v[3 * k + 2]); };
    for (uint32_t fi = 0; fi < nfaces; ++fi) {
        uint32_t n = sizes[fi];
        for (uint32_t t = 1; t + 1 < n; ++t) {
            Vec3 a = P(idx[off]), b = P(idx[off + t]), c = P(idx[off + t + 1]);
            float v6 = a.dot(b.cross(c));
            float sv = v6 / 6.0f;
            if (rabs(sv) < 1.0e-12f) continue;
            float tm = rabs(sv) * density;
            float sg = sv > 0.0f ? 1.0f : -1.0f;
            total += rabs(sv);
            cacc = cacc + ((a + b) + c) * (sv / 4.0f);
            float a2 = a.len2(), b2 = b.len2(), c2 = c.len2();
            float ab = a.dot(b), ac = a.dot(c), bc = b.dot(c);
            float tr = ((a2 + b2) + c2) + ((ab + ac) + bc);
            Mat3 oaa = outer(a, a), obb = outer(b, b), occ = outer(c, c);
            Mat3 xab = mat_add(outer(a, b), outer(b, a));
            Mat3 xac = mat_add(outer(a, c), outer(c, a));
            Mat3 xbc = mat_add(outer(b, c), outer(c, b));
            Mat3 ti = mat_sub(mat_sub(mat_identity_times(tm / 10.0f * tr), mat_scale(mat_add(mat_add(oaa, obb), occ), tm / 10.0f)),
                              mat_scale(mat_add(mat_add(xab, xac), xbc), tm / 20.0f));
            iacc = mat_add(iacc, mat_scale(ti, sg));
        }
        off += n;
    }
    if (total <= kEps) return mp;
    mp.mass = total * density;
    Vec3 com = cacc / total;
    mp.com = com;
    float c2 = com.len2();
    Mat3 shift = mat_sub(mat_identity_times(mp.mass * c2), mat_scale(outer(com, com), mp.mass));
    mp.inertia = mat_sub(iacc, shift);
    return mp;
}

float bounding_radius(const kzg_shape_desc& s, const float* hv) {
    switch (s.type) {
        case KZG_SHAPE_SPHERE: return s.params[0];
        case KZG_SHAPE_BOX: return Vec3(s.params[0], s.params[1], s.params[2]).len();
        case KZG_SHAPE_CAPSULE: return s.params[0] + s.params[1];
        case KZG_SHAPE_HULL: {
            float mn[3], mx[3];
            shape_local_bounds(s, hv, mn, mx);
            Vec3 c = (Vec3(mn[0], mn[1], mn[2]) + Vec3(mx[0], mx[1], mx[2])) * 0.5f;
            float r = 0.0f;
            for (uint32_t k = 0; k < s.num_vertices; ++k) {
                const float* p = hv + 3 * (s.first_vertex + k);
                r = rmax(r, (Vec3(p[0], p[1], p[2]) - c).len());
            }
            return r;
        }
        default: return 0.0f;
    }
}

}  // namespace

void shape_local_bounds(const kzg_shape_desc& s, const float* hv, float* mn, float* mx) {
    Vec3 lo, hi;
    switch (s.type) {
        case KZG_SHAPE_SPHERE: hi = Vec3(s.params[0], s.params[0], s.params[0]); lo = -hi; break;
        case KZG_SHAPE_BOX: hi = Vec3(s.params[0], s.params[1], s.params[2]); lo = -hi; break;
        case KZG_SHAPE_CAPSULE: hi = Vec3(s.params[1], s.params[0] + s.params[1], s.params[1]); lo = -hi; break;
        case KZG_SHAPE_PLANE: {  // PlaneShape::GetLocalBounds, Shape.h:508-515
            const float big = 1.0e6f;
            Vec3 n(s.params[0], s.params[1], s.params[2]);
            Vec3 ext = Vec3(big, big, big) - n.abs() * big;
            Vec3 c = n * s.params[3];
            lo = c - ext;
            hi = c + ext;
            break;
        }
        case KZG_SHAPE_HULL: {
            lo = Vec3(INFINITY, INFINITY, INFINITY);
            hi = Vec3(-INFINITY, -INFINITY, -INFINITY);
            for (uint32_t k = 0; k < s.num_vertices; ++k) {
                const float* p = hv + 3 * (s.first_vertex + k);
                Vec3 q(p[0], p[1], p[2]);
                lo = lo.vmin(q);
                hi = hi.vmax(q);
            }
            break;
        }
        default: break;
    }
    mn[0] = lo.x; mn[1] = lo.y; mn[2] = lo.z;
    mx[0] = hi.x; mx[1] = hi.y; mx[2] = hi.z;
}

int hull_build(const float* in, uint32_t n_in, uint32_t max_points, float* out_v, uint32_t* out_nv, uint8_t* out_sizes,
               uint32_t* out_nf, uint32_t* out_idx, uint32_t* out_ni, uint32_t cap_faces) {
    if (n_in < 4) return -1;
    std::vector<Vec3> pts;
    for (uint32_t i = 0; i < n_in; ++i) {
        Vec3 p(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
        bool dup = false;
        for (const Vec3& q : pts)
            if ((p - q).len2() < 1.0e-10f) { dup = true; break; }
        if (!dup) {
            pts.push_back(p);
            if (pts.size() >= max_points) break;
        }
    }
    const uint32_t np = (uint32_t)pts.size();
    if (np < 4) return -1;
    uint32_t i0 = 0;
    for (uint32_t i = 1; i < np; ++i)
        if (pts[i].x < pts[i0].x) i0 = i;
    uint32_t i1 = 0;
    float best = -1.0f;
    for (uint32_t i = 0; i < np; ++i) {
        if (i == i0) continue;
        float d = (pts[i] - pts[i0]).len2();
        if (d > best) { best = d; i1 = i; }
    }
    uint32_t i2 = 0;
    best = -1.0f;
    Vec3 axis = (pts[i1] - pts[i0]).normalized();
    for (uint32_t i = 0; i < np; ++i) {
        if (i == i0 || i == i1) continue;
        Vec3 rel = pts[i] - pts[i0];
        float d = (rel - axis * rel.dot(axis)).len2();
        if (d > best) { best = d; i2 = i; }
    }
    if (best < 1.0e-12f) return -1;
    Vec3 pn = (pts[i1] - pts[i0]).cross(pts[i2] - pts[i0]).normalized();
    uint32_t i3 = 0;
    best = -1.0f;
    for (uint32_t i = 0; i < np; ++i) {
        if (i == i0 || i == i1 || i == i2) continue;
        float d = rabs(pn.dot(pts[i] - pts[i0]));
        if (d > best) { best = d; i3 = i; }
    }
    if (best < 1.0e-10f) return -1;
    Vec3 interior = (((pts[i0] + pts[i1]) + pts[i2]) + pts[i3]) * 0.25f;
    std::vector<HFace> faces;
    {
        uint32_t id[4] = {i0, i1, i2, i3};
        const int tris[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
        for (auto& t : tris) {
            HFace f{id[t[0]], id[t[1]], id[t[2]], Vec3(0.0f, 1.0f, 0.0f), 0.0f, true};
            make_face(f, pts, interior);
            if (f.alive) faces.push_back(f);
        }
    }
    if (faces.size() < 4) return -1;
    const float eps = 1.0e-7f;
    for (uint32_t pi = 0; pi < np; ++pi) {
        if (pi == i0 || pi == i1 || pi == i2 || pi == i3) continue;
        const Vec3 p = pts[pi];
        std::vector<uint32_t> vis;
        for (size_t fi = 0; fi < faces.size(); ++fi)
            if (faces[fi].alive && faces[fi].n.dot(p) - faces[fi].dist > eps) vis.push_back((uint32_t)fi);
        if (vis.empty()) continue;
        std::vector<uint32_t> hu, hv;
        for (uint32_t fi : vis) {
            const HFace& f = faces[fi];
            uint32_t ev[3][2] = {{f.a, f.b}, {f.b, f.c}, {f.c, f.a}};
            for (auto& e : ev) {
                bool shared = false;
                for (uint32_t fj : vis) {
                    if (fj == fi) continue;
                    const HFace& g = faces[fj];
                    if ((g.a == e[1] && g.b == e[0]) || (g.b == e[1] && g.c == e[0]) || (g.c == e[1] && g.a == e[0])) {
                        shared = true;
                        break;
                    }
                }
                if (!shared) { hu.push_back(e[0]); hv.push_back(e[1]); }
            }
        }
        for (uint32_t fi : vis) faces[fi].alive = false;
        for (size_t k = 0; k < hu.size(); ++k) {
            HFace f{hv[k], hu[k], pi, Vec3(0.0f, 1.0f, 0.0f), 0.0f, true};
            make_face(f, pts, interior);
            if (f.alive) faces.push_back(f);
        }
    }
    std::vector<int32_t> remap(np, -1);
    uint32_t nv = 0, nf = 0, ni = 0;
    for (const HFace& f : faces) {
        if (!f.alive) continue;
        if (nf >= cap_faces) return -2;
        uint32_t tri[3] = {f.a, f.b, f.c};
        for (uint32_t k = 0; k < 3; ++k)
            if (remap[tri[k]] < 0) {
                remap[tri[k]] = (int32_t)nv;
                out_v[3 * nv] = pts[tri[k]].x;
                out_v[3 * nv + 1] = pts[tri[k]].y;
                out_v[3 * nv + 2] = pts[tri[k]].z;
                ++nv;
            }
        out_sizes[nf++] = 3;
        out_idx[ni++] = (uint32_t)remap[f.a];
        out_idx[ni++] = (uint32_t)remap[f.b];
        out_idx[ni++] = (uint32_t)remap[f.c];
    }
    if (nv < 4 || nf < 4) return -1;
    *out_nv = nv;
    *out_nf = nf;
    *out_ni = ni;
    return 0;
}

void mass_properties(const kzg_shape_desc& s, const float* hv, const uint8_t* sizes, const uint32_t* idx,
                     uint32_t motion, float density, float mass_override, float* out_inv_mass, float* out_iil) {
    std::memset(out_iil, 0, 9 * sizeof(float));
    *out_inv_mass = 0.0f;
    if (motion != KZG_MOTION_DYNAMIC) return;
    MassProps mp;
    switch (s.type) {
        case KZG_SHAPE_SPHERE: {
            float r = s.params[0];
            float vol = 4.0f / 3.0f;
            vol = (float)(4.0 / 3.0) * kPi * r * r * r;
            mp.mass = vol * density;
            mp.inertia = mat_identity_times(0.4f * mp.mass * r * r);
            break;
        }
        case KZG_SHAPE_BOX: {
            float hx = s.params[0], hy = s.params[1], hz = s.params[2];
            mp.mass = 8.0f * hx * hy * hz * density;
            float m = mp.mass;
            mp.inertia = mat_diag(m / 3.0f * (hy * hy + hz * hz), m / 3.0f * (hx * hx + hz * hz), m / 3.0f * (hx * hx + hy * hy));
            break;
        }
        case KZG_SHAPE_CAPSULE: {
            float r = s.params[1], h = s.params[0];
            float vcyl = kPi * r * r * (2.0f * h);
            float vsph = (float)(4.0 / 3.0) * kPi * r * r * r;
            float vol = vcyl + vsph;
            if (vol <= kEps) break;
            float mcyl = vcyl * density, msph = vsph * density, m = vol * density;
            float icyl_ax = mcyl * r * r * 0.5f;
            float icyl_tr = mcyl * (3.0f * r * r + 4.0f * h * h) / 12.0f;
            float isph = 0.4f * msph * r * r;
            float dsph = h + 3.0f * r / 8.0f;
            float isph_tr = isph + msph * dsph * dsph;
            float ixx = icyl_tr + isph_tr;
            mp.mass = m;
            mp.inertia = mat_diag(ixx, icyl_ax + isph, ixx);
            break;
        }
        case KZG_SHAPE_HULL:
            mp = hull_mass(hv + 3 * s.first_vertex, sizes + s.first_face, s.num_faces, idx + s.first_index, density);
            break;
        default: break;  // plane: MassProperties{}
    }
    float mass = mass_override > 0.0f ? mass_override : mp.mass;
    if (mass <= kEps) return;
    *out_inv_mass = 1.0f / mass;
    Mat3 inertia = mp.inertia;
    float det = determinant(inertia);
    if (rabs(det) < 1.0e-12f) {
        float r = bounding_radius(s, hv);
        inertia = mat_identity_times(0.4f * mass * r * r);
    }
    Vec3 com = mp.com;
    inertia = mat_add(inertia, mat_scale(mat_sub(mat_identity_times(com.len2()), outer(com, com)), mass));
    Mat3 inv = inversed(inertia);
    const Vec3 cols[3] = {inv.c0, inv.c1, inv.c2};
    for (int c = 0; c < 3; ++c) {
        out_iil[3 * c] = cols[c].x;
        out_iil[3 * c + 1] = cols[c].y;
        out_iil[3 * c + 2] = cols[c].z;
    }
}

}  // namespace kzg
