/* Oracle (test infrastructure only): narrow phase restated from the reference.
 *
 *   support functions      include/Kizuri/Geometry/Shape.h:152-154,183-187,223-226,520-523;
 *                          src/Geometry/Shapes.cpp:538-547
 *   SupportMap             include/Kizuri/Collision/GJK.h:121-146
 *   GJK                    src/Collision/GJK.cpp:11-244
 *   EPA                    src/Collision/EPA.cpp:16-296
 *   face clipping          src/Collision/CollideShape.cpp:30-228
 *   pair routines/dispatch src/Collision/CollideShape.cpp:233-430, 480-592
 */
#include "kzo_internal.h"

#include <string.h>

/* ---------------------------------------------------------------------------- */
/* Shapes                                                                       */
/* ---------------------------------------------------------------------------- */
static v3 support_local(const kzo_shape* s, v3 d) {
    switch (s->type) {
        case KZO_SPHERE: return vmul(vnormalized_or(d, V(0, 1, 0)), s->p[0]);
        case KZO_BOX:
            return V(d.x >= 0.0f ? s->p[0] : -s->p[0], d.y >= 0.0f ? s->p[1] : -s->p[1],
                     d.z >= 0.0f ? s->p[2] : -s->p[2]);
        case KZO_CAPSULE: {
            float sgn = d.y >= 0.0f ? s->p[0] : -s->p[0];
            return vadd(V(0.0f, sgn, 0.0f), vmul(vnormalized_or(d, V(0, 1, 0)), s->p[1]));
        }
        case KZO_HULL: {
            float best_dot = -INFINITY;
            v3 best = s->verts[0];
            for (int i = 0; i < s->nverts; ++i) {
                float dd = vdot(s->verts[i], d);
                if (dd > best_dot) { best_dot = dd; best = s->verts[i]; }
            }
            return best;
        }
        case KZO_PLANE:
            return vadd(vmul(V(s->p[0], s->p[1], s->p[2]), s->p[3]), vmul(d, 1.0e6f));
        default: return V(0, 0, 0);
    }
}

aabb kzo_world_bounds(const kzo_shape* s, qt r, v3 t) { return aabb_transformed(s->local, r, t); }

static kzo_sp smap_support(const kzo_smap* m, v3 d) {
    v3 la = qinv_rotate(m->ra, d);
    v3 lb = qinv_rotate(m->rb, vneg(d));
    kzo_sp sp;
    sp.pA = xform(m->ra, m->ta, support_local(m->a, la));
    sp.pB = xform(m->rb, m->tb, support_local(m->b, lb));
    sp.p = vsub(sp.pA, sp.pB);
    return sp;
}

/* ---------------------------------------------------------------------------- */
/* GJK                                                                          */
/* ---------------------------------------------------------------------------- */
static v3 closest_pt_triangle(v3 p, v3 a, v3 b, v3 c, float* u, float* v, float* w) {
    v3 ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    float d1 = vdot(ab, ap), d2 = vdot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) { *u = 1; *v = 0; *w = 0; return a; }
    v3 bp = vsub(p, b);
    float d3 = vdot(ab, bp), d4 = vdot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) { *u = 0; *v = 1; *w = 0; return b; }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float t = d1 / (d1 - d3);
        *u = 1 - t; *v = t; *w = 0;
        return vadd(a, vmul(ab, t));
    }
    v3 cp = vsub(p, c);
    float d5 = vdot(ab, cp), d6 = vdot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) { *u = 0; *v = 0; *w = 1; return c; }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float t = d2 / (d2 - d6);
        *u = 1 - t; *v = 0; *w = t;
        return vadd(a, vmul(ac, t));
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        *u = 0; *v = 1 - t; *w = t;
        return vadd(b, vmul(vsub(c, b), t));
    }
    float denom = 1.0f / (va + vb + vc);
    *v = vb * denom;
    *w = vc * denom;
    *u = 1.0f - *v - *w;
    return vadd(vadd(a, vmul(ab, *v)), vmul(ac, *w));
}

static int outside_face(v3 p0, v3 p1, v3 p2, v3 opp) {
    v3 n = vcross(vsub(p1, p0), vsub(p2, p0));
    if (vdot(n, vsub(opp, p0)) > 0.0f) n = vneg(n);
    return vdot(n, vsub(V(0, 0, 0), p0)) > 0.0f;
}

/* ReduceSimplex, GJK.cpp:57-148.  Returns 1 when the origin is enclosed. */
static int reduce_simplex(kzo_sp* s, uint32_t* count, v3* closest) {
    switch (*count) {
        case 1: *closest = s[0].p; break;
        case 2: {
            v3 a = s[0].p, b = s[1].p;
            v3 ab = vsub(b, a);
            float t = -vdot(a, ab);
            if (t <= 0.0f) { *closest = a; *count = 1; }
            else if (t >= vlen2(ab)) { s[0] = s[1]; *closest = b; *count = 1; }
            else { *closest = vadd(a, vmul(ab, t / vlen2(ab))); }
            break;
        }
        case 3: {
            float u, v, w;
            *closest = closest_pt_triangle(V(0, 0, 0), s[0].p, s[1].p, s[2].p, &u, &v, &w);
            kzo_sp tmp[3];
            memset(tmp, 0, sizeof tmp);   /* default SupportPoint = zero vectors */
            uint32_t n = 0;
            if (u > 0.0f) tmp[n++] = s[0];
            if (v > 0.0f) tmp[n++] = s[1];
            if (w > 0.0f) tmp[n++] = s[2];
            if (n == 0) n = 1;   /* only reachable with NaN weights: s[0] becomes zero */
            for (uint32_t i = 0; i < n; ++i) s[i] = tmp[i];
            *count = n;
            break;
        }
        case 4: {
            v3 a = s[0].p, b = s[1].p, c = s[2].p, d = s[3].p;
            int oABC = outside_face(a, b, c, d);
            int oACD = outside_face(a, c, d, b);
            int oADB = outside_face(a, d, b, c);
            int oBDC = outside_face(b, d, c, a);
            if (!oABC && !oACD && !oADB && !oBDC) return 1;
            float best = INFINITY;
            kzo_sp bt[3];
            uint32_t bc = 0;
            const uint32_t F[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
            const int O[4] = {oABC, oACD, oADB, oBDC};
            for (int f = 0; f < 4; ++f) {
                if (!O[f]) continue;
                float u, v, w;
                v3 p = closest_pt_triangle(V(0, 0, 0), s[F[f][0]].p, s[F[f][1]].p, s[F[f][2]].p, &u, &v, &w);
                float d2 = vlen2(p);
                if (d2 < best) {
                    best = d2;
                    uint32_t n = 0;
                    if (u > 0.0f) bt[n++] = s[F[f][0]];
                    if (v > 0.0f) bt[n++] = s[F[f][1]];
                    if (w > 0.0f) bt[n++] = s[F[f][2]];
                    bc = n;
                    *closest = p;
                }
            }
            for (uint32_t i = 0; i < bc; ++i) s[i] = bt[i];
            *count = bc;
            break;
        }
        default: break;
    }
    return 0;
}

kzo_gjk kzo_gjk_closest(const kzo_smap* m, float tol, uint32_t max_iter) {
    kzo_gjk r;
    memset(&r, 0, sizeof r);
    r.valid = 1;
    kzo_sp s[4];
    uint32_t count = 0;
    v3 d = V(1, 0, 0);
    s[count++] = smap_support(m, d);
    v3 closest = s[0].p;
    const float tol2 = tol * tol;
    for (uint32_t it = 0; it < max_iter; ++it) {
        r.iterations = it + 1;
        if (vlen2(closest) <= tol2) { r.intersect = 1; r.distance = 0; break; }
        d = vneg(closest);
        kzo_sp w = smap_support(m, d);
        float progress = vlen2(closest) - vdot(closest, w.p);
        if (progress <= tol * vlen2(closest)) break;
        int dup = 0;
        for (uint32_t i = 0; i < count; ++i)
            if (vlen2(vsub(s[i].p, w.p)) < tol2) { dup = 1; break; }
        if (dup) break;
        s[count++] = w;
        if (reduce_simplex(s, &count, &closest)) { r.intersect = 1; r.distance = 0; break; }
    }
    r.simplex_size = count;
    for (uint32_t i = 0; i < count; ++i) r.simplex[i] = s[i];
    if (!r.intersect) {
        float dist = vlen(closest);
        r.distance = dist;
        if (dist < KZO_EPS) r.intersect = 1;
        else r.normal = vdiv(vneg(closest), dist);
        if (count == 1) {
            r.pA = s[0].pA; r.pB = s[0].pB;
        } else if (count == 2) {
            v3 a = s[0].p, b = s[1].p, ab = vsub(b, a);
            float t = fclamp_r(-vdot(a, ab) / fmax_r(vlen2(ab), KZO_EPS), 0.0f, 1.0f);
            r.pA = vlerp(s[0].pA, s[1].pA, t);
            r.pB = vlerp(s[0].pB, s[1].pB, t);
        } else if (count == 3) {
            float u, v, w;
            closest_pt_triangle(V(0, 0, 0), s[0].p, s[1].p, s[2].p, &u, &v, &w);
            r.pA = vadd(vadd(vmul(s[0].pA, u), vmul(s[1].pA, v)), vmul(s[2].pA, w));
            r.pB = vadd(vadd(vmul(s[0].pB, u), vmul(s[1].pB, v)), vmul(s[2].pB, w));
        } else {
            r.pA = s[0].pA; r.pB = s[0].pB;
        }
    }
    return r;
}

/* ---------------------------------------------------------------------------- */
/* EPA                                                                          */
/* ---------------------------------------------------------------------------- */
typedef struct {
    uint32_t a, b, c;
    v3 n;
    float dist;
    int alive;
} epa_face;

static int build_face(epa_face* f, const kzo_sp* vs) {
    v3 A = vs[f->a].p, B = vs[f->b].p, C = vs[f->c].p;
    v3 n = vcross(vsub(B, A), vsub(C, A));
    float len = vlen(n);
    if (len < 1.0e-12f) return 0;
    n = vdiv(n, len);
    float d = vdot(n, A);
    if (d < 0.0f) { n = vneg(n); d = -d; uint32_t t = f->b; f->b = f->c; f->c = t; }
    f->n = n;
    f->dist = d;
    return 1;
}

static v3 epa_perp(v3 v) {
    if (fabs_r(v.x) <= fabs_r(v.y) && fabs_r(v.x) <= fabs_r(v.z)) return V(0.0f, -v.z, v.y);
    if (fabs_r(v.y) <= fabs_r(v.z)) return V(-v.z, 0.0f, v.x);
    return V(-v.y, v.x, 0.0f);
}

static int tet_ok(v3 a, v3 b, v3 c, v3 d) {
    v3 n = vcross(vsub(b, a), vsub(c, a));
    if (vdot(n, vsub(d, a)) > 0.0f) n = vneg(n);
    return vdot(n, vsub(V(0, 0, 0), a)) < -1.0e-9f;
}
static int origin_in_tetra(const kzo_sp* v) {
    return tet_ok(v[0].p, v[1].p, v[2].p, v[3].p) && tet_ok(v[0].p, v[2].p, v[3].p, v[1].p) &&
           tet_ok(v[0].p, v[3].p, v[1].p, v[2].p) && tet_ok(v[1].p, v[3].p, v[2].p, v[0].p);
}

/* BuildInitialTetra, EPA.cpp:58-147 */
static int build_initial_tetra(const kzo_smap* m, const kzo_gjk* g, kzo_sp* out) {
    uint32_t n = 0;
    for (uint32_t i = 0; i < g->simplex_size && n < 4; ++i) {
        int dup = 0;
        for (uint32_t j = 0; j < n; ++j)
            if (vlen2(vsub(out[j].p, g->simplex[i].p)) < 1.0e-12f) dup = 1;
        if (!dup) out[n++] = g->simplex[i];
    }
    if (n == 0) out[n++] = smap_support(m, V(1, 0, 0));
    if (n == 4 && !origin_in_tetra(out)) n = 3;
    if (n == 1) {
        out[n] = smap_support(m, vneg(out[0].p));
        if (vlen2(vsub(out[1].p, out[0].p)) > 1.0e-12f) ++n;
    }
    if (n == 2) {
        v3 ab = vsub(out[1].p, out[0].p);
        if (vlen2(ab) > 1.0e-12f) {
            v3 d1 = vnormalized(epa_perp(ab));
            v3 d2 = vnormalized(vcross(ab, d1));
            kzo_sp k0 = out[0], k1 = out[1];
            out[0] = smap_support(m, d1);
            out[1] = smap_support(m, vneg(d1));
            out[2] = smap_support(m, d2);
            out[3] = smap_support(m, vneg(d2));
            if (origin_in_tetra(out)) return 1;
            out[0] = k0; out[1] = k1;
        }
        kzo_sp s = smap_support(m, epa_perp(ab));
        if (vlen2(vsub(s.p, out[0].p)) > 1.0e-12f && vlen2(vsub(s.p, out[1].p)) > 1.0e-12f) out[n++] = s;
    }
    if (n == 3) {
        v3 tn = vcross(vsub(out[1].p, out[0].p), vsub(out[2].p, out[0].p));
        float len = vlen(tn);
        if (len > 1.0e-12f) {
            tn = vdiv(tn, len);
            float sd = vdot(tn, vsub(V(0, 0, 0), out[0].p));
            kzo_sp a = smap_support(m, sd > 0.0f ? vneg(tn) : tn);
            kzo_sp b = smap_support(m, sd > 0.0f ? tn : vneg(tn));
            out[3] = a;
            if (!origin_in_tetra(out)) out[3] = b;
            if (origin_in_tetra(out)) return 1;
        }
        n = 3;
    }
    if (n == 4 && origin_in_tetra(out)) return 1;

    kzo_sp cand[16];
    uint32_t nc = 0;
#define ADD_CAND(spv)                                                          \
    do {                                                                       \
        kzo_sp _sp = (spv);                                                    \
        int _d = 0;                                                            \
        for (uint32_t _i = 0; _i < nc; ++_i)                                   \
            if (vlen2(vsub(cand[_i].p, _sp.p)) < 1.0e-12f) { _d = 1; break; }  \
        if (!_d && nc < 16) cand[nc++] = _sp;                                  \
    } while (0)
    for (uint32_t i = 0; i < g->simplex_size && i < 4; ++i) ADD_CAND(g->simplex[i]);
    const float s = 0.5773502692f;
    const v3 dirs[14] = {V(1, 0, 0), V(-1, 0, 0), V(0, 1, 0), V(0, -1, 0), V(0, 0, 1), V(0, 0, -1),
                         V(s, s, s), V(s, s, -s), V(s, -s, s), V(-s, s, s), V(-s, -s, s), V(-s, s, -s),
                         V(s, -s, -s), V(-s, -s, -s)};
    for (int i = 0; i < 14; ++i) ADD_CAND(smap_support(m, dirs[i]));
#undef ADD_CAND
    for (uint32_t i = 0; i + 3 < nc; ++i)
        for (uint32_t j = i + 1; j + 2 < nc; ++j)
            for (uint32_t k = j + 1; k + 1 < nc; ++k)
                for (uint32_t l = k + 1; l < nc; ++l) {
                    kzo_sp t[4] = {cand[i], cand[j], cand[k], cand[l]};
                    float vol = vdot(vcross(vsub(t[1].p, t[0].p), vsub(t[2].p, t[0].p)), vsub(t[3].p, t[0].p));
                    if (fabs_r(vol) < 1.0e-12f) continue;
                    if (origin_in_tetra(t)) { for (int q = 0; q < 4; ++q) out[q] = t[q]; return 1; }
                }
    return 0;
}

static void finish_face(const epa_face* f, const kzo_sp* vs, kzo_epa* r) {
    v3 proj = vmul(f->n, f->dist);
    v3 a = vs[f->a].p, b = vs[f->b].p, c = vs[f->c].p;
    v3 v0 = vsub(b, a), v1 = vsub(c, a), v2 = vsub(proj, a);
    float d00 = vdot(v0, v0), d01 = vdot(v0, v1), d11 = vdot(v1, v1);
    float d20 = vdot(v2, v0), d21 = vdot(v2, v1);
    float denom = d00 * d11 - d01 * d01;
    float u, v, w;
    if (fabs_r(denom) < 1.0e-18f) { u = 1; v = 0; w = 0; }
    else {
        v = (d11 * d20 - d01 * d21) / denom;
        w = (d00 * d21 - d01 * d20) / denom;
        u = 1.0f - v - w;
    }
    r->valid = 1;
    r->depth = f->dist;
    r->normal = vneg(f->n);
    r->pA = vadd(vadd(vmul(vs[f->a].pA, u), vmul(vs[f->b].pA, v)), vmul(vs[f->c].pA, w));
    r->pB = vadd(vadd(vmul(vs[f->a].pB, u), vmul(vs[f->b].pB, v)), vmul(vs[f->c].pB, w));
}

kzo_epa kzo_epa_compute(const kzo_smap* m, const kzo_gjk* g, float tol, uint32_t max_iter) {
    kzo_epa r;
    memset(&r, 0, sizeof r);
    r.normal = V(0, 1, 0);
    kzo_sp verts[256];
    uint32_t nv = 0;
    kzo_sp tet[4];
    if (!build_initial_tetra(m, g, tet)) return r;
    for (int i = 0; i < 4; ++i) verts[nv++] = tet[i];
    epa_face faces[512];
    uint32_t nf = 0;
    const uint32_t T[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
    for (int i = 0; i < 4; ++i) {
        epa_face f = {T[i][0], T[i][1], T[i][2], V(0, 1, 0), 0.0f, 1};
        if (build_face(&f, verts)) faces[nf++] = f;
    }
    if (nf < 4) return r;
    const float eps = tol;
    for (uint32_t it = 0; it < max_iter; ++it) {
        r.iterations = it + 1;
        float bd = INFINITY;
        uint32_t bf = 0xFFFFFFFFu;
        for (uint32_t i = 0; i < nf; ++i)
            if (faces[i].alive && faces[i].dist < bd) { bd = faces[i].dist; bf = i; }
        if (bf == 0xFFFFFFFFu) break;
        epa_face* face = &faces[bf];
        kzo_sp w = smap_support(m, face->n);
        float d = vdot(w.p, face->n);
        if (d - face->dist < eps || nv >= 256) { finish_face(face, verts, &r); return r; }
        uint32_t ni = nv;
        verts[nv++] = w;
        uint32_t vis[512];
        uint32_t nvis = 0;
        for (uint32_t i = 0; i < nf; ++i)
            if (faces[i].alive && vdot(faces[i].n, w.p) - faces[i].dist > eps) { faces[i].alive = 0; vis[nvis++] = i; }
        uint32_t hu[256], hv[256];
        uint32_t nh = 0;
        for (uint32_t vi = 0; vi < nvis; ++vi) {
            const epa_face* fi = &faces[vis[vi]];
            uint32_t ev[3][2] = {{fi->a, fi->b}, {fi->b, fi->c}, {fi->c, fi->a}};
            for (int e = 0; e < 3; ++e) {
                int shared = 0;
                for (uint32_t vj = 0; vj < nvis && !shared; ++vj) {
                    if (vis[vj] == vis[vi]) continue;
                    const epa_face* fj = &faces[vis[vj]];
                    uint32_t gv[3][2] = {{fj->a, fj->b}, {fj->b, fj->c}, {fj->c, fj->a}};
                    for (int q = 0; q < 3; ++q)
                        if (gv[q][0] == ev[e][1] && gv[q][1] == ev[e][0]) { shared = 1; break; }
                }
                if (!shared && nh < 256) { hu[nh] = ev[e][0]; hv[nh] = ev[e][1]; ++nh; }
            }
        }
        uint32_t wi = 0;
        for (uint32_t i = 0; i < nf; ++i)
            if (faces[i].alive) faces[wi++] = faces[i];
        nf = wi;
        for (uint32_t i = 0; i < nh; ++i) {
            if (nf >= 512) break;
            epa_face f = {hv[i], hu[i], ni, V(0, 1, 0), 0.0f, 1};
            if (build_face(&f, verts)) faces[nf++] = f;
        }
    }
    float bd = INFINITY;
    uint32_t bf = 0xFFFFFFFFu;
    for (uint32_t i = 0; i < nf; ++i)
        if (faces[i].alive && faces[i].dist < bd) { bd = faces[i].dist; bf = i; }
    if (bf != 0xFFFFFFFFu) finish_face(&faces[bf], verts, &r);
    return r;
}

/* ---------------------------------------------------------------------------- */
/* Face clipping (CollidePolyhedral and helpers)                                */
/* ---------------------------------------------------------------------------- */
static int is_poly(const kzo_shape* s) { return s->type == KZO_BOX || s->type == KZO_HULL; }

/* GetShapeFace, CollideShape.cpp:30-98 */
static int shape_face(const kzo_shape* s, qt r, v3 t, v3 wdir, v3* out, uint32_t* cnt, v3* nworld) {
    if (s->type == KZO_BOX) {
        v3 ld = qinv_rotate(r, wdir);
        int axis = vmax_comp_index(vabs(ld));
        float sgn = vget(ld, axis) >= 0.0f ? 1.0f : -1.0f;
        v3 he = V(s->p[0], s->p[1], s->p[2]);
        v3 n = V(0, 0, 0);
        vset(&n, axis, sgn);
        v3 c = V(he.x * n.x, he.y * n.y, he.z * n.z);
        int a0 = (axis + 1) % 3, a1 = (axis + 2) % 3;
        float s0 = vget(he, a0), s1 = vget(he, a1);
        v3 cr[4];
        cr[0] = c; vset(&cr[0], a0, s0); vset(&cr[0], a1, s1);
        cr[1] = c; vset(&cr[1], a0, -s0); vset(&cr[1], a1, s1);
        cr[2] = c; vset(&cr[2], a0, -s0); vset(&cr[2], a1, -s1);
        cr[3] = c; vset(&cr[3], a0, s0); vset(&cr[3], a1, -s1);
        for (int i = 0; i < 4; ++i) out[i] = xform(r, t, cr[i]);
        *cnt = 4;
        *nworld = qrotate(r, n);
        return 1;
    }
    if (s->type == KZO_HULL) {
        v3 ld = qinv_rotate(r, wdir);
        float bd = -INFINITY;
        uint32_t bf = 0xFFFFFFFFu;
        uint32_t off = 0;
        for (int fi = 0; fi < s->nfaces; ++fi) {
            uint32_t n = s->sizes[fi];
            v3 a = s->verts[s->idx[off]], b = s->verts[s->idx[off + 1]], c = s->verts[s->idx[off + 2]];
            v3 fn = vnormalized_or(vcross(vsub(b, a), vsub(c, a)), V(0, 1, 0));
            float d = vdot(fn, ld);
            if (d > bd) { bd = d; bf = (uint32_t)fi; }
            off += n;
        }
        if (bf == 0xFFFFFFFFu) return 0;
        off = 0;
        for (uint32_t fi = 0; fi < bf; ++fi) off += s->sizes[fi];
        uint32_t n = s->sizes[bf];
        if (n > KZO_MAX_FACE_VERTS) n = KZO_MAX_FACE_VERTS;
        for (uint32_t i = 0; i < n; ++i) out[i] = xform(r, t, s->verts[s->idx[off + i]]);
        *cnt = n;
        v3 a = s->verts[s->idx[off]], b = s->verts[s->idx[off + 1]], c = s->verts[s->idx[off + 2]];
        *nworld = qrotate(r, vnormalized_or(vcross(vsub(b, a), vsub(c, a)), V(0, 1, 0)));
        return 1;
    }
    return 0;
}

typedef struct { v3 v[KZO_MAX_FACE_VERTS * 2]; uint32_t n; } clip_poly;

static void clip_add(clip_poly* p, v3 v) { if (p->n < KZO_MAX_FACE_VERTS * 2) p->v[p->n++] = v; }

static void clip_plane(const clip_poly* in, v3 pn, float pd, clip_poly* out) {
    out->n = 0;
    if (in->n == 0) return;
    for (uint32_t i = 0; i < in->n; ++i) {
        v3 cur = in->v[i], nxt = in->v[(i + 1) % in->n];
        float dc = vdot(pn, cur) - pd, dn = vdot(pn, nxt) - pd;
        if (dc <= 0.0f) clip_add(out, cur);
        if ((dc <= 0.0f) != (dn <= 0.0f)) {
            float t = dc / (dc - dn);
            clip_add(out, vlerp(cur, nxt, t));
        }
    }
}

static uint32_t collide_polyhedral(const kzo_shape* sa, qt ra, v3 ta, const kzo_shape* sb, qt rb, v3 tb,
                                   float max_sep, kzo_manifold* m, v3 normal) {
    v3 fa[KZO_MAX_FACE_VERTS], fb[KZO_MAX_FACE_VERTS], na, nb;
    uint32_t ca = 0, cb = 0;
    int ha = shape_face(sa, ra, ta, vneg(normal), fa, &ca, &na);
    int hb = shape_face(sb, rb, tb, normal, fb, &cb, &nb);
    if (!ha || !hb) return 0;
    float al_a = vdot(na, vneg(normal));
    float al_b = vdot(nb, normal);
    v3 *rv, *iv;
    uint32_t rc, ic;
    int ref_a;
    if (al_a >= al_b) { rv = fa; rc = ca; iv = fb; ic = cb; ref_a = 1; }
    else { rv = fb; rc = cb; iv = fa; ic = ca; ref_a = 0; }
    v3 rn = ref_a ? na : nb;
    float rd = vdot(rn, rv[0]);
    clip_poly poly, tmp;
    poly.n = 0;
    for (uint32_t i = 0; i < ic; ++i) clip_add(&poly, iv[i]);
    v3 cen = V(0, 0, 0);
    for (uint32_t i = 0; i < rc; ++i) cen = vadd(cen, rv[i]);
    cen = vdiv(cen, (float)rc);
    for (uint32_t i = 0; i < rc; ++i) {
        v3 v0 = rv[i], v1 = rv[(i + 1) % rc];
        v3 sn = vcross(vsub(v1, v0), rn);
        float len = vlen(sn);
        if (len < 1.0e-9f) continue;
        sn = vdiv(sn, len);
        if (vdot(sn, vsub(v0, cen)) < 0.0f) sn = vneg(sn);
        float sd = vdot(sn, v0);
        clip_plane(&poly, sn, sd, &tmp);
        poly = tmp;
        if (poly.n == 0) break;
    }
    uint32_t nc = 0;
    for (uint32_t i = 0; i < poly.n && nc < KZO_MAX_MANIFOLD; ++i) {
        v3 p = poly.v[i];
        float sep = vdot(rn, p) - rd;
        if (sep > max_sep) continue;
        kzo_cpoint cp;
        v3 proj = vsub(p, vmul(rn, sep));
        if (ref_a) { cp.pA = proj; cp.pB = p; }
        else { cp.pA = p; cp.pB = proj; }
        cp.n = normal;
        cp.sep = sep;
        cp.feature = i;
        m->pts[nc++] = cp;
    }
    if (nc > 4) {
        kzo_cpoint kept[4];
        for (uint32_t i = 0; i < 4; ++i) kept[i] = m->pts[i * (nc - 1) / 3];
        for (uint32_t i = 0; i < 4; ++i) m->pts[i] = kept[i];
        nc = 4;
    }
    m->n = nc;
    return nc;
}

static void add_point(kzo_manifold* m, v3 pA, v3 pB, v3 n, float sep) {
    if (m->n < KZO_MAX_MANIFOLD) {
        kzo_cpoint* c = &m->pts[m->n++];
        c->pA = pA; c->pB = pB; c->n = n; c->sep = sep; c->feature = 0;
    }
}

static void swap_manifold(kzo_manifold* m) {
    for (uint32_t i = 0; i < m->n; ++i) {
        v3 t = m->pts[i].pA;
        m->pts[i].pA = m->pts[i].pB;
        m->pts[i].pB = t;
        m->pts[i].n = vneg(m->pts[i].n);
    }
}

/* CollideConvexGeneric, CollideShape.cpp:233-299 */
static uint32_t collide_generic(const kzo_shape* sa, qt ra, v3 ta, const kzo_shape* sb, qt rb, v3 tb,
                                float max_sep, float tol, kzo_manifold* m) {
    kzo_smap map = {sa, sb, ra, rb, ta, tb};
    kzo_gjk g = kzo_gjk_closest(&map, tol, 32);
    if (!g.intersect) {
        if (g.distance > max_sep) return 0;
        if (is_poly(sa) && is_poly(sb) && vlen2(g.normal) > 0.0f) {
            if (collide_polyhedral(sa, ra, ta, sb, rb, tb, max_sep, m, g.normal) > 0) return m->n;
        }
        add_point(m, g.pA, g.pB, g.normal, g.distance);
        return m->n;
    }
    if (is_poly(sa) && is_poly(sb)) {
        kzo_epa e = kzo_epa_compute(&map, &g, tol, 64);
        if (e.valid) {
            if (collide_polyhedral(sa, ra, ta, sb, rb, tb, max_sep, m, e.normal) > 0) return m->n;
            add_point(m, e.pA, e.pB, e.normal, -e.depth);
            return m->n;
        }
    }
    kzo_epa e = kzo_epa_compute(&map, &g, tol, 64);
    if (e.valid) {
        add_point(m, e.pA, e.pB, e.normal, -e.depth);
        return m->n;
    }
    add_point(m, g.pA, g.pB, vlen2(g.normal) > 0.0f ? g.normal : V(0, 1, 0), 0.0f);
    return m->n;
}

/* CollideSphereConvex, CollideShape.cpp:304-344 */
static uint32_t collide_sphere_convex(const kzo_shape* sph, qt rs, v3 ts, const kzo_shape* sb, qt rb, v3 tb,
                                      float max_sep, float tol, kzo_manifold* m) {
    kzo_shape point;
    memset(&point, 0, sizeof point);
    point.type = KZO_SPHERE;
    point.p[0] = 1.0e-4f;
    kzo_smap map = {&point, sb, rs, rb, ts, tb};
    kzo_gjk g = kzo_gjk_closest(&map, tol, 32);
    float radius = sph->p[0];
    v3 center = ts;
    v3 cb = g.pB;
    if (g.intersect) {
        kzo_epa e = kzo_epa_compute(&map, &g, tol, 64);
        if (e.valid) {
            v3 n = vneg(e.normal);
            add_point(m, vadd(center, vmul(n, radius)), e.pB, n, -(e.depth + radius));
            return m->n;
        }
        return 0;
    }
    float dist = g.distance;
    float sep = dist - radius;
    if (sep > max_sep) return 0;
    v3 n = (dist > KZO_EPS) ? vdiv(vsub(center, cb), dist) : V(0, 1, 0);
    add_point(m, vsub(center, vmul(n, radius)), cb, n, sep);
    return m->n;
}

/* CollideSphereSphere, CollideShape.cpp:349-365 */
static uint32_t collide_sphere_sphere(const kzo_shape* a, v3 ta, const kzo_shape* b, v3 tb, float max_sep,
                                      kzo_manifold* m) {
    v3 d = vsub(ta, tb);
    float dist = vlen(d);
    float sep = dist - (a->p[0] + b->p[0]);
    if (sep > max_sep) return 0;
    v3 n = dist > KZO_EPS ? vdiv(d, dist) : V(0, 1, 0);
    add_point(m, vsub(ta, vmul(n, a->p[0])), vadd(tb, vmul(n, b->p[0])), n, sep);
    return m->n;
}

/* CollidePlaneConvex, CollideShape.cpp:370-430 */
static uint32_t collide_plane_convex(const kzo_shape* pl, qt rp, v3 tp, const kzo_shape* sb, qt rb, v3 tb,
                                     float max_sep, kzo_manifold* m) {
    v3 pn = qrotate(rp, V(pl->p[0], pl->p[1], pl->p[2]));
    float pd = pl->p[3] + vdot(pn, tp);
    if (is_poly(sb)) {
        v3 verts[KZO_MAX_FACE_VERTS];
        uint32_t n = 0;
        if (sb->type == KZO_BOX) {
            v3 he = V(sb->p[0], sb->p[1], sb->p[2]);
            for (int i = 0; i < 8; ++i) {
                v3 c = V((i & 1) ? he.x : -he.x, (i & 2) ? he.y : -he.y, (i & 4) ? he.z : -he.z);
                verts[n++] = xform(rb, tb, c);
            }
        } else {
            for (int i = 0; i < sb->nverts && n < KZO_MAX_FACE_VERTS; ++i) verts[n++] = xform(rb, tb, sb->verts[i]);
        }
        uint32_t count = 0;
        for (uint32_t i = 0; i < n && count < KZO_MAX_MANIFOLD; ++i) {
            float d = vdot(pn, verts[i]) - pd;
            if (d > max_sep) continue;
            kzo_cpoint* cp = &m->pts[count++];
            cp->n = pn;
            cp->pA = verts[i];
            cp->pB = vsub(verts[i], vmul(pn, d));
            cp->sep = d;
            cp->feature = 0;
        }
        if (count > 4) {
            kzo_cpoint kept[4];
            for (uint32_t i = 0; i < 4; ++i) kept[i] = m->pts[i * (count - 1) / 3];
            for (uint32_t i = 0; i < 4; ++i) m->pts[i] = kept[i];
            count = 4;
        }
        m->n = count;
        return count;
    }
    v3 ld = qinv_rotate(rb, vneg(pn));
    v3 deep = xform(rb, tb, support_local(sb, ld));
    float d = vdot(pn, deep) - pd;
    if (d > max_sep) return 0;
    add_point(m, deep, vsub(deep, vmul(pn, d)), pn, d);
    return m->n;
}

uint32_t kzo_collide(const kzo_shape* sa, qt ra, v3 ta, const kzo_shape* sb, qt rb, v3 tb, float max_sep,
                     float tol, kzo_manifold* out) {
    out->n = 0;
    if (sa->type == KZO_PLANE) {
        uint32_t n = collide_plane_convex(sa, ra, ta, sb, rb, tb, max_sep, out);
        if (n > 0) swap_manifold(out);
        return n;
    }
    if (sb->type == KZO_PLANE) return collide_plane_convex(sb, rb, tb, sa, ra, ta, max_sep, out);
    if (sa->type == KZO_SPHERE && sb->type == KZO_SPHERE) return collide_sphere_sphere(sa, ta, sb, tb, max_sep, out);
    if (sa->type == KZO_SPHERE) return collide_sphere_convex(sa, ra, ta, sb, rb, tb, max_sep, tol, out);
    if (sb->type == KZO_SPHERE) {
        uint32_t n = collide_sphere_convex(sb, rb, tb, sa, ra, ta, max_sep, tol, out);
        if (n > 0) swap_manifold(out);
        return n;
    }
    return collide_generic(sa, ra, ta, sb, rb, tb, max_sep, tol, out);
}

/* NarrowPhase::CastShape (CollideShape.cpp:607-661): conservative advancement of A along
 * `direction` (up to max_distance) against B with GJK distance; planes analytically. */
int kzo_cast_shape(const kzo_shape* sa, qt ra, v3 ta, v3 direction, float max_distance, const kzo_shape* sb, qt rb,
                   v3 tb, float* out_fraction, v3* out_normal) {
    const float dir_len = vlen(direction);
    if (dir_len < KZO_EPS) return 0;
    const v3 dir = vdiv(direction, dir_len);
    if (sb->type == KZO_PLANE) {
        if (sa->type == KZO_PLANE) return 0;
        const v3 pn = V(sb->p[0], sb->p[1], sb->p[2]);
        const v3 n_world = vnormalized(qrotate(rb, pn));
        const v3 point_on_plane = xform(rb, tb, vmul(pn, sb->p[3]));
        const float plane_dist = vdot(n_world, point_on_plane);
        const v3 local_dir_a = qinv_rotate(ra, vneg(n_world));
        const v3 deepest = xform(ra, ta, support_local(sa, local_dir_a));
        const float sd = vdot(n_world, deepest) - plane_dist;
        if (sd <= 1.0e-4f) {
            *out_fraction = 0.0f;
            *out_normal = n_world;
            return 1;
        }
        const float rate = vdot(n_world, dir);
        if (rate >= -KZO_EPS) return 0; /* moving parallel / away */
        const float t_hit = sd / (-rate);
        if (t_hit > max_distance) return 0;
        *out_fraction = t_hit / max_distance;
        *out_normal = n_world;
        return 1;
    }
    float t = 0.0f;
    const float tol = 1.0e-4f;
    for (uint32_t iter = 0; iter < 64; ++iter) {
        const v3 cur = vadd(ta, vmul(dir, t));
        kzo_smap map = {sa, sb, ra, rb, cur, tb};
        kzo_gjk g = kzo_gjk_closest(&map, tol, 32);
        if (g.intersect || g.distance <= tol) {
            *out_fraction = t / max_distance;
            *out_normal = g.normal;
            return 1;
        }
        if (t >= max_distance) return 0;
        float advance = g.distance - tol;
        if (advance <= 0.0f) advance = tol;
        t += advance;
        if (t > max_distance) return 0;
    }
    return 0;
}
