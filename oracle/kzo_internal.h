/* Oracle internals (test infrastructure only).  See kzo.h for the test-facing API. */
#ifndef KZO_INTERNAL_H
#define KZO_INTERNAL_H

#include "kzo_math.h"
#include <stddef.h>

enum { KZO_SPHERE = 0, KZO_BOX = 1, KZO_CAPSULE = 2, KZO_HULL = 4, KZO_PLANE = 8 };
enum { KZO_STATIC = 0, KZO_KINEMATIC = 1, KZO_DYNAMIC = 2 };

#define KZO_MAX_MANIFOLD 8   /* kMaxManifoldPoints, ContactManifold.h:11 */
#define KZO_MAX_FACE_VERTS 16 /* kMaxFaceVerts, CollideShape.cpp:26 */

typedef struct {
    int type;
    float p[4];               /* sphere r | box half xyz | capsule halfHeight, radius | plane n, d */
    int nverts, nfaces, nidx;
    v3* verts;                /* hull vertices in ConvexHullShape order */
    uint8_t* sizes;           /* hull face sizes */
    uint32_t* idx;            /* hull face indices */
    aabb local;               /* GetLocalBounds() */
} kzo_shape;

typedef struct {
    v3 pA, pB, n;
    float sep;
    uint32_t feature;
} kzo_cpoint;

typedef struct {
    kzo_cpoint pts[KZO_MAX_MANIFOLD];
    uint32_t n;
} kzo_manifold;

/* Narrow phase entry (NarrowPhase::Collide, CollideShape.cpp:480-592). */
uint32_t kzo_collide(const kzo_shape* sa, qt ra, v3 ta, const kzo_shape* sb, qt rb, v3 tb,
                     float max_sep, float tol, kzo_manifold* out);
aabb kzo_world_bounds(const kzo_shape* s, qt r, v3 t);
int kzo_cast_shape(const kzo_shape* sa, qt ra, v3 ta, v3 direction, float max_distance, const kzo_shape* sb, qt rb,
                   v3 tb, float* out_fraction, v3* out_normal);

/* GJK / EPA results exposed for the known-answer tests. */
typedef struct { v3 pA, pB, p; } kzo_sp;
typedef struct {
    int intersect, valid;
    float distance;
    v3 pA, pB, normal;
    uint32_t iterations, simplex_size;
    kzo_sp simplex[4];
} kzo_gjk;
typedef struct {
    int valid;
    float depth;
    v3 normal, pA, pB;
    uint32_t iterations;
} kzo_epa;

typedef struct {
    const kzo_shape *a, *b;
    qt ra, rb;
    v3 ta, tb;
} kzo_smap;

kzo_gjk kzo_gjk_closest(const kzo_smap* m, float tol, uint32_t max_iter);
kzo_epa kzo_epa_compute(const kzo_smap* m, const kzo_gjk* g, float tol, uint32_t max_iter);

#endif
