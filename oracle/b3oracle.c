/*
 * b3oracle.c -- CPU oracle for the GPU rigid-body step.  TEST INFRASTRUCTURE ONLY
 * (used by tests/, the smoke check and the bench's CPU-baseline leg; never by the product).
 *
 * Restates, in plain C, the reference CPU code the GPU path must agree with.  Paths are
 * relative to the reference project's src/ directory.  Compile with -ffp-contract=off.
 */
#include "b3oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SHAPE_CONVEX_HULL 3
#define SHAPE_PLANE 4
#define SHAPE_SPHERE 7
#define SHAPE_COMPOUND_OF_CONVEX_HULLS 6

static int g_threads = 1;
int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void oracle_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

/* ------------------------------------------------------------------ vector math (fixed order) */
typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } qt;
typedef struct { v3 r0, r1, r2; } m3;

static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 f4v(of4 a) { return mk(a.x, a.y, a.z); }
static inline qt f4q(of4 a) { qt q = {a.x, a.y, a.z, a.w}; return q; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 lscl(float s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
/* b3Vector3::normalized / normalize: scale by the reciprocal length (Bullet3Common/b3Vector3.h:260-300) */
static inline v3 nrm(v3 a) { float inv = 1.0f / sqrtf(dot(a, a)); return mk(a.x * inv, a.y * inv, a.z * inv); }

static inline m3 qmat(qt q) {
    float d = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    float s = 2.0f / d;
    float xs = q.x * s, ys = q.y * s, zs = q.z * s;
    float wx = q.w * xs, wy = q.w * ys, wz = q.w * zs;
    float xx = q.x * xs, xy = q.x * ys, xz = q.x * zs;
    float yy = q.y * ys, yz = q.y * zs, zz = q.z * zs;
    m3 m;
    m.r0 = mk(1.0f - (yy + zz), xy - wz, xz + wy);
    m.r1 = mk(xy + wz, 1.0f - (xx + zz), yz - wx);
    m.r2 = mk(xz - wy, yz + wx, 1.0f - (xx + yy));
    return m;
}
static inline v3 mmul(const m3* m, v3 v) { return mk(dot(m->r0, v), dot(m->r1, v), dot(m->r2, v)); }
static inline v3 mtmul(const m3* m, v3 v) {
    return mk(m->r0.x * v.x + m->r1.x * v.y + m->r2.x * v.z, m->r0.y * v.x + m->r1.y * v.y + m->r2.y * v.z,
              m->r0.z * v.x + m->r1.z * v.y + m->r2.z * v.z);
}
static inline v3 imul(const omat3* m, v3 v) {
    return mk(m->row[0].x * v.x + m->row[0].y * v.y + m->row[0].z * v.z,
              m->row[1].x * v.x + m->row[1].y * v.y + m->row[1].z * v.z,
              m->row[2].x * v.x + m->row[2].y * v.y + m->row[2].z * v.z);
}
static inline qt qmul(qt a, qt b) {
    qt r;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
    r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    return r;
}

/* b3Quaternion * b3Vector3, scalar branch (Bullet3Common/b3Quaternion.h:651-729) */
static inline qt qmulv(qt q, v3 w) {
    qt r;
    r.x = q.w * w.x + q.y * w.z - q.z * w.y;
    r.y = q.w * w.y + q.z * w.x - q.x * w.z;
    r.z = q.w * w.z + q.x * w.y - q.y * w.x;
    r.w = -q.x * w.x - q.y * w.y - q.z * w.z;
    return r;
}
static inline qt qconj(qt q) { qt r = {-q.x, -q.y, -q.z, q.w}; return r; }
/* b3QuatRotate (b3Quaternion.h:868-879): (q * v) * q^-1 */
static inline v3 qrotq(qt q, v3 v) { qt t = qmul(qmulv(q, v), qconj(q)); return mk(t.x, t.y, t.z); }
/* b3Matrix3x3::getRotation, scalar branch (Bullet3Common/b3Matrix3x3.h:457-491) */
static qt quat_from_mat(const m3* m) {
    float e[3][3] = {{m->r0.x, m->r0.y, m->r0.z}, {m->r1.x, m->r1.y, m->r1.z}, {m->r2.x, m->r2.y, m->r2.z}};
    float t[4], trace = e[0][0] + e[1][1] + e[2][2];
    qt q;
    if (trace > 0.0f) {
        float s = sqrtf(trace + 1.0f);
        t[3] = s * 0.5f;
        s = 0.5f / s;
        t[0] = (e[2][1] - e[1][2]) * s;
        t[1] = (e[0][2] - e[2][0]) * s;
        t[2] = (e[1][0] - e[0][1]) * s;
    } else {
        int i = e[0][0] < e[1][1] ? (e[1][1] < e[2][2] ? 2 : 1) : (e[0][0] < e[2][2] ? 2 : 0);
        int j = (i + 1) % 3, k = (i + 2) % 3;
        float s = sqrtf(e[i][i] - e[j][j] - e[k][k] + 1.0f);
        t[i] = s * 0.5f;
        s = 0.5f / s;
        t[3] = (e[k][j] - e[j][k]) * s;
        t[j] = (e[j][i] + e[i][j]) * s;
        t[k] = (e[k][i] + e[i][k]) * s;
    }
    q.x = t[0]; q.y = t[1]; q.z = t[2]; q.w = t[3];
    return q;
}
static inline m3 mtrans(const m3* m) {
    m3 r;
    r.r0 = mk(m->r0.x, m->r1.x, m->r2.x);
    r.r1 = mk(m->r0.y, m->r1.y, m->r2.y);
    r.r2 = mk(m->r0.z, m->r1.z, m->r2.z);
    return r;
}
/* m1 * m2 with element (i,j) = m2.tdot_j(m1[i]) (b3Matrix3x3.h:1190-1272) */
static inline v3 mrow_times(v3 a, const m3* m2) {
    return mk(m2->r0.x * a.x + m2->r1.x * a.y + m2->r2.x * a.z, m2->r0.y * a.x + m2->r1.y * a.y + m2->r2.y * a.z,
              m2->r0.z * a.x + m2->r1.z * a.y + m2->r2.z * a.z);
}
static inline m3 mmul33(const m3* m1, const m3* m2) {
    m3 r;
    r.r0 = mrow_times(m1->r0, m2);
    r.r1 = mrow_times(m1->r1, m2);
    r.r2 = mrow_times(m1->r2, m2);
    return r;
}
/* b3Transform::inverse applied to p: basis^T p + basis^T (-origin) (b3Transform.h:182-186) */
static inline v3 xform_inv(const m3* R, v3 origin, v3 p) {
    m3 t = mtrans(R);
    return add(mmul(&t, p), mmul(&t, neg(origin)));
}

/* ------------------------------------------------------------------ AABBs */
/* b3TransformAabb2 (Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h:24-43) */
static void transform_aabb(const oaabb* local, v3 pos, qt q, float margin, v3* mn, v3* mx) {
    v3 lmin = mk(local->minv[0], local->minv[1], local->minv[2]);
    v3 lmax = mk(local->maxv[0], local->maxv[1], local->maxv[2]);
    v3 he = lscl(0.5f, sub(lmax, lmin));
    he = add(he, mk(margin, margin, margin));
    v3 lc = lscl(0.5f, add(lmax, lmin));
    m3 m = qmat(q);
    m3 a;
    a.r0 = mk(fabsf(m.r0.x), fabsf(m.r0.y), fabsf(m.r0.z));
    a.r1 = mk(fabsf(m.r1.x), fabsf(m.r1.y), fabsf(m.r1.z));
    a.r2 = mk(fabsf(m.r2.x), fabsf(m.r2.y), fabsf(m.r2.z));
    v3 c = add(mmul(&m, lc), pos);
    v3 e = mk(dot(he, a.r0), dot(he, a.r1), dot(he, a.r2));
    *mn = sub(c, e);
    *mx = add(c, e);
}

void oracle_aabbs(const obody* bodies, int n, const oshapes* sh, oaabb* out) {
    int i;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (i = 0; i < n; i++) {
        const obody* b = &bodies[i];
        v3 mn, mx;
        qt q = f4q(b->quat);
        transform_aabb(&sh->local_aabbs[b->collidableIdx], f4v(b->pos), q, 0.f, &mn, &mx);
        out[i].minv[0] = mn.x; out[i].minv[1] = mn.y; out[i].minv[2] = mn.z; out[i].minw = i;
        out[i].maxv[0] = mx.x; out[i].maxv[1] = mx.y; out[i].maxv[2] = mx.z;
        out[i].maxw = b->invMass == 0.f ? 0 : 1;
    }
}

/* ------------------------------------------------------------------ pairs */
static inline int overlap(const oaabb* a, const oaabb* b) {
    return (a->minv[0] <= b->maxv[0]) && (b->minv[0] <= a->maxv[0]) && (a->minv[1] <= b->maxv[1]) &&
           (b->minv[1] <= a->maxv[1]) && (a->minv[2] <= b->maxv[2]) && (b->minv[2] <= a->maxv[2]);
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

int oracle_pairs_bruteforce(const oaabb* aabbs, int n, opair* out, int cap) {
    int count = 0, i, j;
    for (i = 0; i < n; i++)
        for (j = i + 1; j < n; j++) {
            if (aabbs[i].maxw == 0 && aabbs[j].maxw == 0) continue; /* static-static */
            if (overlap(&aabbs[i], &aabbs[j])) {
                if (count < cap) {
                    out[count].x = i; out[count].y = j; out[count].z = -1; out[count].w = -1;
                }
                count++;
            }
        }
    return count;
}

typedef struct { int64_t cx, cy, cz; int idx; } cellrec;
static int cmp_cell(const void* a, const void* b) {
    const cellrec* p = (const cellrec*)a;
    const cellrec* q = (const cellrec*)b;
    if (p->cx != q->cx) return p->cx < q->cx ? -1 : 1;
    if (p->cy != q->cy) return p->cy < q->cy ? -1 : 1;
    if (p->cz != q->cz) return p->cz < q->cz ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx ? 1 : 0);
}
static int find_cell(const cellrec* r, int n, int64_t x, int64_t y, int64_t z) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        const cellrec* m = &r[mid];
        int less = m->cx < x || (m->cx == x && (m->cy < y || (m->cy == y && m->cz < z)));
        if (less) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* Exact pair set through an unbounded integer grid (no hash wrap): dynamic bodies in cells
 * of size `cell` (>= every dynamic AABB extent), neighbours in 27 cells; statics test every
 * dynamic body.  Output sorted by (a, b). */
int oracle_pairs_grid(const oaabb* aabbs, int n, float cell, opair* out, int cap) {
    float inv = 1.f / cell;
    int nd = 0, ns = 0, i;
    cellrec* rec = (cellrec*)malloc(sizeof(cellrec) * (size_t)(n > 0 ? n : 1));
    int* statics = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (i = 0; i < n; i++) {
        if (aabbs[i].maxw) {
            float cx = (aabbs[i].minv[0] + aabbs[i].maxv[0]) * 0.5f;
            float cy = (aabbs[i].minv[1] + aabbs[i].maxv[1]) * 0.5f;
            float cz = (aabbs[i].minv[2] + aabbs[i].maxv[2]) * 0.5f;
            rec[nd].cx = (int64_t)floorf(cx * inv);
            rec[nd].cy = (int64_t)floorf(cy * inv);
            rec[nd].cz = (int64_t)floorf(cz * inv);
            rec[nd].idx = i;
            nd++;
        } else {
            statics[ns++] = i;
        }
    }
    qsort(rec, (size_t)nd, sizeof(cellrec), cmp_cell);
    size_t kcap = 1024, kn = 0;
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * kcap);
    int t;
    for (t = 0; t < nd; t++) {
        int a = rec[t].idx;
        int dx, dy, dz;
        for (dx = -1; dx <= 1; dx++)
            for (dy = -1; dy <= 1; dy++)
                for (dz = -1; dz <= 1; dz++) {
                    int64_t x = rec[t].cx + dx, y = rec[t].cy + dy, z = rec[t].cz + dz;
                    int s = find_cell(rec, nd, x, y, z);
                    for (; s < nd && rec[s].cx == x && rec[s].cy == y && rec[s].cz == z; s++) {
                        int b = rec[s].idx;
                        if (b <= a) continue;
                        if (overlap(&aabbs[a], &aabbs[b])) {
                            if (kn == kcap) { kcap *= 2; keys = (uint64_t*)realloc(keys, sizeof(uint64_t) * kcap); }
                            keys[kn++] = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
                        }
                    }
                }
        {
            int l;
            for (l = 0; l < ns; l++) {
                int s2 = statics[l];
                if (overlap(&aabbs[a], &aabbs[s2])) {
                    int lo = a < s2 ? a : s2, hi = a < s2 ? s2 : a;
                    if (kn == kcap) { kcap *= 2; keys = (uint64_t*)realloc(keys, sizeof(uint64_t) * kcap); }
                    keys[kn++] = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
                }
            }
        }
    }
    qsort(keys, kn, sizeof(uint64_t), cmp_u64);
    {
        size_t k;
        for (k = 0; k < kn && (int)k < cap; k++) {
            out[k].x = (int)(keys[k] >> 32);
            out[k].y = (int)(keys[k] & 0xffffffffu);
            out[k].z = -1;
            out[k].w = -1;
        }
    }
    free(keys);
    free(rec);
    free(statics);
    return (int)kn;
}

/* ------------------------------------------------------------------ contacts */
static int sgn_index(const obody* bodies, int i) { return bodies[i].invMass == 0.f ? -i : i; }

static void write_header(ocontact* c, const obody* bodies, int A, int B, v3 n, int np, unsigned short fr) {
    c->worldNormalOnB.x = n.x; c->worldNormalOnB.y = n.y; c->worldNormalOnB.z = n.z; c->worldNormalOnB.w = (float)np;
    c->restitutionCmp = 0;
    c->frictionCmp = fr;
    c->batchIdx = 0;
    c->bodyA = sgn_index(bodies, A);
    c->bodyB = sgn_index(bodies, B);
    c->childIndexA = -1;
    c->childIndexB = -1;
    c->unused1 = 0;
    c->unused2 = 0;
}

typedef struct { float x, y, z, w; } p4;

/* b3ReduceContacts (Bullet3Collision/NarrowPhaseCollision/shared/b3ReduceContacts.h:4-87) and its
 * twin extractManifoldSequentialGlobal (b3ConvexHullContact.cpp:418-500) */
static int reduce_contacts(const p4* p, int n, v3 nearNormal, int idx[4]) {
    float cx = 0.f, cy = 0.f, cz = 0.f, inv, minW = FLT_MAX, m0 = FLT_MIN, m1 = FLT_MIN, m2 = FLT_MIN, m3v = FLT_MIN;
    int i, ie, minIndex = -1;
    v3 center, aVector, u, v, nu, nv;
    idx[0] = 0; idx[1] = 1; idx[2] = 2; idx[3] = 3;
    if (n == 0) return 0;
    if (n <= 4) return n;
    if (n > 64) n = 64;
    for (i = 0; i < n; i++) {
        cx = cx + p[i].x;
        cy = cy + p[i].y;
        cz = cz + p[i].z;
    }
    inv = 1.0f / (float)n;
    cx = cx * inv; cy = cy * inv; cz = cz * inv;
    center = mk(cx, cy, cz);
    aVector = sub(mk(p[0].x, p[0].y, p[0].z), center);
    u = cross(nearNormal, aVector);
    v = cross(nearNormal, u);
    u = nrm(u);
    v = nrm(v);
    nu = neg(u);
    nv = neg(v);
    for (ie = 0; ie < n; ie++) {
        v3 r;
        float f;
        if (p[ie].w < minW) { minW = p[ie].w; minIndex = ie; }
        r = sub(mk(p[ie].x, p[ie].y, p[ie].z), center);
        f = dot(u, r); if (f < m0) { m0 = f; idx[0] = ie; }
        f = dot(nu, r); if (f < m1) { m1 = f; idx[1] = ie; }
        f = dot(v, r); if (f < m2) { m2 = f; idx[2] = ie; }
        f = dot(nv, r); if (f < m3v) { m3v = f; idx[3] = ie; }
    }
    if (idx[0] != minIndex && idx[1] != minIndex && idx[2] != minIndex && idx[3] != minIndex) idx[0] = minIndex;
    return 4;
}

/* computeContactPlaneConvex (Bullet3OpenCL/NarrowphaseCollision/b3ConvexHullContact.cpp:1272-1395);
 * A = plane body, B = hull body */
static int plane_hull(const obody* bodies, const oshapes* sh, int A, int B, ocontact* c, unsigned short fr) {
    const obody* BA = &bodies[A];
    const obody* BB = &bodies[B];
    const ohull* hull = &sh->hulls[sh->cols[BB->collidableIdx].shapeIndex];
    v3 posB = f4v(BB->pos), posA = f4v(BA->pos);
    of4 pe = sh->faces[sh->cols[BA->collidableIdx].shapeIndex].plane;
    v3 planeNormal = mk(pe.x, pe.y, pe.z);
    float planeConstant = pe.w, maxDot = -1e30f;
    m3 RA = qmat(f4q(BA->quat)), RB = qmat(f4q(BB->quat));
    v3 planeNormalWorld = qrotq(f4q(BA->quat), planeNormal);
    /* planeInConvex = convexWorldTransform.inverse() * planeTransform (b3ConvexHullContact.cpp:1310-1318) */
    m3 RBt = mtrans(&RB);
    m3 PinC = mmul33(&RBt, &RA);
    v3 planeNormalInConvex = mmul(&PinC, neg(planeNormal));
    p4 pts[64];
    int numPoints = 0, i, idx[4], nred;
    for (i = 0; i < hull->numVertices; i++) {
        v3 vtx = f4v(sh->verts[hull->vertexOffset + i]);
        float curDot = dot(vtx, planeNormalInConvex);
        if (curDot > maxDot) {
            maxDot = curDot;
            if (numPoints == 64) numPoints--;
        }
        if (numPoints < 64) {
            v3 vtxWorld = add(mmul(&RB, vtx), posB);
            v3 vtxInPlane = xform_inv(&RA, posA, vtxWorld);
            float dist = dot(planeNormal, vtxInPlane) - planeConstant;
            if (dist < 0.f) {
                pts[numPoints].x = vtxWorld.x; pts[numPoints].y = vtxWorld.y; pts[numPoints].z = vtxWorld.z;
                pts[numPoints].w = dist;
                numPoints++;
            }
        }
    }
    nred = reduce_contacts(pts, numPoints, planeNormalInConvex, idx);
    if (nred > 0) {
        write_header(c, bodies, A, B, neg(planeNormalWorld), nred, fr);
        for (i = 0; i < nred; i++) {
            p4 q = pts[idx[i]];
            c->worldPosB[i].x = q.x; c->worldPosB[i].y = q.y; c->worldPosB[i].z = q.z; c->worldPosB[i].w = q.w;
        }
        return 1;
    }
    return 0;
}

/* computeContactPlaneSphere (Bullet3OpenCL/NarrowphaseCollision/kernels/primitiveContacts.cl:729-790);
 * A = plane, B = sphere.  The .cl has no CPU twin; this is the restatement. */
static int plane_sphere(const obody* bodies, const oshapes* sh, int A, int B, ocontact* c, unsigned short fr) {
    const obody* BA = &bodies[A];
    const obody* BB = &bodies[B];
    of4 pe = sh->faces[sh->cols[BA->collidableIdx].shapeIndex].plane;
    float radius = sh->cols[BB->collidableIdx].radius;
    v3 posA = f4v(BA->pos), posB = f4v(BB->pos);
    v3 n = mk(pe.x, pe.y, pe.z);
    float planeConstant = pe.w, distance;
    m3 RA = qmat(f4q(BA->quat)), RB = qmat(f4q(BB->quat));
    v3 vtx1 = scl(mtmul(&RB, mmul(&RA, neg(n))), radius);
    v3 vtxInPlane = mtmul(&RA, sub(add(mmul(&RB, vtx1), posB), posA));
    distance = dot(n, vtxInPlane) - planeConstant;
    if (distance < 0.f) {
        v3 projected = sub(vtxInPlane, lscl(distance, n));
        v3 world = add(mmul(&RA, projected), posA);
        v3 nB = mmul(&RA, n);
        v3 pOnB = add(world, scl(nB, distance));
        write_header(c, bodies, A, B, neg(nB), 1, fr);
        c->worldPosB[0].x = pOnB.x; c->worldPosB[0].y = pOnB.y; c->worldPosB[0].z = pOnB.z; c->worldPosB[0].w = distance;
        return 1;
    }
    return 0;
}

/* IsPointInPolygon (b3ConvexHullContact.cpp:362-411) */
static int point_in_polygon(v3 p, const oface* face, const of4* base, const int* indices, v3* out) {
    v3 plane = mk(face->plane.x, face->plane.y, face->plane.z), a, b;
    int i;
    if (face->numIndices < 2) return 0;
    b = f4v(base[indices[face->indexOffset + face->numIndices - 1]]);
    for (i = 0; i < face->numIndices; i++) {
        v3 ab, ap, v;
        a = b;
        b = f4v(base[indices[face->indexOffset + i]]);
        ab = sub(b, a);
        ap = sub(p, a);
        v = cross(ab, plane);
        if (dot(ap, v) > 0.f) {
            float ab_m2 = dot(ab, ab);
            float rt = ab_m2 != 0.f ? dot(ab, ap) / ab_m2 : 0.f;
            if (rt <= 0.f) *out = a;
            else if (rt >= 1.f) *out = b;
            else {
                float s = 1.f - rt;
                *out = mk(s * a.x + rt * b.x, s * a.y + rt * b.y, s * a.z + rt * b.z);
            }
            return 0;
        }
    }
    return 1;
}

/* computeContactSphereConvex (b3ConvexHullContact.cpp:2323-2470); A = sphere, B = hull */
static int sphere_hull(const obody* bodies, const oshapes* sh, int A, int B, ocontact* c, unsigned short fr) {
    const obody* BA = &bodies[A];
    const obody* BB = &bodies[B];
    float radius = sh->cols[BA->collidableIdx].radius, minDist = -1000000.f;
    v3 pos = f4v(BB->pos);
    m3 R = qmat(f4q(BB->quat));
    v3 spherePos = xform_inv(&R, pos, f4v(BA->pos));
    const ohull* hull = &sh->hulls[sh->cols[BB->collidableIdx].shapeIndex];
    v3 closest = mk(0, 0, 0), localHitNormal = mk(0, 0, 0);
    int bCollide = 1, f;
    const of4* base = &sh->verts[hull->vertexOffset];
    for (f = 0; f < hull->numFaces; f++) {
        const oface* face = &sh->faces[hull->faceOffset + f];
        v3 n = mk(face->plane.x, face->plane.y, face->plane.z);
        float dist = dot(n, spherePos) + face->plane.w;
        v3 pntReturn = sub(spherePos, lscl(dist, n));
        if (dist > radius) { bCollide = 0; break; }
        if (dist > 0.f) {
            v3 out = mk(0.f, 0.f, 0.f);
            if (point_in_polygon(spherePos, face, base, sh->indices, &out)) {
                if (dist > minDist) { minDist = dist; closest = pntReturn; localHitNormal = n; }
            } else {
                v3 tmp = sub(spherePos, out);
                float l2 = dot(tmp, tmp);
                if (l2 < radius * radius) {
                    dist = sqrtf(l2);
                    if (dist > minDist) {
                        minDist = dist;
                        closest = out;
                        float inv = 1.0f / dist; /* b3Vector3 operator/ scales by the reciprocal */
                        localHitNormal = mk(tmp.x * inv, tmp.y * inv, tmp.z * inv);
                    }
                } else { bCollide = 0; break; }
            }
        } else {
            if (dist > minDist) { minDist = dist; closest = pntReturn; localHitNormal = n; }
        }
    }
    if (bCollide && minDist > -10000.f) {
        v3 nB = mmul(&R, localHitNormal);
        v3 pOnB = add(mmul(&R, closest), pos);
        float actualDepth = minDist - radius;
        if (actualDepth < 0.f) {
            write_header(c, bodies, A, B, nB, 1, fr);
            c->worldPosB[0].x = pOnB.x; c->worldPosB[0].y = pOnB.y; c->worldPosB[0].z = pOnB.z;
            c->worldPosB[0].w = actualDepth;
            return 1;
        }
    }
    return 0;
}

/* sphere-sphere branch of primitiveContactsKernel (primitiveContacts.cl:926-972) */
static int sphere_sphere(const obody* bodies, const oshapes* sh, int A, int B, ocontact* c, unsigned short fr) {
    float rA = sh->cols[bodies[A].collidableIdx].radius, rB = sh->cols[bodies[B].collidableIdx].radius;
    v3 diff = sub(f4v(bodies[A].pos), f4v(bodies[B].pos));
    float len = sqrtf(dot(diff, diff));
    if (len <= (rA + rB)) {
        float dist = len - (rA + rB);
        v3 n = mk(1.f, 0.f, 0.f), cp;
        if (len > 0.00001f) n = mk(diff.x / len, diff.y / len, diff.z / len);
        cp = add(f4v(bodies[B].pos), scl(n, rB));
        write_header(c, bodies, A, B, n, 1, fr);
        c->worldPosB[0].x = cp.x; c->worldPosB[0].y = cp.y; c->worldPosB[0].z = cp.z; c->worldPosB[0].w = dist;
        return 1;
    }
    return 0;
}

/* b3ProjectAxis (Bullet3Collision/NarrowPhaseCollision/shared/b3FindSeparatingAxis.h:4-33) */
static void project(const of4* verts, int nv, v3 pos, qt orn, v3 dir, float* mn, float* mx) {
    v3 localDir = qrotq(qconj(orn), dir);
    float offset = dot(pos, dir);
    int i;
    *mn = FLT_MAX;
    *mx = -FLT_MAX;
    for (i = 0; i < nv; i++) {
        float dp = dot(f4v(verts[i]), localDir);
        if (dp < *mn) *mn = dp;
        if (dp > *mx) *mx = dp;
    }
    if (*mn > *mx) { float t = *mn; *mn = *mx; *mx = t; }
    *mn = *mn + offset;
    *mx = *mx + offset;
}

/* b3TestSepAxis (b3FindSeparatingAxis.h:35-53) */
static int test_sep_axis(const ohull* hA, const ohull* hB, v3 posA, qt qA, v3 posB, qt qB, v3 axis,
                         const of4* verts, float* depth) {
    float min0, max0, min1, max1, d0, d1;
    project(&verts[hA->vertexOffset], hA->numVertices, posA, qA, axis, &min0, &max0);
    project(&verts[hB->vertexOffset], hB->numVertices, posB, qB, axis, &min1, &max1);
    if (max0 < min1 || max1 < min0) return 0;
    d0 = max0 - min1;
    d1 = max1 - min0;
    *depth = d0 < d1 ? d0 : d1;
    return 1;
}

/* b3FindSeparatingAxis (b3FindSeparatingAxis.h:55-195): face normals of A, of B, exact edge-edge;
 * rotations by b3QuatRotate, centres by b3TransformPoint (matrix form) */
static int find_separating_axis(const ohull* hA, const ohull* hB, v3 posA, qt qA, v3 posB, qt qB,
                                const oshapes* sh, v3* sep) {
    m3 RA = qmat(qA), RB = qmat(qB);
    v3 c0 = add(mmul(&RA, f4v(hA->localCenter)), posA);
    v3 c1 = add(mmul(&RB, f4v(hB->localCenter)), posB);
    v3 deltaC2 = sub(c0, c1);
    float dmin = FLT_MAX, d;
    int i, e0, e1;
    for (i = 0; i < hA->numFaces; i++) {
        v3 n = qrotq(qA, f4v(sh->faces[hA->faceOffset + i].plane));
        if (dot(deltaC2, n) < 0.f) n = neg(n);
        if (!test_sep_axis(hA, hB, posA, qA, posB, qB, n, sh->verts, &d)) return 0;
        if (d < dmin) { dmin = d; *sep = n; }
    }
    for (i = 0; i < hB->numFaces; i++) {
        v3 n = qrotq(qB, f4v(sh->faces[hB->faceOffset + i].plane));
        if (dot(deltaC2, n) < 0.f) n = neg(n);
        if (!test_sep_axis(hA, hB, posA, qA, posB, qB, n, sh->verts, &d)) return 0;
        if (d < dmin) { dmin = d; *sep = n; }
    }
    for (e0 = 0; e0 < hA->numUniqueEdges; e0++) {
        v3 w0 = qrotq(qA, f4v(sh->edges[hA->uniqueEdgesOffset + e0]));
        for (e1 = 0; e1 < hB->numUniqueEdges; e1++) {
            v3 w1 = qrotq(qB, f4v(sh->edges[hB->uniqueEdgesOffset + e1]));
            v3 cr = cross(w0, w1);
            /* b3IsAlmostZero compares against the double constant 1e-6 */
            if ((double)fabsf(cr.x) > 1e-6 || (double)fabsf(cr.y) > 1e-6 || (double)fabsf(cr.z) > 1e-6) {
                cr = nrm(cr);
                if (dot(deltaC2, cr) < 0.f) cr = neg(cr);
                if (!test_sep_axis(hA, hB, posA, qA, posB, qB, cr, sh->verts, &d)) return 0;
                if (d < dmin) { dmin = d; *sep = cr; }
            }
        }
    }
    if (dmin == FLT_MAX) return 0;
    if (dot(neg(deltaC2), *sep) > 0.0f) *sep = neg(*sep);
    return 1;
}

#define CLIP_CAP 64
/* b3ClipFace (b3ContactConvexConvexSAT.h:20-63) */
static int clip_face(const p4* in, int nin, v3 n, float eq, p4* out) {
    int nout = 0, ve;
    p4 first;
    float ds;
    if (nin < 2) return 0;
    first = in[nin - 1];
    ds = dot(n, mk(first.x, first.y, first.z)) + eq;
    for (ve = 0; ve < nin; ve++) {
        p4 end = in[ve];
        float de = dot(n, mk(end.x, end.y, end.z)) + eq;
        if (ds < 0.f) {
            if (de < 0.f) {
                if (nout < CLIP_CAP) out[nout++] = end;
            } else {
                float t = ds * 1.f / (ds - de);
                p4 l = {first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                        first.z + (end.z - first.z) * t, 0.f};
                if (nout < CLIP_CAP) out[nout++] = l;
            }
        } else {
            if (de < 0.f) {
                float t = ds * 1.f / (ds - de);
                p4 l = {first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                        first.z + (end.z - first.z) * t, 0.f};
                if (nout < CLIP_CAP) out[nout++] = l;
                if (nout < CLIP_CAP) out[nout++] = end;
            }
        }
        first = end;
        ds = de;
    }
    return nout;
}

/* b3ContactConvexConvexSAT (b3ContactConvexConvexSAT.h:403-486) -> b3ClipHullHullSingle (:262-401)
 * -> b3ClipHullAgainstHull (:169-260) -> b3ClipFaceAgainstHull (:65-167), minDist -1, maxDist 0 */
static int hull_hull(const obody* bodies, const oshapes* sh, int A, int B, ocontact* c, unsigned short fr) {
    const obody* BA = &bodies[A];
    const obody* BB = &bodies[B];
    const ohull* hA = &sh->hulls[sh->cols[BA->collidableIdx].shapeIndex];
    const ohull* hB = &sh->hulls[sh->cols[BB->collidableIdx].shapeIndex];
    v3 posA = f4v(BA->pos), posB = f4v(BB->pos), sep, planeNormalA, worldPlaneAnormal1;
    qt qA = f4q(BA->quat), qB = f4q(BB->quat), cA, cB;
    m3 RA = qmat(qA), RB = qmat(qB), CA, CB;
    p4 buf0[CLIP_CAP], buf1[CLIP_CAP];
    p4 *pin = buf0, *pout = buf1;
    int fb = -1, fa = -1, f, nin = 0, e, e0, nva, ncont = 0, i;
    float dmax = -FLT_MAX, dmn = FLT_MAX, planeEqWS;
    const of4* vA = &sh->verts[hA->vertexOffset];
    const of4* vB = &sh->verts[hB->vertexOffset];
    const oface *polyA, *polyB;
    if (!find_separating_axis(hA, hB, posA, qA, posB, qB, sh, &sep)) return 0;
    /* b3ClipHullHullSingle clips with the orientation round-tripped through a b3Transform
     * (setRotation then getRotation, b3ContactConvexConvexSAT.h:315-330) */
    cA = quat_from_mat(&RA);
    cB = quat_from_mat(&RB);
    CA = qmat(cA);
    CB = qmat(cB);
    for (f = 0; f < hB->numFaces; f++) {
        float d = dot(qrotq(cB, f4v(sh->faces[hB->faceOffset + f].plane)), sep);
        if (d > dmax) { dmax = d; fb = f; }
    }
    for (f = 0; f < hA->numFaces; f++) {
        float d = dot(qrotq(cA, f4v(sh->faces[hA->faceOffset + f].plane)), sep);
        if (d < dmn) { dmn = d; fa = f; }
    }
    if (fb < 0 || fa < 0) return 0;
    polyB = &sh->faces[hB->faceOffset + fb];
    for (e = 0; e < polyB->numIndices && e < CLIP_CAP; e++) {
        v3 w = add(mmul(&CB, f4v(vB[sh->indices[polyB->indexOffset + e]])), posB);
        pin[nin].x = w.x; pin[nin].y = w.y; pin[nin].z = w.z; pin[nin].w = 0.f;
        nin++;
    }
    polyA = &sh->faces[hA->faceOffset + fa];
    planeNormalA = mk(polyA->plane.x, polyA->plane.y, polyA->plane.z);
    worldPlaneAnormal1 = qrotq(cA, planeNormalA);
    nva = polyA->numIndices;
    for (e0 = 0; e0 < nva; e0++) {
        v3 va = f4v(vA[sh->indices[polyA->indexOffset + e0]]);
        v3 vb = f4v(vA[sh->indices[polyA->indexOffset + ((e0 + 1) % nva)]]);
        v3 worldEdge0 = qrotq(cA, sub(va, vb));
        v3 planeNormalWS1 = neg(cross(worldEdge0, worldPlaneAnormal1));
        v3 worldA1 = add(mmul(&CA, va), posA);
        float planeEqWS1 = -dot(worldA1, planeNormalWS1);
        int nout = clip_face(pin, nin, planeNormalWS1, planeEqWS1, pout);
        p4* tmp = pout; pout = pin; pin = tmp;
        nin = nout;
    }
    planeEqWS = polyA->plane.w - dot(worldPlaneAnormal1, posA);
    for (i = 0; i < nin; i++) {
        float depth = dot(worldPlaneAnormal1, mk(pin[i].x, pin[i].y, pin[i].z)) + planeEqWS;
        if (depth <= -1.0f) depth = -1.0f;
        if (depth <= 0.0f) {
            pout[ncont].x = pin[i].x; pout[ncont].y = pin[i].y; pout[ncont].z = pin[i].z; pout[ncont].w = depth;
            ncont++;
        }
    }
    if (ncont > 0) {
        int idx[4], np = reduce_contacts(pout, ncont, sep, idx), q;
        write_header(c, bodies, A, B, sep, np, fr);
        for (q = 0; q < np; q++) {
            p4 v = pout[idx[q]];
            c->worldPosB[q].x = v.x; c->worldPosB[q].y = v.y; c->worldPosB[q].z = v.z; c->worldPosB[q].w = v.w;
        }
        return 1;
    }
    return 0;
}

static int pair_contact(const obody* bodies, const oshapes* sh, int A, int B, ocontact* c, unsigned short fr) {
    int ta = sh->cols[bodies[A].collidableIdx].shapeType, tb = sh->cols[bodies[B].collidableIdx].shapeType;
    memset(c, 0, sizeof(*c));
    /* dispatch as in computeConvexConvexContactsGPUSAT (b3ConvexHullContact.cpp:2655-2735) */
    if (ta == SHAPE_CONVEX_HULL && tb == SHAPE_CONVEX_HULL) return hull_hull(bodies, sh, A, B, c, fr);
    if (ta == SHAPE_PLANE && tb == SHAPE_CONVEX_HULL) return plane_hull(bodies, sh, A, B, c, fr);
    if (tb == SHAPE_PLANE && ta == SHAPE_CONVEX_HULL) return plane_hull(bodies, sh, B, A, c, fr);
    if (ta == SHAPE_SPHERE && tb == SHAPE_CONVEX_HULL) return sphere_hull(bodies, sh, A, B, c, fr);
    if (tb == SHAPE_SPHERE && ta == SHAPE_CONVEX_HULL) return sphere_hull(bodies, sh, B, A, c, fr);
    if (ta == SHAPE_SPHERE && tb == SHAPE_SPHERE) return sphere_sphere(bodies, sh, A, B, c, fr);
    if (ta == SHAPE_PLANE && tb == SHAPE_SPHERE) return plane_sphere(bodies, sh, A, B, c, fr);
    if (tb == SHAPE_PLANE && ta == SHAPE_SPHERE) return plane_sphere(bodies, sh, B, A, c, fr);
    return 0;
}

int oracle_contacts(const obody* bodies, const oshapes* sh, opair* pairs, int npairs, ocontact* out, int cap,
                    unsigned short friction_cmp) {
    ocontact* tmp = (ocontact*)malloc(sizeof(ocontact) * (size_t)(npairs > 0 ? npairs : 1));
    char* has = (char*)malloc((size_t)(npairs > 0 ? npairs : 1));
    int p, n = 0;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 256)
    for (p = 0; p < npairs; p++) has[p] = (char)pair_contact(bodies, sh, pairs[p].x, pairs[p].y, &tmp[p], friction_cmp);
    for (p = 0; p < npairs; p++) {
        if (has[p]) {
            if (n < cap) out[n] = tmp[p];
            pairs[p].z = n;
            n++;
        } else {
            pairs[p].z = -1;
        }
    }
    free(tmp);
    free(has);
    return n;
}

/* ------------------------------------------------------------------ compound shapes
 * A compound (SHAPE_COMPOUND_OF_CONVEX_HULLS) lists child convex hulls with local poses.  Its
 * pairs expand to child pairs in the order (pair, child of A, child of B) -- the set of
 * findCompoundPairsKernel (b3ConvexHullContact.cpp:1419-1775): compound-compound child pairs whose
 * world AABBs overlap (the reference walks quantized child BVHs, whose conservative boxes add only
 * child pairs that cannot touch), compound-hull every child against the hull, plane-compound
 * every child against the plane.  Each child pair yields at most one manifold. */

/* child pose: newPos = b3QuatRotate(orn, childPos) + pos, newOrn = b3QuatMul(orn, childOrn)
 * (processCompoundPairsKernel, b3ConvexHullContact.cpp:1813-1829) */
static void child_pose(const obody* b, const ochild* ch, v3* pos, qt* orn) {
    qt q = f4q(b->quat);
    *pos = add(qrotq(q, f4v(ch->pos)), f4v(b->pos));
    *orn = qmul(q, f4q(ch->orn));
}

static int is_compound(const oshapes* sh, const obody* b) {
    return sh->cols[b->collidableIdx].shapeType == SHAPE_COMPOUND_OF_CONVEX_HULLS;
}

/* registerCompoundShape's local AABB (b3GpuNarrowPhase.cpp:391-431): the union (b3Vector3 setMin /
 * setMax) of the children's local AABBs moved by b3TransformAabb with margin 0 into the compound's
 * frame (the same arithmetic as b3TransformAabb2 of a quaternion pose) */
void oracle_compound_local_aabb(const oaabb* child_local, const ochild* children, int n, oaabb* out) {
    v3 mn = mk(1e30f, 1e30f, 1e30f), mx = mk(-1e30f, -1e30f, -1e30f);
    int i;
    for (i = 0; i < n; i++) {
        v3 a, b;
        transform_aabb(&child_local[i], f4v(children[i].pos), f4q(children[i].orn), 0.f, &a, &b);
        if (a.x < mn.x) mn.x = a.x;
        if (a.y < mn.y) mn.y = a.y;
        if (a.z < mn.z) mn.z = a.z;
        if (mx.x < b.x) mx.x = b.x;
        if (mx.y < b.y) mx.y = b.y;
        if (mx.z < b.z) mx.z = b.z;
    }
    out->minv[0] = mn.x; out->minv[1] = mn.y; out->minv[2] = mn.z; out->minw = 0;
    out->maxv[0] = mx.x; out->maxv[1] = mx.y; out->maxv[2] = mx.z; out->maxw = 0;
}

int oracle_compound_pairs(const obody* bodies, const oshapes* sh, const opair* pairs, int npairs, opair* out,
                          int cap) {
    int p, n = 0;
    for (p = 0; p < npairs; p++) {
        const int A = pairs[p].x, B = pairs[p].y;
        const ocollidable* cA = &sh->cols[bodies[A].collidableIdx];
        const ocollidable* cB = &sh->cols[bodies[B].collidableIdx];
        const int compA = cA->shapeType == SHAPE_COMPOUND_OF_CONVEX_HULLS;
        const int compB = cB->shapeType == SHAPE_COMPOUND_OF_CONVEX_HULLS;
        int a, b;
        if (!compA && !compB) continue;
        /* once the broadphase avoids static-static pairs this test goes (findCompoundPairsKernel :1446) */
        if (bodies[A].invMass == 0.f && bodies[B].invMass == 0.f) continue;
        if (compA && compB) {
            for (a = 0; a < cA->numChildShapes; a++) {
                const ochild* chA = &sh->children[cA->shapeIndex + a];
                oaabb la = sh->local_aabbs[chA->shapeIndex], wa;
                v3 pA, mnA, mxA;
                qt qA;
                child_pose(&bodies[A], chA, &pA, &qA);
                transform_aabb(&la, pA, qA, 0.f, &mnA, &mxA);
                wa.minv[0] = mnA.x; wa.minv[1] = mnA.y; wa.minv[2] = mnA.z;
                wa.maxv[0] = mxA.x; wa.maxv[1] = mxA.y; wa.maxv[2] = mxA.z;
                for (b = 0; b < cB->numChildShapes; b++) {
                    const ochild* chB = &sh->children[cB->shapeIndex + b];
                    oaabb lb = sh->local_aabbs[chB->shapeIndex], wb;
                    v3 pB, mnB, mxB;
                    qt qB;
                    child_pose(&bodies[B], chB, &pB, &qB);
                    transform_aabb(&lb, pB, qB, 0.f, &mnB, &mxB);
                    wb.minv[0] = mnB.x; wb.minv[1] = mnB.y; wb.minv[2] = mnB.z;
                    wb.maxv[0] = mxB.x; wb.maxv[1] = mxB.y; wb.maxv[2] = mxB.z;
                    if (!overlap(&wa, &wb)) continue;
                    if (n < cap) { out[n].x = A; out[n].y = B; out[n].z = cA->shapeIndex + a; out[n].w = cB->shapeIndex + b; }
                    n++;
                }
            }
        } else if (compA) {
            for (a = 0; a < cA->numChildShapes; a++) {
                if (n < cap) { out[n].x = A; out[n].y = B; out[n].z = cA->shapeIndex + a; out[n].w = -1; }
                n++;
            }
        } else {
            for (b = 0; b < cB->numChildShapes; b++) {
                if (n < cap) { out[n].x = A; out[n].y = B; out[n].z = -1; out[n].w = cB->shapeIndex + b; }
                n++;
            }
        }
    }
    return n;
}

/* findSeparatingAxisEdgeEdge (b3ConvexHullContact.cpp:702-785): every edge-edge axis projected
 * (no early exit, the separation test is discarded), the smallest overlap kept in *sep / *dmin */
static void edge_edge_axis(const ohull* hA, const ohull* hB, v3 posA, qt qA, v3 posB, qt qB, v3 deltaC2,
                           const oshapes* sh, v3* sep, float* dmin) {
    int e0, e1;
    for (e0 = 0; e0 < hA->numUniqueEdges; e0++) {
        v3 w0 = qrotq(qA, f4v(sh->edges[hA->uniqueEdgesOffset + e0]));
        for (e1 = 0; e1 < hB->numUniqueEdges; e1++) {
            v3 w1 = qrotq(qB, f4v(sh->edges[hB->uniqueEdgesOffset + e1]));
            v3 cr = cross(w0, w1);
            if ((double)fabsf(cr.x) > 1e-6 || (double)fabsf(cr.y) > 1e-6 || (double)fabsf(cr.z) > 1e-6) {
                float min0, max0, min1, max1, d0, d1, dist;
                cr = nrm(cr);
                if (dot(deltaC2, cr) < 0.f) cr = neg(cr);
                project(&sh->verts[hA->vertexOffset], hA->numVertices, posA, qA, cr, &min0, &max0);
                project(&sh->verts[hB->vertexOffset], hB->numVertices, posB, qB, cr, &min1, &max1);
                d0 = max0 - min1;
                d1 = max1 - min0;
                dist = d0 < d1 ? d0 : d1;
                if (dist < *dmin) { *dmin = dist; *sep = cr; }
            }
        }
    }
    if (dot(neg(deltaC2), *sep) > 0.0f) *sep = neg(*sep);
}

/* clipHullAgainstHull -> clipFaceAgainstHull -> clipFace (b3ConvexHullContact.cpp:939-1044,
 * :834-937, :787-832): incident face of B by max dot with the separating normal, reference face of
 * A by min, points behind A's side planes, depth clamped at minDist and kept if <= maxDist (at most
 * 64); rotations by b3QuatRotate of the poses themselves, points by b3Transform */
static int clip_hull_against_hull(v3 sep, const ohull* hA, const ohull* hB, v3 posA, qt qA, v3 posB, qt qB,
                                  float minDist, float maxDist, const oshapes* sh, p4* out) {
    m3 RA = qmat(qA), RB = qmat(qB);
    p4 buf0[CLIP_CAP], buf1[CLIP_CAP];
    p4 *pin = buf0, *pout = buf1;
    int fb = -1, fa = -1, f, nin = 0, e, e0, nva, n = 0, i;
    float dmax = -FLT_MAX, dmn = FLT_MAX, planeEqWS;
    v3 planeNormalWS;
    const oface *polyA, *polyB;
    for (f = 0; f < hB->numFaces; f++) {
        float d = dot(qrotq(qB, f4v(sh->faces[hB->faceOffset + f].plane)), sep);
        if (d > dmax) { dmax = d; fb = f; }
    }
    if (fb < 0) return 0;
    polyB = &sh->faces[hB->faceOffset + fb];
    for (e = 0; e < polyB->numIndices && e < CLIP_CAP; e++) {
        v3 w = add(mmul(&RB, f4v(sh->verts[hB->vertexOffset + sh->indices[polyB->indexOffset + e]])), posB);
        pin[nin].x = w.x; pin[nin].y = w.y; pin[nin].z = w.z; pin[nin].w = 0.f;
        nin++;
    }
    for (f = 0; f < hA->numFaces; f++) {
        float d = dot(qrotq(qA, f4v(sh->faces[hA->faceOffset + f].plane)), sep);
        if (d < dmn) { dmn = d; fa = f; }
    }
    if (fa < 0) return 0;
    polyA = &sh->faces[hA->faceOffset + fa];
    nva = polyA->numIndices;
    for (e0 = 0; e0 < nva; e0++) {
        v3 a = f4v(sh->verts[hA->vertexOffset + sh->indices[polyA->indexOffset + e0]]);
        v3 b = f4v(sh->verts[hA->vertexOffset + sh->indices[polyA->indexOffset + ((e0 + 1) % nva)]]);
        v3 worldEdge0 = qrotq(qA, sub(a, b));
        v3 worldPlaneAnormal1 = qrotq(qA, mk(polyA->plane.x, polyA->plane.y, polyA->plane.z));
        v3 planeNormalWS1 = neg(cross(worldEdge0, worldPlaneAnormal1));
        v3 worldA1 = add(mmul(&RA, a), posA);
        float planeEqWS1 = -dot(worldA1, planeNormalWS1);
        int nout = clip_face(pin, nin, planeNormalWS1, planeEqWS1, pout);
        p4* tmp = pout; pout = pin; pin = tmp;
        nin = nout;
    }
    planeNormalWS = qrotq(qA, mk(polyA->plane.x, polyA->plane.y, polyA->plane.z));
    planeEqWS = polyA->plane.w - dot(planeNormalWS, posA);
    for (i = 0; i < nin; i++) {
        float depth = dot(planeNormalWS, mk(pin[i].x, pin[i].y, pin[i].z)) + planeEqWS;
        if (depth <= minDist) depth = minDist;
        if (n < CLIP_CAP && depth <= maxDist) {
            out[n].x = pin[i].x; out[n].y = pin[i].y; out[n].z = pin[i].z; out[n].w = depth;
            n++;
        }
    }
    return n;
}

/* processCompoundPairsKernel + clipCompoundsHullHullKernel (b3ConvexHullContact.cpp:1777-2022)
 * for one child pair of hulls: the separating axis of findSeparatingAxis(A, B), then of
 * findSeparatingAxis(B, A) (which overwrites it), then the edge-edge pass from FLT_MAX; clipped
 * with minDist -1e30, maxDist 0, reduced by extractManifoldSequentialGlobal against -sep */
static int compound_hulls(const obody* bodies, const oshapes* sh, const opair* cp, int index, ocontact* c) {
    const obody* BA = &bodies[cp->x];
    const obody* BB = &bodies[cp->y];
    v3 posA = f4v(BA->pos), posB = f4v(BB->pos), sep = mk(1.f, 0.f, 0.f), deltaC2;
    qt qA = f4q(BA->quat), qB = f4q(BB->quat);
    int colA = BA->collidableIdx, colB = BB->collidableIdx, np, idx[4], q;
    const ohull *hA, *hB;
    m3 RA, RB;
    p4 pts[CLIP_CAP];
    float dmin = FLT_MAX;
    if (cp->z >= 0) { colA = sh->children[cp->z].shapeIndex; child_pose(BA, &sh->children[cp->z], &posA, &qA); }
    if (cp->w >= 0) { colB = sh->children[cp->w].shapeIndex; child_pose(BB, &sh->children[cp->w], &posB, &qB); }
    if (sh->cols[colA].shapeType != SHAPE_CONVEX_HULL || sh->cols[colB].shapeType != SHAPE_CONVEX_HULL) return 0;
    hA = &sh->hulls[sh->cols[colA].shapeIndex];
    hB = &sh->hulls[sh->cols[colB].shapeIndex];
    RA = qmat(qA);
    RB = qmat(qB);
    deltaC2 = sub(add(mmul(&RA, f4v(hA->localCenter)), posA), add(mmul(&RB, f4v(hB->localCenter)), posB));
    if (!find_separating_axis(hA, hB, posA, qA, posB, qB, sh, &sep)) return 0;
    if (!find_separating_axis(hB, hA, posB, qB, posA, qA, sh, &sep)) return 0;
    edge_edge_axis(hA, hB, posA, qA, posB, qB, deltaC2, sh, &sep, &dmin);
    np = clip_hull_against_hull(sep, hA, hB, posA, qA, posB, qB, -1e30f, 0.0f, sh, pts);
    if (np <= 0) return 0;
    np = reduce_contacts(pts, np, neg(sep), idx);
    write_header(c, bodies, cp->x, cp->y, sep, np, (unsigned short)(0.7f * 0xffff));
    c->batchIdx = index;
    c->childIndexA = cp->z;
    c->childIndexB = cp->w;
    for (q = 0; q < np; q++) {
        p4 v = pts[idx[q]];
        c->worldPosB[q].x = v.x; c->worldPosB[q].y = v.y; c->worldPosB[q].z = v.z; c->worldPosB[q].w = v.w;
    }
    return 1;
}

/* computeContactPlaneCompound (b3ConvexHullContact.cpp:2182-2321), one child: A = plane body, B =
 * compound body, child = child shape index; the plane-hull contact with the child's pose */
static int plane_child(const obody* bodies, const oshapes* sh, int A, int B, int child, int index, ocontact* c) {
    obody body = bodies[B];
    const ochild* ch = &sh->children[child];
    v3 pos;
    qt orn;
    int r;
    child_pose(&bodies[B], ch, &pos, &orn);
    body.pos.x = pos.x; body.pos.y = pos.y; body.pos.z = pos.z;
    body.quat.x = orn.x; body.quat.y = orn.y; body.quat.z = orn.z; body.quat.w = orn.w;
    body.collidableIdx = ch->shapeIndex;
    {
        /* plane_hull reads both bodies from one array: a two-body view with the child in B's place */
        obody two[2];
        two[0] = bodies[A];
        two[1] = body;
        r = plane_hull(two, sh, 0, 1, c, (unsigned short)(0.7f * 0xffff));
    }
    if (r) {
        c->bodyA = sgn_index(bodies, A);
        c->bodyB = sgn_index(bodies, B);
        c->batchIdx = index;
        c->childIndexA = -1;
        c->childIndexB = child;
    }
    return r;
}

int oracle_compound_contacts(const obody* bodies, const oshapes* sh, const opair* child_pairs, int n, ocontact* out,
                             int* out_index, int cap) {
    int i, m = 0;
    for (i = 0; i < n; i++) {
        const opair* cp = &child_pairs[i];
        ocontact c;
        int tA = cp->z >= 0 ? SHAPE_CONVEX_HULL : sh->cols[bodies[cp->x].collidableIdx].shapeType;
        int tB = cp->w >= 0 ? SHAPE_CONVEX_HULL : sh->cols[bodies[cp->y].collidableIdx].shapeType;
        int r = 0;
        memset(&c, 0, sizeof(c));
        if (tA == SHAPE_CONVEX_HULL && tB == SHAPE_CONVEX_HULL)
            r = compound_hulls(bodies, sh, cp, i, &c);
        else if (tA == SHAPE_PLANE && cp->w >= 0)
            r = plane_child(bodies, sh, cp->x, cp->y, cp->w, i, &c);
        else if (tB == SHAPE_PLANE && cp->z >= 0)
            r = plane_child(bodies, sh, cp->y, cp->x, cp->z, i, &c);
        if (r) {
            if (m < cap) { out[m] = c; if (out_index) out_index[m] = i; }
            m++;
        }
    }
    return m;
}

/* ------------------------------------------------------------------ concave meshes
 * A concave mesh (SHAPE_CONCAVE_TRIMESH) is a shape record whose faces are its triangles
 * (registerConcaveMeshShape, b3GpuNarrowPhase.cpp:615-667) with a quantized triangle BVH over its
 * local AABB widened by 1 (b3QuantizedBvh::setQuantizationValues, b3QuantizedBvh.cpp:79-88; its
 * collidable's numChildShapes is the BVH index).  A pair whose first body is the mesh and whose
 * second is a hull or a compound yields the triangles whose quantized leaf box overlaps the second
 * body's quantized world AABB (b3BvhTraversal, shared/b3BvhTraversal.h:11-111) -- any BVH over
 * those leaf boxes finds the same set -- with every child of a compound, in (pair, triangle,
 * child) order.  Each triangle-convex pair yields at most one manifold
 * (b3FindConcaveSeparatingAxisKernel, shared/b3FindConcaveSatAxis.h:506-797; b3FindClippingFaces
 * :421-504; clipFacesAndFindContactsKernel, shared/b3ClipFaces.h:67-177;
 * b3NewContactReductionKernel, shared/b3NewContactReduction.h:88-177).  The leaf boxes are taken
 * from the scaled vertices (the reference builds them from the unscaled ones: the same for a
 * scaling of 1). */
#define SHAPE_CONCAVE_TRIMESH 5

typedef struct { float mn[3], mx[3], q[3]; } obvhq;

static void mesh_bvhq(const oaabb* local, obvhq* b) {
    int k;
    for (k = 0; k < 3; k++) {
        b->mn[k] = local->minv[k] - 1.0f;
        b->mx[k] = local->maxv[k] + 1.0f;
        b->q[k] = 65533.0f / (b->mx[k] - b->mn[k]);
    }
}

/* b3QuantizedBvh::quantize (clamp = 0) and b3QuantizeWithClamp (clamp = 1) */
static void bvh_quantize(unsigned short out[3], const float p[3], int isMax, const obvhq* b, int clamp) {
    int k;
    for (k = 0; k < 3; k++) {
        float c = p[k], v;
        if (clamp) {
            if (c < b->mn[k]) c = b->mn[k];
            if (b->mx[k] < c) c = b->mx[k];
        }
        v = (c - b->mn[k]) * b->q[k];
        out[k] = isMax ? (unsigned short)(((unsigned short)(v + 1.f)) | 1) : (unsigned short)(((unsigned short)v) & 0xfffe);
    }
}

static const ohull* mesh_of(const oshapes* sh, const obody* b) { return &sh->hulls[sh->cols[b->collidableIdx].shapeIndex]; }

static v3 mesh_vertex(const oshapes* sh, const ohull* mesh, int t, int k) {
    const oface* f = &sh->faces[mesh->faceOffset + t];
    return f4v(sh->verts[mesh->vertexOffset + sh->indices[f->indexOffset + k]]);
}

/* the quantized leaf box of triangle t: its AABB widened to at least 0.002 per axis
 * (b3OptimizedBvh::build, QuantizedNodeTriangleCallback) */
static void tri_leaf(const oshapes* sh, const ohull* mesh, int t, const obvhq* b, unsigned short qmn[3],
                     unsigned short qmx[3]) {
    float lo[3] = {1e18f, 1e18f, 1e18f}, hi[3] = {-1e18f, -1e18f, -1e18f};
    int k, a;
    for (k = 0; k < 3; k++) {
        v3 p = mesh_vertex(sh, mesh, t, k);
        float c[3];
        c[0] = p.x; c[1] = p.y; c[2] = p.z;
        for (a = 0; a < 3; a++) {
            if (c[a] < lo[a]) lo[a] = c[a];
            if (hi[a] < c[a]) hi[a] = c[a];
        }
    }
    for (a = 0; a < 3; a++)
        if (hi[a] - lo[a] < 0.002f) {
            hi[a] = hi[a] + 0.001f;
            lo[a] = lo[a] - 0.001f;
        }
    bvh_quantize(qmn, lo, 0, b, 0);
    bvh_quantize(qmx, hi, 1, b, 0);
}

int oracle_concave_pairs(const obody* bodies, const oshapes* sh, const oaabb* aabbs, const opair* pairs, int npairs,
                         opair* out, int cap) {
    int p, n = 0;
    for (p = 0; p < npairs; p++) {
        int A = pairs[p].x, B = pairs[p].y, t, c, tB, nch;
        const ocollidable *cA, *cB;
        const ohull* mesh;
        obvhq bq;
        unsigned short qmn[3], qmx[3];
        if (bodies[A].invMass == 0.f && bodies[B].invMass == 0.f) continue;
        cA = &sh->cols[bodies[A].collidableIdx];
        cB = &sh->cols[bodies[B].collidableIdx];
        if (cA->shapeType != SHAPE_CONCAVE_TRIMESH) continue;
        tB = cB->shapeType;
        if (tB != SHAPE_CONVEX_HULL && tB != SHAPE_SPHERE && tB != SHAPE_COMPOUND_OF_CONVEX_HULLS) continue;
        nch = tB == SHAPE_COMPOUND_OF_CONVEX_HULLS ? cB->numChildShapes : 1;
        mesh = &sh->hulls[cA->shapeIndex];
        mesh_bvhq(&sh->local_aabbs[bodies[A].collidableIdx], &bq);
        bvh_quantize(qmn, aabbs[B].minv, 0, &bq, 1);
        bvh_quantize(qmx, aabbs[B].maxv, 1, &bq, 1);
        for (t = 0; t < mesh->numFaces; t++) {
            unsigned short lmn[3], lmx[3];
            tri_leaf(sh, mesh, t, &bq, lmn, lmx);
            /* b3TestQuantizedAabbAgainstQuantizedAabbSlow */
            if (qmn[0] > lmx[0] || qmx[0] < lmn[0] || qmn[1] > lmx[1] || qmx[1] < lmn[1] || qmn[2] > lmx[2] ||
                qmx[2] < lmn[2])
                continue;
            for (c = 0; c < nch; c++) {
                if (n < cap) {
                    out[n].x = A;
                    out[n].y = B;
                    out[n].z = t;
                    out[n].w = tB == SHAPE_COMPOUND_OF_CONVEX_HULLS ? cB->shapeIndex + c : 0;
                }
                n++;
            }
        }
    }
    return n;
}

/* clipFaceGlobal (shared/b3ClipFaces.h:20-61): no lower bound on the input polygon */
static int clip_face_global(const p4* in, int nin, v3 n, float eq, p4* out) {
    int nout = 0, ve;
    p4 first;
    float ds;
    if (nin < 1) return 0;
    first = in[nin - 1];
    ds = dot(n, mk(first.x, first.y, first.z)) + eq;
    for (ve = 0; ve < nin; ve++) {
        p4 end = in[ve];
        float de = dot(n, mk(end.x, end.y, end.z)) + eq;
        if (ds < 0.f) {
            if (de < 0.f) {
                if (nout < CLIP_CAP) out[nout++] = end;
            } else {
                float t = ds * 1.f / (ds - de);
                p4 l = {first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                        first.z + (end.z - first.z) * t, 0.f};
                if (nout < CLIP_CAP) out[nout++] = l;
            }
        } else if (de < 0.f) {
            float t = ds * 1.f / (ds - de);
            p4 l = {first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t, first.z + (end.z - first.z) * t,
                    0.f};
            if (nout < CLIP_CAP) out[nout++] = l;
            if (nout < CLIP_CAP) out[nout++] = end;
        }
        first = end;
        ds = de;
    }
    return nout;
}

/* b3Project over the triangle's 3 local vertices */
static void project_tri(const v3* tv, v3 pos, qt orn, v3 dir, float* mn, float* mx) {
    v3 localDir = qrotq(qconj(orn), dir);
    float offset = dot(pos, dir);
    int i;
    *mn = FLT_MAX;
    *mx = -FLT_MAX;
    for (i = 0; i < 3; i++) {
        float dp = dot(tv[i], localDir);
        if (dp < *mn) *mn = dp;
        if (dp > *mx) *mx = dp;
    }
    if (*mn > *mx) { float t = *mn; *mn = *mx; *mx = t; }
    *mn = *mn + offset;
    *mx = *mx + offset;
}

/* computeContactSphereTriangle (kernels/primitiveContacts.cl:1163-1302, run by
 * findConcaveSphereContactsKernel :1319-1370; GPU-only in the reference, so this restatement is
 * not pinned to reference output): the sphere centre in the mesh's frame; the triangle's plane
 * (normalised (v1 - v0) x (v2 - v0), turned towards the centre); a contact on the face when the
 * centre's projection is inside the triangle (pointInTriangle :1100-1133), else the nearest point
 * of an edge within the radius (segmentSqrDistance :1136-1160, the last such edge); normal from
 * the contact point to the centre; one point, at most the radius deep.  The sphere is body A of
 * the manifold, the mesh body B, childIndexB the triangle. */
static int point_in_triangle(const v3* tv, v3 n, v3 p) {
    v3 e1 = sub(tv[1], tv[0]), e2 = sub(tv[2], tv[1]), e3 = sub(tv[0], tv[2]);
    float r1 = dot(cross(e1, n), sub(p, tv[0]));
    float r2 = dot(cross(e2, n), sub(p, tv[1]));
    float r3 = dot(cross(e3, n), sub(p, tv[2]));
    if (r1 > 0.f && r2 > 0.f && r3 > 0.f) return 1;
    if (r1 <= 0.f && r2 <= 0.f && r3 <= 0.f) return 1;
    return 0;
}

static float segment_sqr_distance(v3 from, v3 to, v3 p, v3* nearest) {
    v3 diff = sub(p, from), v = sub(to, from);
    float t = dot(v, diff);
    if (t > 0.f) {
        float dotVV = dot(v, v);
        if (t < dotVV) {
            t = t / dotVV;
            diff = sub(diff, lscl(t, v));
        } else {
            t = 1.f;
            diff = sub(diff, v);
        }
    } else {
        t = 0.f;
    }
    *nearest = add(from, lscl(t, v));
    return dot(diff, diff);
}

static int concave_sphere(const obody* bodies, const oshapes* sh, const opair* cp, int index, ocontact* c) {
    const obody* BM = &bodies[cp->x];
    const obody* BS = &bodies[cp->y];
    const ohull* mesh = mesh_of(sh, BM);
    const float radius = sh->cols[BS->collidableIdx].radius;
    v3 tv[3], pos = f4v(BM->pos), centre, normal, hit, cpt = mk(0.f, 0.f, 0.f);
    qt q = f4q(BM->quat), qi = qconj(f4q(BM->quat));
    float dist;
    int i, has = 0;
    for (i = 0; i < 3; i++) tv[i] = mesh_vertex(sh, mesh, cp->z, i);
    centre = add(qrotq(qi, f4v(BS->pos)), qrotq(qi, neg(pos)));
    normal = nrm(cross(sub(tv[1], tv[0]), sub(tv[2], tv[0])));
    dist = dot(sub(centre, tv[0]), normal);
    if (dist < 0.f) { dist = dist * -1.f; normal = scl(normal, -1.f); }
    hit = normal;
    if (dist < radius) {
        if (point_in_triangle(tv, normal, centre)) {
            has = 1;
            cpt = sub(centre, scl(normal, dist));
        } else {
            float r2 = radius * radius;
            for (i = 0; i < 3; i++) {
                v3 nearest;
                float d2 = segment_sqr_distance(tv[i], tv[(i + 1) % 3], centre, &nearest);
                if (d2 < r2) { has = 1; cpt = nearest; }
            }
        }
    }
    if (has) {
        v3 toc = sub(centre, cpt);
        float md = sqrtf(dot(toc, toc));
        if (md > FLT_EPSILON) {
            v3 n1, pB;
            float depth = md - radius;
            hit = nrm(toc);
            n1 = qrotq(q, neg(hit));
            pB = add(qrotq(q, cpt), pos);
            if (depth <= 0.f && dot(n1, n1) > FLT_EPSILON) {
                write_header(c, bodies, cp->y, cp->x, neg(n1), 1, (unsigned short)(0.7f * 0xffff));
                c->batchIdx = index;
                c->childIndexB = cp->z;
                c->worldPosB[0].x = pB.x; c->worldPosB[0].y = pB.y; c->worldPosB[0].z = pB.z; c->worldPosB[0].w = depth;
                return 1;
            }
        }
    }
    return 0;
}

/* one triangle-convex pair: the triangle as a five-face prism (front, back, three edge planes),
 * the SAT over its faces, the hull's faces and the edge pairs with one running minimum, then the
 * clipping faces, the clip (minDist -1e30, maxDist 0.02) and the reduction */
static int concave_tri(const obody* bodies, const oshapes* sh, const oaabb* aabbs, const opair* cp, int index,
                       ocontact* c) {
    const obody* BA = &bodies[cp->x];
    const obody* BB = &bodies[cp->y];
    const ohull* mesh = mesh_of(sh, BA);
    const oface* face = &sh->faces[mesh->faceOffset + cp->z];
    v3 tv[3], fn[5], te[3], lc = mk(0.f, 0.f, 0.f), normal, posA, posB, c0, c1, D, sep = mk(1.f, 2.f, 3.f);
    qt qA, qB;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f}, dmin = FLT_MAX, d, min0, max0, min1, max1;
    int i, k, prev, colB = BB->collidableIdx, e0, e1, f, fb, fa, na, ia[3], nin, np, idx[4];
    const ohull* hB;
    v3 nA = mk(0.f, 0.f, 0.f), wA[3];
    m3 RA, RB;
    p4 buf0[CLIP_CAP], buf1[CLIP_CAP], *pin, *pout;
    float dmax;
    int tB = sh->cols[colB].shapeType;
    if (tB != SHAPE_CONVEX_HULL && tB != SHAPE_COMPOUND_OF_CONVEX_HULLS) return 0;
    for (i = 0; i < 3; i++) {
        float q3[3];
        tv[i] = mesh_vertex(sh, mesh, cp->z, i);
        lc = add(lc, tv[i]);
        q3[0] = tv[i].x; q3[1] = tv[i].y; q3[2] = tv[i].z;
        for (k = 0; k < 3; k++) {
            if (q3[k] < lo[k]) lo[k] = q3[k];
            if (hi[k] < q3[k]) hi[k] = q3[k];
        }
    }
    for (k = 0; k < 3; k++)
        if (lo[k] > aabbs[cp->y].maxv[k] || hi[k] < aabbs[cp->y].minv[k]) return 0;
    te[0] = sub(tv[1], tv[0]);
    te[1] = sub(tv[2], tv[1]);
    te[2] = sub(tv[0], tv[2]);
    normal = f4v(face->plane);
    fn[0] = normal;
    fn[1] = neg(normal);
    prev = 2;
    for (i = 0; i < 3; i++) {
        fn[2 + i] = nrm(cross(normal, sub(tv[prev], tv[i])));
        prev = i;
    }
    lc = scl(lc, 1.f / 3.f);
    posA = f4v(BA->pos);
    qA = f4q(BA->quat);
    posB = f4v(BB->pos);
    qB = f4q(BB->quat);
    /* b3TransformPoint of the host code is b3Transform's: the rotation matrix of the quaternion
     * (b3Quat.h's C++ branch), for the child pose, the centres and the clipping faces' vertices */
    if (tB == SHAPE_COMPOUND_OF_CONVEX_HULLS) {
        const ochild* ch = &sh->children[cp->w];
        m3 RB0 = qmat(qB);
        colB = ch->shapeIndex;
        posB = add(mmul(&RB0, f4v(ch->pos)), posB);
        qB = qmul(qB, f4q(ch->orn));
    }
    hB = &sh->hulls[sh->cols[colB].shapeIndex];
    RA = qmat(qA);
    RB = qmat(qB);
    c0 = add(mmul(&RA, lc), posA);
    c1 = add(mmul(&RB, f4v(hB->localCenter)), posB);
    D = sub(c0, c1);
    /* the prism's faces */
    for (f = 0; f < 5; f++) {
        v3 n = qrotq(qA, fn[f]);
        if (dot(D, n) < 0.f) n = neg(n);
        project_tri(tv, posA, qA, n, &min0, &max0);
        project(&sh->verts[hB->vertexOffset], hB->numVertices, posB, qB, n, &min1, &max1);
        if (max0 < min1 || max1 < min0) return 0;
        d = (max0 - min1) < (max1 - min0) ? (max0 - min1) : (max1 - min0);
        if (d < dmin) { dmin = d; sep = n; }
    }
    if (dot(neg(D), sep) > 0.0f) sep = neg(sep);
    /* the hull's faces (the hull projected first) */
    for (f = 0; f < hB->numFaces; f++) {
        v3 n = qrotq(qB, f4v(sh->faces[hB->faceOffset + f].plane));
        if (dot(D, n) < 0.f) n = neg(n);
        project(&sh->verts[hB->vertexOffset], hB->numVertices, posB, qB, n, &min0, &max0);
        project_tri(tv, posA, qA, n, &min1, &max1);
        if (max0 < min1 || max1 < min0) return 0;
        d = (max0 - min1) < (max1 - min0) ? (max0 - min1) : (max1 - min0);
        if (d < dmin) { dmin = d; sep = n; }
    }
    if (dot(neg(D), sep) > 0.0f) sep = neg(sep);
    /* the edge pairs */
    for (e0 = 0; e0 < 3; e0++) {
        v3 w0 = qrotq(qA, te[e0]);
        for (e1 = 0; e1 < hB->numUniqueEdges; e1++) {
            v3 w1 = qrotq(qB, f4v(sh->edges[hB->uniqueEdgesOffset + e1]));
            v3 cr = cross(w0, w1);
            if ((double)fabsf(cr.x) > 1e-6 || (double)fabsf(cr.y) > 1e-6 || (double)fabsf(cr.z) > 1e-6) {
                cr = nrm(cr);
                if (dot(D, cr) < 0.f) cr = neg(cr);
                project_tri(tv, posA, qA, cr, &min0, &max0);
                project(&sh->verts[hB->vertexOffset], hB->numVertices, posB, qB, cr, &min1, &max1);
                if (max0 < min1 || max1 < min0) return 0;
                d = (max0 - min1) < (max1 - min0) ? (max0 - min1) : (max1 - min0);
                if (d < dmin) { dmin = d; sep = cr; }
            }
        }
    }
    if (dot(neg(D), sep) > 0.0f) sep = neg(sep);
    /* b3FindClippingFaces */
    fb = -1;
    dmax = -FLT_MAX;
    for (f = 0; f < hB->numFaces; f++) {
        float dd = dot(qrotq(qB, f4v(sh->faces[hB->faceOffset + f].plane)), sep);
        if (dd > dmax) { dmax = dd; fb = f; }
    }
    if (fb < 0) return 0;
    fa = -1;
    {
        float dmn = FLT_MAX;
        for (f = 0; f < 5; f++) {
            v3 wn = qrotq(qA, fn[f]);
            float dd = dot(wn, sep);
            if (dd < dmn) { dmn = dd; fa = f; nA = wn; }
        }
    }
    if (fa < 0) return 0;
    if (fa == 0) { ia[0] = 0; ia[1] = 1; ia[2] = 2; na = 3; }
    else if (fa == 1) { ia[0] = 2; ia[1] = 1; ia[2] = 0; na = 3; }
    else { i = fa - 2; ia[0] = i; ia[1] = i == 0 ? 2 : i - 1; na = 2; }
    for (i = 0; i < na; i++) wA[i] = add(mmul(&RA, tv[ia[i]]), posA);
    {
        const oface* polyB = &sh->faces[hB->faceOffset + fb];
        pin = buf0;
        pout = buf1;
        nin = 0;
        for (i = 0; i < polyB->numIndices && i < CLIP_CAP; i++) {
            v3 w = add(mmul(&RB, f4v(sh->verts[hB->vertexOffset + sh->indices[polyB->indexOffset + i]])), posB);
            p4 q = {w.x, w.y, w.z, 0.f};
            pin[nin++] = q;
        }
    }
    /* clipFacesAndFindContactsKernel */
    for (e0 = 0; e0 < na; e0++) {
        v3 aw = wA[e0], bw = wA[(e0 + 1) % na];
        v3 pn = neg(cross(sub(aw, bw), nA));
        float eq = -dot(aw, pn);
        int nout = clip_face_global(pin, nin, pn, eq, pout);
        p4* t = pout;
        pout = pin;
        pin = t;
        nin = nout;
    }
    {
        float eqA = -dot(nA, wA[0]);
        np = 0;
        for (i = 0; i < nin; i++) {
            float depth = dot(nA, mk(pin[i].x, pin[i].y, pin[i].z)) + eqA;
            if (depth <= -1e30f) depth = -1e30f;
            if (depth <= 0.02f) {
                p4 q = {pin[i].x, pin[i].y, pin[i].z, depth};
                pout[np++] = q;
            }
        }
    }
    if (np <= 0) return 0;
    /* b3NewContactReductionKernel */
    np = reduce_contacts(pout, np, neg(sep), idx);
    write_header(c, bodies, cp->x, cp->y, sep, np, (unsigned short)(0.7f * 0xffff));
    c->batchIdx = index;
    for (k = 0; k < np; k++) {
        p4 v = pout[idx[k]];
        c->worldPosB[k].x = v.x; c->worldPosB[k].y = v.y; c->worldPosB[k].z = v.z; c->worldPosB[k].w = v.w;
    }
    return 1;
}

int oracle_concave_contacts(const obody* bodies, const oshapes* sh, const oaabb* aabbs, const opair* tri_pairs, int n,
                            ocontact* out, int* out_index, int cap) {
    int i, m = 0;
    for (i = 0; i < n; i++) {
        ocontact c;
        memset(&c, 0, sizeof(c));
        if (sh->cols[bodies[tri_pairs[i].y].collidableIdx].shapeType == SHAPE_SPHERE
                ? concave_sphere(bodies, sh, &tri_pairs[i], i, &c)
                : concave_tri(bodies, sh, aabbs, &tri_pairs[i], i, &c)) {
            if (m < cap) { out[m] = c; if (out_index) out_index[m] = i; }
            m++;
        }
    }
    return m;
}

/* ------------------------------------------------------------------ solver */
typedef struct {
    v3 n;
    float jac, rhs, applied, fric;
    v3 r1xn, r2xn, angA, angB;
} orow;

typedef struct {
    int A, B, mask;
    float imA, imB;
    orow rows[12]; /* 4 contact rows, then per point (dir2, dir1) friction rows */
} omanifold;

/* b3PlaneSpace1 (Bullet3Common/b3Vector3.h:1184-1212) */
static void plane_space(v3 n, v3* p, v3* q) {
    if (fabsf(n.z) > 0.7071067811865475244008443621048490f) {
        float a = n.y * n.y + n.z * n.z, k = 1.0f / sqrtf(a);
        *p = mk(0.f, -n.z * k, n.y * k);
        *q = mk(a * k, -n.x * p->z, n.x * p->y);
    } else {
        float a = n.x * n.x + n.y * n.y, k = 1.0f / sqrtf(a);
        *p = mk(-n.y * k, n.x * k, 0.f);
        *q = mk(-n.z * p->y, n.z * p->x, a * k);
    }
}

/* convertContact + setupContactConstraint + setupFrictionConstraint
 * (Bullet3Dynamics/ConstraintSolver/b3PgsJacobiSolver.cpp:457-536, :654-804, :847-983) */
static void setup_manifold(const obody* bodies, const oinertia* inertias, const ocontact* c, const int* counts,
                           int pgs, float dt, float erp, float threshold, omanifold* M) {
    int iA = abs(c->bodyA), iB = abs(c->bodyB), np = (int)c->worldNormalOnB.w, j, k;
    const obody* A = &bodies[iA];
    const obody* B = &bodies[iB];
    float imA = A->invMass, imB = B->invMass, countA = 1.f, countB = 1.f, fric;
    const omat3* IA = &inertias[iA].invInertiaWorld;
    const omat3* IB = &inertias[iB].invInertiaWorld;
    v3 posA = f4v(A->pos), posB = f4v(B->pos), linA = f4v(A->linVel), angA = f4v(A->angVel), linB = f4v(B->linVel),
       angB = f4v(B->angVel), n;
    memset(M, 0, sizeof(*M));
    M->A = iA; M->B = iB; M->imA = imA; M->imB = imB;
    if (np > 4) np = 4;
    if (imA == 0.f && imB == 0.f) np = 0;
    if (!pgs) {
        if (imA != 0.f) countA = (float)counts[iA];
        if (imB != 0.f) countB = (float)counts[iB];
    }
    n = nrm(mk(c->worldNormalOnB.x, c->worldNormalOnB.y, c->worldNormalOnB.z));
    fric = (float)c->frictionCmp / (float)0xffff;
    for (j = 0; j < np; j++) {
        float dist = c->worldPosB[j].w;
        v3 pos2, pos1, rel1, rel2;
        if (!(dist <= threshold)) continue;
        M->mask |= 1 << j;
        pos2 = mk(c->worldPosB[j].x, c->worldPosB[j].y, c->worldPosB[j].z);
        pos1 = add(pos2, scl(n, dist));
        rel1 = sub(pos1, posA);
        rel2 = sub(pos2, posB);
        {
            v3 torqueAxis0 = cross(rel1, n), angCompA = imul(IA, torqueAxis0);
            v3 torqueAxis1 = cross(rel2, n), angCompB = imul(IB, neg(torqueAxis1));
            float denom0 = imA + dot(n, cross(angCompA, rel1));
            float denom1 = imB + dot(n, cross(neg(angCompB), rel2));
            float jac = 1.0f / (denom0 + denom1);
            float scaled = pgs ? jac : 1.0f / (denom0 * countA + denom1 * countB);
            v3 r1xn = torqueAxis0, r2xn = neg(torqueAxis1);
            float penetration = dist + 0.0f;
            float vel1Dotn = dot(n, linA) + dot(r1xn, angA);
            float vel2Dotn = -dot(n, linB) + dot(r2xn, angB);
            float rel_vel = vel1Dotn + vel2Dotn;
            float positionalError = 0.f, velocityError = 0.0f - rel_vel;
            orow* r = &M->rows[j];
            if (penetration > 0.f)
                velocityError -= penetration / dt;
            else
                positionalError = -penetration * erp / dt;
            r->n = n; r->jac = jac;
            r->rhs = positionalError * scaled + velocityError * scaled;
            r->applied = 0.f; r->fric = fric;
            r->r1xn = r1xn; r->r2xn = r2xn; r->angA = angCompA; r->angB = angCompB;
        }
        {
            v3 vel1 = add(linA, cross(angA, rel1)), vel2 = add(linB, cross(angB, rel2)), vel = sub(vel1, vel2);
            float rel_vel = dot(n, vel), lat;
            v3 dir1 = sub(vel, scl(n, rel_vel)), dir2, dirs[2];
            lat = dot(dir1, dir1);
            if (lat > FLT_EPSILON) {
                float inv = 1.f / sqrtf(lat), l2;
                dir1 = scl(dir1, inv);
                dir2 = cross(dir1, n);
                l2 = sqrtf(dot(dir2, dir2));
                dir2 = scl(dir2, 1.f / l2);
            } else {
                plane_space(n, &dir1, &dir2);
            }
            dirs[0] = dir2;
            dirs[1] = dir1;
            for (k = 0; k < 2; k++) {
                v3 d = dirs[k];
                v3 r1xn = cross(rel1, d), angCompA = imul(IA, r1xn);
                v3 r2xn = cross(rel2, neg(d)), angCompB = imul(IB, r2xn);
                float denom0 = imA + dot(d, cross(angCompA, rel1));
                float denom1 = imB + dot(d, cross(neg(angCompB), rel2));
                float jac = 1.0f / (denom0 + denom1);
                float scaled = pgs ? jac : 1.0f / (denom0 * countA + denom1 * countB);
                float v1 = dot(d, linA) + dot(r1xn, angA);
                float v2 = -dot(d, linB) + dot(r2xn, angB);
                float rv = v1 + v2;
                float velocityError = 0.0f - rv;
                orow* r = &M->rows[4 + 2 * j + k];
                r->n = d; r->jac = jac; r->rhs = velocityError * scaled; r->applied = 0.f; r->fric = fric;
                r->r1xn = r1xn; r->r2xn = r2xn; r->angA = angCompA; r->angB = angCompB;
            }
        }
    }
}

/* resolveSingleConstraintRowLowerLimit / Generic (b3PgsJacobiSolver.cpp:236-317) */
static float solve_row(orow* r, float lower, float upper, int friction, v3* dlA, v3* daA, v3* dlB, v3* daB,
                       float imA, float imB) {
    float applied = r->applied, old = applied;
    float deltaImpulse = r->rhs - applied * 0.0f;
    float dv1 = dot(r->n, *dlA) + dot(r->r1xn, *daA);
    float dv2 = -dot(r->n, *dlB) + dot(r->r2xn, *daB);
    float sum;
    deltaImpulse -= dv1 * r->jac;
    deltaImpulse -= dv2 * r->jac;
    sum = applied + deltaImpulse;
    if (sum < lower) {
        deltaImpulse = lower - applied;
        applied = lower;
    } else if (friction && sum > upper) {
        deltaImpulse = upper - applied;
        applied = upper;
    } else {
        applied = sum;
    }
    r->applied = applied;
    *dlA = add(*dlA, scl(scl(r->n, imA), deltaImpulse));
    *daA = add(*daA, scl(r->angA, deltaImpulse));
    *dlB = add(*dlB, scl(scl(neg(r->n), imB), deltaImpulse));
    *daB = add(*daB, scl(r->angB, deltaImpulse));
    return applied - old;
}

/* pass 0: contact rows, 1: friction rows, 2: interleaved (per point: its contact row, then its
 * two friction rows bounded by that row's new impulse), the B3_SOLVER_INTERLEAVE_CONTACT_AND_
 * FRICTION_CONSTRAINTS branch of solveSingleIteration (b3PgsJacobiSolver.cpp:1334-1377). */
static void solve_manifold(omanifold* M, int pass, v3* dlA, v3* daA, v3* dlB, v3* daB, double* rd, double* rl) {
    int j, k;
    if (pass == 2) {
        for (j = 0; j < 4; j++) {
            float d, total;
            if (!(M->mask & (1 << j))) continue;
            d = solve_row(&M->rows[j], 0.f, 1e10f, 0, dlA, daA, dlB, daB, M->imA, M->imB);
            *rd += (double)d * d;
            *rl += (double)M->rows[j].applied * M->rows[j].applied;
            total = M->rows[j].applied;
            for (k = 0; k < 2; k++) {
                orow* r = &M->rows[4 + 2 * j + k];
                if (total > 0.f) {
                    float fr = r->fric;
                    float dd = solve_row(r, -(fr * total), fr * total, 1, dlA, daA, dlB, daB, M->imA, M->imB);
                    *rd += (double)dd * dd;
                }
                *rl += (double)r->applied * r->applied;
            }
        }
        return;
    }
    if (pass == 0) {
        for (j = 0; j < 4; j++) {
            float d;
            if (!(M->mask & (1 << j))) continue;
            d = solve_row(&M->rows[j], 0.f, 1e10f, 0, dlA, daA, dlB, daB, M->imA, M->imB);
            *rd += (double)d * d;
            *rl += (double)M->rows[j].applied * M->rows[j].applied;
        }
    } else {
        for (j = 0; j < 4; j++) {
            float total;
            if (!(M->mask & (1 << j))) continue;
            total = M->rows[j].applied;
            for (k = 0; k < 2; k++) {
                orow* r = &M->rows[4 + 2 * j + k];
                if (total > 0.f) {
                    float fr = r->fric;
                    float d = solve_row(r, -(fr * total), fr * total, 1, dlA, daA, dlB, daB, M->imA, M->imB);
                    *rd += (double)d * d;
                }
                *rl += (double)r->applied * r->applied;
            }
        }
    }
}

/* a row's impulse delta applied to the body deltas, as solve_row applies it */
static void apply_row_impulse(const orow* r, float delta, v3* dlA, v3* daA, v3* dlB, v3* daB, float imA, float imB) {
    *dlA = add(*dlA, scl(scl(r->n, imA), delta));
    *daA = add(*daA, scl(r->angA, delta));
    *dlB = add(*dlB, scl(scl(neg(r->n), imB), delta));
    *daB = add(*daB, scl(r->angB, delta));
}

/* Warm start: each active point's initial impulses (w: normal, first lateral = dir1, second
 * lateral = dir2, the layout of impulses_out) become the rows' applied impulses and are applied
 * to the body deltas, contact row first, then the dir2 row, then the dir1 row -- the
 * internalApplyImpulse calls of setupContactConstraint / setupFrictionConstraint under
 * B3_SOLVER_USE_WARMSTARTING (b3PgsJacobiSolver.cpp:745-752, 815-843). */
static void warm_manifold(omanifold* M, const float* w, v3* dlA, v3* daA, v3* dlB, v3* daB) {
    int j;
    for (j = 0; j < 4; j++) {
        orow* c;
        if (!(M->mask & (1 << j))) continue;
        c = &M->rows[j];
        c->applied = w[3 * j + 0];
        apply_row_impulse(c, c->applied, dlA, daA, dlB, daB, M->imA, M->imB);
        c = &M->rows[4 + 2 * j + 0];
        c->applied = w[3 * j + 2];
        apply_row_impulse(c, c->applied, dlA, daA, dlB, daB, M->imA, M->imB);
        c = &M->rows[4 + 2 * j + 1];
        c->applied = w[3 * j + 1];
        apply_row_impulse(c, c->applied, dlA, daA, dlB, daB, M->imA, M->imB);
    }
}

static void gather_impulses(const omanifold* Ms, int nc, float* out) {
    int m, j;
    if (!out) return;
    for (m = 0; m < nc; m++)
        for (j = 0; j < 4; j++) {
            out[(size_t)m * 12 + 3 * j + 0] = Ms[m].rows[j].applied;
            out[(size_t)m * 12 + 3 * j + 1] = Ms[m].rows[4 + 2 * j + 1].applied;
            out[(size_t)m * 12 + 3 * j + 2] = Ms[m].rows[4 + 2 * j + 0].applied;
        }
}

static int solve_pgs_impl(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts, int nc,
                          const int* order, int interleave, const float* warm, int iterations, float dt, float erp,
                          float threshold, float tol, float* impulses_out, float* residual_out, int* discarded) {
    omanifold* Ms = (omanifold*)malloc(sizeof(omanifold) * (size_t)(nc > 0 ? nc : 1));
    v3* dl = (v3*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(v3));
    v3* da = (v3*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(v3));
    int m, it, pass, k, b, done = 0, extra = 0, warm_live = warm != NULL;
    double r = 0.0;
    for (m = 0; m < nc; m++) setup_manifold(bodies, inertias, &contacts[m], NULL, 1, dt, erp, threshold, &Ms[m]);
    if (discarded) *discarded = 0;
    if (warm)
        for (k = 0; k < nc; k++) {
            const int mm = order ? order[k] : k;
            omanifold* M = &Ms[mm];
            v3 dlA = dl[M->A], daA = da[M->A], dlB = dl[M->B], daB = da[M->B];
            if (!M->mask) continue;
            warm_manifold(M, warm + (size_t)mm * 12, &dlA, &daA, &dlB, &daB);
            if (M->imA != 0.f) { dl[M->A] = dlA; da[M->A] = daA; }
            if (M->imB != 0.f) { dl[M->B] = dlB; da[M->B] = daB; }
        }
    for (it = 0; it < iterations; it++) {
        double rd = 0.0, rl = 0.0;
        for (pass = 0; pass < (interleave ? 1 : 2); pass++)
            for (k = 0; k < nc; k++) {
                omanifold* M = &Ms[order ? order[k] : k];
                v3 dlA = dl[M->A], daA = da[M->A], dlB = dl[M->B], daB = da[M->B];
                if (!M->mask) continue;
                solve_manifold(M, interleave ? 2 : pass, &dlA, &daA, &dlB, &daB, &rd, &rl);
                if (M->imA != 0.f) { dl[M->A] = dlA; da[M->A] = daA; }
                if (M->imB != 0.f) { dl[M->B] = dlB; da[M->B] = daB; }
            }
        done = it + 1;
        r = sqrt(rd) / fmax(sqrt(rl), 1e-12);
        /* a warm start whose first sweep moved the impulses more than a cold start does (a cold
         * first sweep has residual exactly 1) is dropped: restart cold with the full budget */
        if (it == 0 && warm_live && r > 1.0) {
            int j;
            warm_live = 0;
            extra = 1;
            if (discarded) *discarded = 1;
            for (b = 0; b < nbodies; b++) { dl[b] = mk(0, 0, 0); da[b] = mk(0, 0, 0); }
            for (m = 0; m < nc; m++)
                for (j = 0; j < 12; j++) Ms[m].rows[j].applied = 0.f;
            it = -1;
            continue;
        }
        if (tol > 0.f && r <= (double)tol) break;
    }
    done += extra;
    /* solveGroupCacheFriendlyFinish, PGS branch: v += dv */
    for (b = 0; b < nbodies; b++) {
        if (bodies[b].invMass == 0.f) continue;
        bodies[b].linVel.x = bodies[b].linVel.x + dl[b].x;
        bodies[b].linVel.y = bodies[b].linVel.y + dl[b].y;
        bodies[b].linVel.z = bodies[b].linVel.z + dl[b].z;
        bodies[b].angVel.x = bodies[b].angVel.x + da[b].x;
        bodies[b].angVel.y = bodies[b].angVel.y + da[b].y;
        bodies[b].angVel.z = bodies[b].angVel.z + da[b].z;
    }
    gather_impulses(Ms, nc, impulses_out);
    if (residual_out) *residual_out = (float)r;
    free(Ms); free(dl); free(da);
    return done;
}

/* Jacobi (usePgs=false): split solver bodies per manifold, averaging after the contact and
 * the friction sweep (solveSingleIteration :1389-1391, solveGroupCacheFriendlyIterations :1541-1546),
 * summation in solver-body pool order (= manifold order, A before B), finish adds S/count once per
 * split copy (:1654-1668). */
static int solve_jacobi_impl(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts, int nc,
                             int iterations, float dt, float erp, float threshold, float tol, float* impulses_out,
                             float* residual_out) {
    omanifold* Ms = (omanifold*)malloc(sizeof(omanifold) * (size_t)(nc > 0 ? nc : 1));
    int* counts = (int*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(int));
    v3* avgl = (v3*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(v3));
    v3* avga = (v3*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(v3));
    v3* suml = (v3*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(v3));
    v3* suma = (v3*)calloc((size_t)(nbodies > 0 ? nbodies : 1), sizeof(v3));
    v3* split = (v3*)calloc((size_t)(nc > 0 ? nc : 1) * 4, sizeof(v3));
    int m, it, pass, b, done = 0, k;
    double r = 0.0;
    for (m = 0; m < nc; m++) {
        int a = abs(contacts[m].bodyA), bb = abs(contacts[m].bodyB);
        if (bodies[a].invMass != 0.f) counts[a]++;
        if (bodies[bb].invMass != 0.f) counts[bb]++;
    }
    for (m = 0; m < nc; m++) setup_manifold(bodies, inertias, &contacts[m], counts, 0, dt, erp, threshold, &Ms[m]);
    for (it = 0; it < iterations; it++) {
        double rd = 0.0, rl = 0.0;
        for (pass = 0; pass < 2; pass++) {
            for (m = 0; m < nc; m++) {
                omanifold* M = &Ms[m];
                v3 z = mk(0, 0, 0), dlA = z, daA = z, dlB = z, daB = z;
                if (M->imA != 0.f) { dlA = avgl[M->A]; daA = avga[M->A]; }
                if (M->imB != 0.f) { dlB = avgl[M->B]; daB = avga[M->B]; }
                if (M->mask) solve_manifold(M, pass, &dlA, &daA, &dlB, &daB, &rd, &rl);
                split[4 * m + 0] = dlA; split[4 * m + 1] = daA; split[4 * m + 2] = dlB; split[4 * m + 3] = daB;
            }
            /* averageVelocities */
            for (b = 0; b < nbodies; b++) { suml[b] = mk(0, 0, 0); suma[b] = mk(0, 0, 0); }
            for (m = 0; m < nc; m++) {
                omanifold* M = &Ms[m];
                if (M->imA != 0.f) { suml[M->A] = add(suml[M->A], split[4 * m + 0]); suma[M->A] = add(suma[M->A], split[4 * m + 1]); }
                if (M->imB != 0.f) { suml[M->B] = add(suml[M->B], split[4 * m + 2]); suma[M->B] = add(suma[M->B], split[4 * m + 3]); }
            }
            for (b = 0; b < nbodies; b++) {
                if (counts[b] <= 0) continue;
                {
                    float f = 1.f / (float)counts[b];
                    avgl[b] = scl(suml[b], f);
                    avga[b] = scl(suma[b], f);
                }
            }
        }
        done = it + 1;
        r = sqrt(rd) / fmax(sqrt(rl), 1e-12);
        if (tol > 0.f && r <= (double)tol) break;
    }
    for (b = 0; b < nbodies; b++) {
        float f;
        v3 dl, da, lv, av;
        if (counts[b] <= 0) continue;
        f = 1.f / (float)counts[b];
        dl = scl(suml[b], f);
        da = scl(suma[b], f);
        lv = f4v(bodies[b].linVel);
        av = f4v(bodies[b].angVel);
        for (k = 0; k < counts[b]; k++) { lv = add(lv, dl); av = add(av, da); }
        bodies[b].linVel.x = lv.x; bodies[b].linVel.y = lv.y; bodies[b].linVel.z = lv.z;
        bodies[b].angVel.x = av.x; bodies[b].angVel.y = av.y; bodies[b].angVel.z = av.z;
    }
    gather_impulses(Ms, nc, impulses_out);
    if (residual_out) *residual_out = (float)r;
    free(Ms); free(counts); free(avgl); free(avga); free(suml); free(suma); free(split);
    return done;
}

int oracle_solve(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts, int ncontacts,
                 int mode, int iterations, float dt, float erp, float threshold, float residual_tol,
                 float* impulses_out, float* residual_out) {
    if (mode == 1)
        return solve_jacobi_impl(bodies, inertias, nbodies, contacts, ncontacts, iterations, dt, erp, threshold,
                                 residual_tol, impulses_out, residual_out);
    return solve_pgs_impl(bodies, inertias, nbodies, contacts, ncontacts, NULL, mode == 2, NULL, iterations, dt, erp,
                          threshold, residual_tol, impulses_out, residual_out, NULL);
}

int oracle_solve_ordered(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts,
                         int ncontacts, const int* order, int interleave, int iterations, float dt, float erp,
                         float threshold, float* impulses_out) {
    return solve_pgs_impl(bodies, inertias, nbodies, contacts, ncontacts, order, interleave, NULL, iterations, dt, erp,
                          threshold, 0.f, impulses_out, NULL, NULL);
}

int oracle_solve_ordered_ex(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts,
                            int ncontacts, const int* order, int interleave, const float* warm, int iterations,
                            float dt, float erp, float threshold, float residual_tol, float* impulses_out,
                            float* residual_out, int* discarded_out) {
    return solve_pgs_impl(bodies, inertias, nbodies, contacts, ncontacts, order, interleave, warm, iterations, dt, erp,
                          threshold, residual_tol, impulses_out, residual_out, discarded_out);
}

/* ------------------------------------------------------------------ integrate */
void oracle_integrate(obody* bodies, int n, float dt, float damping, const float g[3]) {
    int i;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (i = 0; i < n; i++) {
        obody* b = &bodies[i];
        const float threshold = 0.25f * 3.14159254f;
        float fAngle, len;
        v3 w, axis;
        qt dorn, q;
        if (b->invMass == 0.f) continue;
        b->angVel.x *= damping;
        b->angVel.y *= damping;
        b->angVel.z *= damping;
        w = mk(b->angVel.x, b->angVel.y, b->angVel.z);
        fAngle = sqrtf(dot(w, w));
        if (fAngle * dt > threshold) fAngle = threshold / dt;
        if (fAngle < 0.001f)
            axis = scl(w, (0.5f * dt - (dt * dt * dt) * 0.020833333333f * fAngle * fAngle));
        else
            axis = scl(w, (sinf(0.5f * fAngle * dt) / fAngle));
        dorn.x = axis.x; dorn.y = axis.y; dorn.z = axis.z; dorn.w = cosf(fAngle * dt * 0.5f);
        q = qmul(dorn, f4q(b->quat));
        len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
        if (len > 0.f) {
            float inv = 1.f / len;
            q.x *= inv; q.y *= inv; q.z *= inv; q.w *= inv;
        } else {
            q.x = q.y = q.z = 0.f; q.w = 1.f;
        }
        b->quat.x = q.x; b->quat.y = q.y; b->quat.z = q.z; b->quat.w = q.w;
        b->pos.x = b->pos.x + b->linVel.x * dt;
        b->pos.y = b->pos.y + b->linVel.y * dt;
        b->pos.z = b->pos.z + b->linVel.z * dt;
        b->linVel.x = b->linVel.x + g[0] * dt;
        b->linVel.y = b->linVel.y + g[1] * dt;
        b->linVel.z = b->linVel.z + g[2] * dt;
    }
}

/* ------------------------------------------------------------------ batching legality */
int oracle_check_batches(const ocontact* contacts, int n, const int* color, const obody* bodies, int nbodies) {
    int maxc = 0, m, bad = 0;
    for (m = 0; m < n; m++) if (color[m] > maxc) maxc = color[m];
    {
        int* last = (int*)malloc(sizeof(int) * (size_t)(nbodies > 0 ? nbodies : 1));
        int c;
        for (c = 0; c <= maxc; c++) {
            int b;
            for (b = 0; b < nbodies; b++) last[b] = -1;
            for (m = 0; m < n; m++) {
                int a, bb;
                if (color[m] != c) continue;
                a = abs(contacts[m].bodyA);
                bb = abs(contacts[m].bodyB);
                if (bodies[a].invMass != 0.f) { if (last[a] >= 0) bad++; last[a] = m; }
                if (bodies[bb].invMass != 0.f) { if (last[bb] >= 0) bad++; last[bb] = m; }
            }
        }
        free(last);
    }
    for (m = 0; m < n; m++) if (color[m] < 0) bad++;
    return bad;
}

/* ------------------------------------------------------------------ composed step */
int oracle_step(obody* bodies, const oinertia* inertias, int n, const oshapes* sh, const ostep_params* p,
                int* npairs_out, int* npoints_out) {
    oaabb* aabbs = (oaabb*)malloc(sizeof(oaabb) * (size_t)(n > 0 ? n : 1));
    int cap = 16 * n + 1024, np, nc, m, pts = 0;
    opair* pairs;
    ocontact* contacts;
    oracle_aabbs(bodies, n, sh, aabbs);
    pairs = (opair*)malloc(sizeof(opair) * (size_t)cap);
    np = p->use_grid ? oracle_pairs_grid(aabbs, n, p->cell, pairs, cap) : oracle_pairs_bruteforce(aabbs, n, pairs, cap);
    if (np > cap) np = cap;
    contacts = (ocontact*)malloc(sizeof(ocontact) * (size_t)(np > 0 ? np : 1));
    nc = oracle_contacts(bodies, sh, pairs, np, contacts, np, p->friction_cmp);
    for (m = 0; m < nc; m++) pts += (int)contacts[m].worldNormalOnB.w;
    oracle_solve(bodies, inertias, n, contacts, nc, p->mode, p->iterations, p->dt, p->erp, p->threshold,
                 p->residual_tol, NULL, NULL);
    oracle_integrate(bodies, n, p->dt, p->damping, p->gravity);
    if (npairs_out) *npairs_out = np;
    if (npoints_out) *npoints_out = pts;
    free(aabbs);
    free(pairs);
    free(contacts);
    return nc;
}

/* ------------------------------------------------------------------ ray casts */
/* qtMul / qtRotate of rayCastKernels.cl:101-131: ans = cross(a, b) + (a.w b + b.w a),
 * ans.w = a.w b.w - dot3(a, b) */
static inline qt cl_qmul(qt a, qt b) {
    qt r;
    r.x = (a.y * b.z - a.z * b.y) + (a.w * b.x + b.w * a.x);
    r.y = (a.z * b.x - a.x * b.z) + (a.w * b.y + b.w * a.y);
    r.z = (a.x * b.y - a.y * b.x) + (a.w * b.z + b.w * a.z);
    r.w = a.w * b.w - (a.x * b.x + a.y * b.y + a.z * b.z);
    return r;
}
static inline v3 cl_qrot(qt q, v3 v) {
    qt vq = {v.x, v.y, v.z, 0.0f};
    qt inv = {-q.x, -q.y, -q.z, q.w};
    qt t = cl_qmul(cl_qmul(q, vq), inv);
    return mk(t.x, t.y, t.z);
}

/* rayConvex (rayCastKernels.cl:157-217) with hitFraction in/out */
static int ray_convex(v3 from, v3 to, const oface* faces, int nf, float* hitFraction, v3* hitNormal) {
    float exitFraction = *hitFraction, enterFraction = -0.3f;
    v3 cur = mk(0.0f, 0.0f, 0.0f);
    int result = 1, i;
    for (i = 0; i < nf && result; i++) {
        const oface* f = &faces[i];
        v3 n = mk(f->plane.x, f->plane.y, f->plane.z);
        float fromd = dot(from, n) + f->plane.w;
        float tod = dot(to, n) + f->plane.w;
        if (fromd < 0.0f) {
            if (tod >= 0.0f) {
                float fraction = fromd / (fromd - tod);
                if (exitFraction > fraction) exitFraction = fraction;
            }
        } else {
            if (tod < 0.0f) {
                float fraction = fromd / (fromd - tod);
                if (enterFraction <= fraction) {
                    enterFraction = fraction;
                    cur = n;
                }
            } else {
                result = 0;
            }
        }
        if (exitFraction <= enterFraction) result = 0;
    }
    if (enterFraction < 0.0f) result = 0;
    if (result) {
        *hitFraction = enterFraction;
        *hitNormal = cur;
    }
    return result;
}

/* sphere_intersect (rayCastKernels.cl:224-248) */
static int ray_sphere(v3 c, float radius, v3 from, v3 to, float* hitFraction) {
    v3 rs = sub(from, c), d = sub(to, from);
    float A = dot(d, d), B = dot(rs, d), C = dot(rs, rs) - radius * radius;
    float D = B * B - A * C;
    if (D > 0.0f) {
        float t = (-B - sqrtf(D)) / A;
        if (t >= 0.0f && t < *hitFraction) {
            *hitFraction = t;
            return 1;
        }
    }
    return 0;
}

/* setInterpolate3 (rayCastKernels.cl:250-258) */
static inline v3 ray_lerp(v3 a, v3 b, float t) {
    float s = 1.0f - t;
    return mk(s * a.x + t * b.x, s * a.y + t * b.y, s * a.z + t * b.z);
}

void oracle_cast_rays(const obody* bodies, int nbodies, const oshapes* sh, const oray* rays, oray_hit* hits,
                      int nrays, const int* body_scene) {
    int r;
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 64)
    for (r = 0; r < nrays; r++) {
        v3 from = f4v(rays[r].from), to = f4v(rays[r].to), hp = mk(0, 0, 0), hn = mk(0, 0, 0);
        float hf = 1.0f;
        int hb = -1, b;
        const int scene = body_scene ? (int)rays[r].from.w : 0;
        hits[r].hitFraction = 1.0f;
        for (b = 0; b < nbodies; b++) {
            const obody* B = &bodies[b];
            const ocollidable* c = &sh->cols[B->collidableIdx];
            if (hits[r].hitResult2 == b) continue;
            if (body_scene && body_scene[b] != scene) continue;
            if (c->shapeType == 3) {
                qt inv = {-B->quat.x, -B->quat.y, -B->quat.z, B->quat.w};
                v3 invPos = cl_qrot(inv, neg(f4v(B->pos)));
                v3 lf = add(cl_qrot(inv, from), invPos), lt = add(cl_qrot(inv, to), invPos);
                const ohull* hull = &sh->hulls[c->shapeIndex];
                if (hull->numFaces && ray_convex(lf, lt, &sh->faces[hull->faceOffset], hull->numFaces, &hf, &hn)) {
                    hb = b;
                    hp = ray_lerp(from, to, hf);
                }
            } else if (c->shapeType == 7) {
                if (ray_sphere(f4v(B->pos), c->radius, from, to, &hf)) {
                    hb = b;
                    hp = ray_lerp(from, to, hf);
                    hn = sub(hp, f4v(B->pos));
                }
            }
        }
        if (hb >= 0) {
            v3 n = nrm(hn);
            hits[r].hitFraction = hf;
            hits[r].hitBody = hb;
            hits[r].hitPoint.x = hp.x; hits[r].hitPoint.y = hp.y; hits[r].hitPoint.z = hp.z; hits[r].hitPoint.w = 0.0f;
            hits[r].hitNormal.x = n.x; hits[r].hitNormal.y = n.y; hits[r].hitNormal.z = n.z; hits[r].hitNormal.w = 0.0f;
        }
    }
}

/* ------------------------------------------------------------------ joints */
/* The joint kernels' quaternion product is the ray kernels' (cl_qmul / cl_qrot above:
 * jointSolver.cl:222-262 has the same qtMul / qtRotate). */

/* acos for getAngle (jointSolver.cl:557-572): asin(z) = sum (2n)!/(4^n n!^2 (2n+1)) z^(2n+1),
 * 12 terms in Horner form, with acos(x) = 2 asin(sqrt((1-x)/2)) for x > 1/2,
 * pi - 2 asin(sqrt((1+x)/2)) for x < -1/2, pi/2 - asin(x) between. */
static const float j_asin[11] = {0.166666672f,   0.075000003f,   0.0446428582f,  0.030381944f,
                                 0.0223721582f,  0.0173527636f,  0.0139648439f,  0.0115518011f,
                                 0.00976160914f, 0.00839033537f, 0.007312526f};
static float j_asin_series(float z) {
    float t = z * z, p = j_asin[10];
    int i;
    for (i = 9; i >= 0; --i) p = j_asin[i] + t * p;
    return z + (z * t) * p;
}
float oracle_joint_acos(float x) {
    if (x > 0.5f) return 2.0f * j_asin_series(sqrtf((1.0f - x) * 0.5f));
    if (x < -0.5f) return 3.14159274f - 2.0f * j_asin_series(sqrtf((1.0f + x) * 0.5f));
    return 1.57079637f - j_asin_series(x);
}

int oracle_joint_batches(const ojoint* joints, int n, const obody* bodies, int nbodies, int* order, int* batch_off) {
    int *A = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1)), *B = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    unsigned* used = (unsigned*)calloc((size_t)nbodies / 32 + 1, sizeof(unsigned));
    int i, valid = 0, nb = 0;
    for (i = 0; i < n; i++) {
        A[i] = bodies[joints[i].rbA].invMass != 0.f ? joints[i].rbA : -joints[i].rbA;
        B[i] = bodies[joints[i].rbB].invMass != 0.f ? joints[i].rbB : -joints[i].rbB;
        order[i] = i;
    }
    batch_off[0] = 0;
    while (valid < n) {
        int count = 0;
        memset(used, 0, sizeof(unsigned) * ((size_t)nbodies / 32 + 1));
        for (i = valid; i < n; i++) {
            int as = A[i], bs = B[i], a = abs(as), b = abs(bs);
            int a_static = as < 0 || as == -1, b_static = bs < 0 || bs == -1; /* staticIdx = -1 */
            int a_busy = 0, b_busy = 0;
            if (!a_static) a_busy = (used[a / 32] >> (a & 31)) & 1u;
            if (!a_busy && !b_static) b_busy = (used[b / 32] >> (b & 31)) & 1u;
            if (a_busy || b_busy) continue;
            if (!a_static) used[a / 32] |= 1u << (a & 31);
            if (!b_static) used[b / 32] |= 1u << (b & 31);
            if (i != valid) {
                int t;
                t = A[i]; A[i] = A[valid]; A[valid] = t;
                t = B[i]; B[i] = B[valid]; B[valid] = t;
                t = order[i]; order[i] = order[valid]; order[valid] = t;
            }
            valid++;
            count++;
        }
        batch_off[nb + 1] = batch_off[nb] + count;
        nb++;
    }
    free(A);
    free(B);
    free(used);
    return nb;
}

typedef struct {
    v3 n, r1, r2, angA, angB;
    float rhs, jinv, lo, hi, applied;
} ojrow;

static inline v3 j_mtmul1(const omat3* m, v3 b) {
    return mk(dot(f4v(m->row[0]), b), dot(f4v(m->row[1]), b), dot(f4v(m->row[2]), b));
}
static inline v3 j_mtmul3(v3 a, const omat3* m) {
    return mk(dot(a, mk(m->row[0].x, m->row[1].x, m->row[2].x)), dot(a, mk(m->row[0].y, m->row[1].y, m->row[2].y)),
              dot(a, mk(m->row[0].z, m->row[1].z, m->row[2].z)));
}

/* calculateDiffAxisAngleQuaternion with nearest / getAngle / b3Acos (jointSolver.cl:543-590) */
static void j_diff_axis_angle(qt orn0, qt orn1a, v3* axis, float* angle) {
    qt d = {orn0.x - orn1a.x, orn0.y - orn1a.y, orn0.z - orn1a.z, orn0.w - orn1a.w};
    qt s = {orn0.x + orn1a.x, orn0.y + orn1a.y, orn0.z + orn1a.z, orn0.w + orn1a.w};
    float dd = d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w, ss = s.x * s.x + s.y * s.y + s.z * s.z + s.w * s.w;
    qt orn1 = orn1a, dorn;
    float w, len;
    if (!(dd < ss)) { orn1.x = -orn1a.x; orn1.y = -orn1a.y; orn1.z = -orn1a.z; orn1.w = -orn1a.w; }
    dorn = cl_qmul(orn1, qconj(orn0));
    w = dorn.w;
    if (w >= 1.f) w = 1.f;
    if (w < -1.f) w = -1.f;
    *angle = 2.f * oracle_joint_acos(w);
    *axis = mk(dorn.x, dorn.y, dorn.z);
    len = dot(*axis, *axis);
    if (len < FLT_EPSILON * FLT_EPSILON) {
        *axis = mk(1.f, 0.f, 0.f);
    } else {
        float r = sqrtf(len);
        *axis = mk(axis->x / r, axis->y / r, axis->z / r);
    }
}

static int j_rows(int type) { return type == 4 ? 6 : type == 3 ? 3 : 0; }

/* getInfo2Kernel (jointSolver.cl:651-870) for one joint: getInfo2Point2Point (:488-541),
 * getInfo2FixedOrientation (:592-628), then the finalize loop */
static void j_setup(const obody* bodies, const oinertia* inertias, const ojoint* c, ojrow* rows) {
    const float dt = 1.f / 60.f, erp = 0.2f, damping = 1.f, k = (1.f / dt) * erp;
    const obody *bA = &bodies[c->rbA], *bB = &bodies[c->rbB];
    int nr = j_rows(c->type), j;
    qt qA = f4q(bA->quat), qB = f4q(bB->quat);
    v3 a1 = cl_qrot(qA, f4v(c->pivotInA)), a2 = cl_qrot(qB, f4v(c->pivotInB)), m1 = neg(a1);
    v3 vA = f4v(bA->linVel), wA = f4v(bA->angVel), vB = f4v(bB->linVel), wB = f4v(bB->angVel);
    const omat3 *IA = &inertias[c->rbA].invInertiaWorld, *IB = &inertias[c->rbB].invInertiaWorld;
    rows[0].n = mk(1.f, 0.f, 0.f);
    rows[1].n = mk(0.f, 1.f, 0.f);
    rows[2].n = mk(0.f, 0.f, 1.f);
    rows[0].r1 = mk(0.f, -m1.z, m1.y);
    rows[1].r1 = mk(m1.z, 0.f, -m1.x);
    rows[2].r1 = mk(-m1.y, m1.x, 0.f);
    rows[0].r2 = mk(0.f, -a2.z, a2.y);
    rows[1].r2 = mk(a2.z, 0.f, -a2.x);
    rows[2].r2 = mk(-a2.y, a2.x, 0.f);
    rows[0].rhs = k * (((a2.x + bB->pos.x) - a1.x) - bA->pos.x);
    rows[1].rhs = k * (((a2.y + bB->pos.y) - a1.y) - bA->pos.y);
    rows[2].rhs = k * (((a2.z + bB->pos.z) - a1.z) - bA->pos.z);
    if (nr == 6) {
        v3 axis;
        float angle, na;
        for (j = 0; j < 3; j++) {
            rows[3 + j].n = mk(0.f, 0.f, 0.f);
            rows[3 + j].r1 = mk(j == 0 ? 1.f : 0.f, j == 1 ? 1.f : 0.f, j == 2 ? 1.f : 0.f);
            rows[3 + j].r2 = mk(j == 0 ? -1.f : 0.f, j == 1 ? -1.f : 0.f, j == 2 ? -1.f : 0.f);
        }
        j_diff_axis_angle(f4q(c->relTargetAB), cl_qmul(qA, qconj(qB)), &axis, &angle);
        na = -angle;
        rows[3].rhs = k * (axis.x * na);
        rows[4].rhs = k * (axis.y * na);
        rows[5].rhs = k * (axis.z * na);
    }
    for (j = 0; j < nr; j++) {
        ojrow* r = &rows[j];
        float sum, vel1, vel2, rel;
        r->lo = -1e30f;
        r->hi = 1e30f;
        if (r->hi >= c->breakingImpulseThreshold) r->hi = c->breakingImpulseThreshold;
        if (r->lo <= -c->breakingImpulseThreshold) r->lo = -c->breakingImpulseThreshold;
        r->angA = j_mtmul1(IA, r->r1);
        r->angB = j_mtmul1(IB, r->r2);
        sum = dot(scl(r->n, bA->invMass), r->n);
        sum += dot(j_mtmul3(r->r1, IA), r->r1);
        sum += dot(scl(r->n, bB->invMass), r->n);
        sum += dot(j_mtmul3(r->r2, IB), r->r2);
        r->jinv = fabsf(sum) > FLT_EPSILON ? 1.f / sum : 0.f;
        vel1 = dot(r->n, vA) + dot(r->r1, wA);
        vel2 = -dot(r->n, vB) + dot(r->r2, wB);
        rel = vel1 + vel2;
        r->rhs = r->rhs * r->jinv + (0.f - rel * damping) * r->jinv;
        r->applied = 0.f;
    }
}

/* resolveSingleConstraintRowGeneric (jointSolver.cl:273-301) */
static void j_resolve(ojrow* r, float imA, float imB, v3* dlA, v3* daA, v3* dlB, v3* daB) {
    const float cfm = 0.f;
    float delta = r->rhs - r->applied * cfm, d1, d2, sum;
    d1 = dot(r->n, *dlA) + dot(r->r1, *daA);
    d2 = -dot(r->n, *dlB) + dot(r->r2, *daB);
    delta -= d1 * r->jinv;
    delta -= d2 * r->jinv;
    sum = r->applied + delta;
    if (sum < r->lo) {
        delta = r->lo - r->applied;
        r->applied = r->lo;
    } else if (sum > r->hi) {
        delta = r->hi - r->applied;
        r->applied = r->hi;
    } else {
        r->applied = sum;
    }
    *dlA = add(*dlA, scl(scl(r->n, imA), delta));
    *daA = add(*daA, scl(r->angA, delta));
    *dlB = add(*dlB, scl(scl(neg(r->n), imB), delta));
    *daB = add(*daB, scl(r->angB, delta));
}

void oracle_solve_joints(obody* bodies, const oinertia* inertias, int nbodies, ojoint* joints, int n,
                         const int* order, const int* batch_off, int nbatches) {
    ojrow* rows = (ojrow*)calloc((size_t)(n > 0 ? n : 1) * 6, sizeof(ojrow));
    v3* dl = (v3*)calloc((size_t)nbodies, sizeof(v3));
    v3* da = (v3*)calloc((size_t)nbodies, sizeof(v3));
    int i, j, it, b, k;
    for (i = 0; i < n; i++) j_setup(bodies, inertias, &joints[i], rows + 6 * (size_t)i);
    for (it = 0; it < 4; it++)
        for (b = 0; b < nbatches; b++)
            for (k = batch_off[b]; k < batch_off[b + 1]; k++) {
                const ojoint* c = &joints[order[k]];
                ojrow* r = rows + 6 * (size_t)order[k];
                if (!(c->flags & 1)) continue;
                for (j = 0; j < j_rows(c->type); j++)
                    j_resolve(&r[j], bodies[c->rbA].invMass, bodies[c->rbB].invMass, &dl[c->rbA], &da[c->rbA],
                              &dl[c->rbB], &da[c->rbB]);
            }
    for (i = 0; i < n; i++)
        for (j = 0; j < j_rows(joints[i].type); j++)
            if (fabsf(rows[6 * (size_t)i + j].applied) >= joints[i].breakingImpulseThreshold) joints[i].flags = 0;
    for (i = 0; i < nbodies; i++) {
        if (bodies[i].invMass == 0.f) continue;
        bodies[i].linVel.x += dl[i].x;
        bodies[i].linVel.y += dl[i].y;
        bodies[i].linVel.z += dl[i].z;
        bodies[i].angVel.x += da[i].x;
        bodies[i].angVel.y += da[i].y;
        bodies[i].angVel.z += da[i].z;
    }
    free(rows);
    free(dl);
    free(da);
}
