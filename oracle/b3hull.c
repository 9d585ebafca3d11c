/* b3hull.c -- the oracle's restatement of the reference's shape and body registration: convex-hull
 * topology, hull tables, and the body / inertia records registerPhysicsInstance writes.
 * TEST INFRASTRUCTURE ONLY: called by tests/, the smoke check and the bench's CPU legs (which
 * build their scene tables with it, so that they load nothing of the product).  Compiled with
 * -ffp-contract=off so every float operation rounds where the reference's does.
 *
 * Reference functions restated (paths relative to the reference project's src/):
 *   b3ConvexHullComputer::compute and b3ConvexHullInternal (Kniemeyer's Preparata-Hong hull on a
 *     quantised integer grid)       Bullet3Geometry/b3ConvexHullComputer.cpp
 *       input quantisation + sort                       :1943-2062
 *       divide and conquer                              :1209-1324
 *       merge of the two x/y projections                :1024-1207
 *       3-D merge (gift wrapping between the halves)    :1651-1936
 *       orientation / max-angle / coplanar-face search  :1390-1649
 *       output vertices, edges, faces                   :2625-2745
 *     b3AlignedObjectArray::quickSortInternal           Bullet3Common/b3AlignedObjectArray.h:330-357
 *   b3ConvexUtility::initializePolyhedralFeatures       Bullet3Collision/NarrowPhaseCollision/b3ConvexUtility.cpp:26-246
 *     b3ConvexUtility::initialize (unique edges)        :319-375
 *     b3GrahamScanConvexHull2D                          Bullet3Geometry/b3GrahamScan2dConvexHull.h:56-111
 *     b3PlaneSpace1                                     Bullet3Common/b3Vector3.h:1184-1212
 *   b3GpuNarrowPhase::registerConvexHullShape           Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.cpp:298-368
 *   b3GpuNarrowPhase::registerSphereShape / PlaneShape  :159-232
 *   b3GpuRigidBodyPipeline::registerPhysicsInstance     Bullet3OpenCL/RigidBody/b3GpuRigidBodyPipeline.cpp:603-669
 *   b3GpuNarrowPhase::registerRigidBody                 Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.cpp:816-908
 *     b3TransformAabb (margin 0.01)                     Bullet3Geometry/b3AabbUtil.h:146-159
 *     b3Matrix3x3(quaternion), scaled, transpose, *     Bullet3Common/b3Matrix3x3.h
 *
 * All integer arithmetic of the hull is exact (64-bit, 128-bit products through unsigned __int128);
 * the coordinates after quantisation lie within +-10216, so no product overflows.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "b3oracle.h"

/* ------------------------------------------------------------------ integer hull */
typedef struct { int32_t x, y, z; } hp32;
typedef struct { int64_t x, y, z; } hp64;

typedef struct hv hv;
typedef struct he he;
struct hv {           /* b3ConvexHullInternal::Vertex (the fields the unshrunk hull uses) */
    hv *next, *prev;  /* ring of the current 2-D projection */
    he *edges;        /* one outgoing edge; the others follow through next */
    hp32 p;
    int copy;         /* output index, -1 before */
};
struct he {           /* b3ConvexHullInternal::Edge */
    he *next, *prev;  /* ring of the edges leaving the same vertex */
    he *reverse;
    hv *target;
    int copy;         /* merge stamp while building, output index when extracting */
};
typedef struct { hv *minXy, *maxXy, *minYx, *maxYx; } hhull;

typedef struct edge_chunk { struct edge_chunk *prev; int used, cap; he e[]; } edge_chunk;

typedef struct {
    hv *verts;            /* sorted quantised points (originalVertices) */
    edge_chunk *chunks;   /* edge storage, never moved */
    he *free_edges;       /* edges released by remove_edge_pair */
    int chunk_cap;
    int merge_stamp;
    int fail;             /* allocation failure */
} hctx;

static hp32 p_sub(hp32 a, hp32 b) { hp32 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static hp64 p_cross(hp32 a, hp32 b) {
    hp64 r = {(int64_t)a.y * b.z - (int64_t)a.z * b.y, (int64_t)a.z * b.x - (int64_t)a.x * b.z,
              (int64_t)a.x * b.y - (int64_t)a.y * b.x};
    return r;
}
static hp64 p_cross64(hp32 a, hp64 b) {
    hp64 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static int64_t p_dot(hp32 a, hp32 b) { return (int64_t)a.x * b.x + (int64_t)a.y * b.y + (int64_t)a.z * b.z; }
static int64_t p_dot64(hp32 a, hp64 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static int64_t q_dot(hp64 a, hp64 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static int p_eq(hp32 a, hp32 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
static hp32 v_sub(const hv *a, const hv *b) { return p_sub(a->p, b->p); }

/* b3ConvexHullInternal::Rational64: sign and magnitudes, compared through 128-bit products */
typedef struct { uint64_t num, den; int sign; } rat64;
static rat64 rat_make(int64_t n, int64_t d) {
    rat64 r;
    if (n > 0) { r.sign = 1; r.num = (uint64_t)n; }
    else if (n < 0) { r.sign = -1; r.num = (uint64_t)(-n); }
    else { r.sign = 0; r.num = 0; }
    if (d > 0) r.den = (uint64_t)d;
    else if (d < 0) { r.sign = -r.sign; r.den = (uint64_t)(-d); }
    else r.den = 0;
    return r;
}
static int rat_is_neg_inf(rat64 r) { return r.sign < 0 && r.den == 0; }
static int rat_is_nan(rat64 r) { return r.sign == 0 && r.den == 0; }
static int rat_cmp(rat64 a, rat64 b) {
    if (a.sign != b.sign) return a.sign - b.sign;
    if (a.sign == 0) return 0;
    unsigned __int128 l = (unsigned __int128)a.num * b.den, r = (unsigned __int128)a.den * b.num;
    return a.sign * (l < r ? -1 : l > r ? 1 : 0);
}

static he *edge_alloc(hctx *c) {
    he *e = c->free_edges;
    if (e) {
        c->free_edges = e->next;
    } else {
        edge_chunk *k = c->chunks;
        if (!k || k->used == k->cap) {
            k = (edge_chunk *)malloc(sizeof(edge_chunk) + sizeof(he) * (size_t)c->chunk_cap);
            if (!k) { c->fail = 1; return NULL; }
            k->prev = c->chunks;
            k->used = 0;
            k->cap = c->chunk_cap;
            c->chunks = k;
        }
        e = &k->e[k->used++];
    }
    memset(e, 0, sizeof(*e));
    return e;
}

/* newEdgePair (:1003-1022): an edge from -> to and its reverse, stamped with the merge stamp */
static he *new_edge_pair(hctx *c, hv *from, hv *to) {
    he *e = edge_alloc(c), *r = edge_alloc(c);
    if (!e || !r) return NULL;
    e->reverse = r; r->reverse = e;
    e->copy = c->merge_stamp; r->copy = c->merge_stamp;
    e->target = to; r->target = from;
    return e;
}

/* removeEdgePair (:777-808) */
static void remove_edge_pair(hctx *c, he *edge) {
    he *n = edge->next, *r = edge->reverse;
    if (n != edge) {
        n->prev = edge->prev;
        edge->prev->next = n;
        r->target->edges = n;
    } else {
        r->target->edges = NULL;
    }
    n = r->next;
    if (n != r) {
        n->prev = r->prev;
        r->prev->next = n;
        edge->target->edges = n;
    } else {
        edge->target->edges = NULL;
    }
    edge->next = c->free_edges; c->free_edges = edge;
    r->next = c->free_edges; c->free_edges = r;
}

static void link_edges(he *a, he *n) { a->next = n; n->prev = a; } /* Edge::link */

enum { OR_NONE = 0, OR_CW = 1, OR_CCW = 2 };

/* getOrientation (:1390-1414) */
static int get_orientation(const he *prev, const he *next, hp32 s, hp32 t) {
    if (prev->next == next) {
        if (prev->prev == next) {
            hp64 n = p_cross(t, s);
            hp64 m = p_cross(v_sub(prev->target, next->reverse->target), v_sub(next->target, next->reverse->target));
            int64_t dot = q_dot(n, m);
            return dot > 0 ? OR_CCW : OR_CW;
        }
        return OR_CCW;
    } else if (prev->prev == next) {
        return OR_CW;
    }
    return OR_NONE;
}

/* findMaxAngle (:1416-1466) */
static he *find_max_angle(hctx *c, int ccw, const hv *start, hp32 s, hp64 rxs, hp64 sxrxs, rat64 *minCot) {
    he *minEdge = NULL;
    he *e = start->edges;
    if (e) {
        do {
            if (e->copy > c->merge_stamp) {
                hp32 t = v_sub(e->target, start);
                rat64 cot = rat_make(p_dot64(t, sxrxs), p_dot64(t, rxs));
                if (!rat_is_nan(cot)) {
                    int cmp;
                    if (minEdge == NULL) {
                        *minCot = cot;
                        minEdge = e;
                    } else if ((cmp = rat_cmp(cot, *minCot)) < 0) {
                        *minCot = cot;
                        minEdge = e;
                    } else if (cmp == 0 && ccw == (get_orientation(minEdge, e, s, t) == OR_CCW)) {
                        minEdge = e;
                    }
                }
            }
            e = e->next;
        } while (e != start->edges);
    }
    return minEdge;
}

/* findEdgeForCoplanarFaces (:1468-1649) */
static void find_edge_for_coplanar_faces(hctx *c, hv *c0, hv *c1, he **pe0, he **pe1, hv *stop0, hv *stop1) {
    he *e0 = *pe0, *e1 = *pe1;
    he *start0 = e0, *start1 = e1;
    hp32 et0 = start0 ? start0->target->p : c0->p;
    hp32 et1 = start1 ? start1->target->p : c1->p;
    hp32 s = p_sub(c1->p, c0->p);
    hp64 normal = p_cross(p_sub((start0 ? start0 : start1)->target->p, c0->p), s);
    int64_t dist = p_dot64(c0->p, normal);
    hp64 perp = p_cross64(s, normal);

    int64_t maxDot0 = p_dot64(et0, perp);
    if (e0) {
        while (e0->target != stop0) {
            he *e = e0->reverse->prev;
            if (p_dot64(e->target->p, normal) < dist) break;
            if (e->copy == c->merge_stamp) break;
            int64_t dot = p_dot64(e->target->p, perp);
            if (dot <= maxDot0) break;
            maxDot0 = dot;
            e0 = e;
            et0 = e->target->p;
        }
    }
    int64_t maxDot1 = p_dot64(et1, perp);
    if (e1) {
        while (e1->target != stop1) {
            he *e = e1->reverse->next;
            if (p_dot64(e->target->p, normal) < dist) break;
            if (e->copy == c->merge_stamp) break;
            int64_t dot = p_dot64(e->target->p, perp);
            if (dot <= maxDot1) break;
            maxDot1 = dot;
            e1 = e;
            et1 = e->target->p;
        }
    }

    int64_t dx = maxDot1 - maxDot0;
    if (dx > 0) {
        for (;;) {
            int64_t dy = p_dot(p_sub(et1, et0), s);
            if (e0 && e0->target != stop0) {
                he *f0 = e0->next->reverse;
                if (f0->copy > c->merge_stamp) {
                    int64_t dx0 = p_dot64(p_sub(f0->target->p, et0), perp);
                    int64_t dy0 = p_dot(p_sub(f0->target->p, et0), s);
                    if ((dx0 == 0) ? (dy0 < 0) : ((dx0 < 0) && rat_cmp(rat_make(dy0, dx0), rat_make(dy, dx)) >= 0)) {
                        et0 = f0->target->p;
                        dx = p_dot64(p_sub(et1, et0), perp);
                        e0 = (e0 == start0) ? NULL : f0;
                        continue;
                    }
                }
            }
            if (e1 && e1->target != stop1) {
                he *f1 = e1->reverse->next;
                if (f1->copy > c->merge_stamp) {
                    hp32 d1 = p_sub(f1->target->p, et1);
                    if (p_dot64(d1, normal) == 0) {
                        int64_t dx1 = p_dot64(d1, perp);
                        int64_t dy1 = p_dot(d1, s);
                        int64_t dxn = p_dot64(p_sub(f1->target->p, et0), perp);
                        if (dxn > 0 &&
                            ((dx1 == 0) ? (dy1 < 0) : ((dx1 < 0) && rat_cmp(rat_make(dy1, dx1), rat_make(dy, dx)) > 0))) {
                            e1 = f1;
                            et1 = e1->target->p;
                            dx = dxn;
                            continue;
                        }
                    }
                }
            }
            break;
        }
    } else if (dx < 0) {
        for (;;) {
            int64_t dy = p_dot(p_sub(et1, et0), s);
            if (e1 && e1->target != stop1) {
                he *f1 = e1->prev->reverse;
                if (f1->copy > c->merge_stamp) {
                    int64_t dx1 = p_dot64(p_sub(f1->target->p, et1), perp);
                    int64_t dy1 = p_dot(p_sub(f1->target->p, et1), s);
                    if ((dx1 == 0) ? (dy1 > 0) : ((dx1 < 0) && rat_cmp(rat_make(dy1, dx1), rat_make(dy, dx)) <= 0)) {
                        et1 = f1->target->p;
                        dx = p_dot64(p_sub(et1, et0), perp);
                        e1 = (e1 == start1) ? NULL : f1;
                        continue;
                    }
                }
            }
            if (e0 && e0->target != stop0) {
                he *f0 = e0->reverse->prev;
                if (f0->copy > c->merge_stamp) {
                    hp32 d0 = p_sub(f0->target->p, et0);
                    if (p_dot64(d0, normal) == 0) {
                        int64_t dx0 = p_dot64(d0, perp);
                        int64_t dy0 = p_dot(d0, s);
                        int64_t dxn = p_dot64(p_sub(et1, f0->target->p), perp);
                        if (dxn < 0 &&
                            ((dx0 == 0) ? (dy0 > 0) : ((dx0 < 0) && rat_cmp(rat_make(dy0, dx0), rat_make(dy, dx)) < 0))) {
                            e0 = f0;
                            et0 = e0->target->p;
                            dx = dxn;
                            continue;
                        }
                    }
                }
            }
            break;
        }
    }
    *pe0 = e0;
    *pe1 = e1;
}

/* mergeProjection (:1024-1207): joins the 2-D (x, y) projection rings of two hulls separated
 * along x and returns the lower bridge (c0, c1); false when h1 degenerates to a vertical segment
 * directly above h0's last point. */
static int merge_projection(hhull *h0, hhull *h1, hv **c0, hv **c1) {
    hv *v0 = h0->maxYx, *v1 = h1->minYx;
    if (v0->p.x == v1->p.x && v0->p.y == v1->p.y) {
        hv *v1p = v1->prev;
        if (v1p == v1) {
            *c0 = v0;
            if (v1->edges) v1 = v1->edges->target;
            *c1 = v1;
            return 0;
        }
        hv *v1n = v1->next;
        v1p->next = v1n;
        v1n->prev = v1p;
        if (v1 == h1->minXy) {
            if (v1n->p.x < v1p->p.x || (v1n->p.x == v1p->p.x && v1n->p.y < v1p->p.y)) h1->minXy = v1n;
            else h1->minXy = v1p;
        }
        if (v1 == h1->maxXy) {
            if (v1n->p.x > v1p->p.x || (v1n->p.x == v1p->p.x && v1n->p.y > v1p->p.y)) h1->maxXy = v1n;
            else h1->maxXy = v1p;
        }
    }

    v0 = h0->maxXy;
    v1 = h1->maxXy;
    hv *v00 = NULL, *v10 = NULL;
    int32_t sign = 1;
    for (int side = 0; side <= 1; side++) {
        int32_t dx = (v1->p.x - v0->p.x) * sign;
        if (dx > 0) {
            for (;;) {
                int32_t dy = v1->p.y - v0->p.y;
                hv *w0 = side ? v0->next : v0->prev;
                if (w0 != v0) {
                    int32_t dx0 = (w0->p.x - v0->p.x) * sign;
                    int32_t dy0 = w0->p.y - v0->p.y;
                    if (dy0 <= 0 && (dx0 == 0 || (dx0 < 0 && (int64_t)dy0 * dx <= (int64_t)dy * dx0))) {
                        v0 = w0;
                        dx = (v1->p.x - v0->p.x) * sign;
                        continue;
                    }
                }
                hv *w1 = side ? v1->next : v1->prev;
                if (w1 != v1) {
                    int32_t dx1 = (w1->p.x - v1->p.x) * sign;
                    int32_t dy1 = w1->p.y - v1->p.y;
                    int32_t dxn = (w1->p.x - v0->p.x) * sign;
                    if (dxn > 0 && dy1 < 0 && (dx1 == 0 || (dx1 < 0 && (int64_t)dy1 * dx < (int64_t)dy * dx1))) {
                        v1 = w1;
                        dx = dxn;
                        continue;
                    }
                }
                break;
            }
        } else if (dx < 0) {
            for (;;) {
                int32_t dy = v1->p.y - v0->p.y;
                hv *w1 = side ? v1->prev : v1->next;
                if (w1 != v1) {
                    int32_t dx1 = (w1->p.x - v1->p.x) * sign;
                    int32_t dy1 = w1->p.y - v1->p.y;
                    if (dy1 >= 0 && (dx1 == 0 || (dx1 < 0 && (int64_t)dy1 * dx <= (int64_t)dy * dx1))) {
                        v1 = w1;
                        dx = (v1->p.x - v0->p.x) * sign;
                        continue;
                    }
                }
                hv *w0 = side ? v0->prev : v0->next;
                if (w0 != v0) {
                    int32_t dx0 = (w0->p.x - v0->p.x) * sign;
                    int32_t dy0 = w0->p.y - v0->p.y;
                    int32_t dxn = (v1->p.x - w0->p.x) * sign;
                    if (dxn < 0 && dy0 > 0 && (dx0 == 0 || (dx0 < 0 && (int64_t)dy0 * dx < (int64_t)dy * dx0))) {
                        v0 = w0;
                        dx = dxn;
                        continue;
                    }
                }
                break;
            }
        } else {
            int32_t x = v0->p.x;
            int32_t y0 = v0->p.y;
            hv *w0 = v0, *t;
            while ((t = side ? w0->next : w0->prev) != v0 && t->p.x == x && t->p.y <= y0) {
                w0 = t;
                y0 = t->p.y;
            }
            v0 = w0;
            int32_t y1 = v1->p.y;
            hv *w1 = v1;
            while ((t = side ? w1->prev : w1->next) != v1 && t->p.x == x && t->p.y >= y1) {
                w1 = t;
                y1 = t->p.y;
            }
            v1 = w1;
        }
        if (side == 0) {
            v00 = v0;
            v10 = v1;
            v0 = h0->minXy;
            v1 = h1->minXy;
            sign = -1;
        }
    }
    v0->prev = v1;
    v1->next = v0;
    v00->next = v10;
    v10->prev = v00;
    if (h1->minXy->p.x < h0->minXy->p.x) h0->minXy = h1->minXy;
    if (h1->maxXy->p.x >= h0->maxXy->p.x) h0->maxXy = h1->maxXy;
    h0->maxYx = h1->maxYx;
    *c0 = v00;
    *c1 = v10;
    return 1;
}

/* merge (:1651-1936): wraps the band of triangles that joins the two hulls, removing the edges of
 * each half that the band hides */
static void hull_merge(hctx *c, hhull *h0, hhull *h1) {
    if (!h1->maxXy) return;
    if (!h0->maxXy) { *h0 = *h1; return; }
    c->merge_stamp--;
    hv *c0 = NULL, *c1 = NULL;
    he *toPrev0 = NULL, *firstNew0 = NULL, *pendingHead0 = NULL, *pendingTail0 = NULL;
    he *toPrev1 = NULL, *firstNew1 = NULL, *pendingHead1 = NULL, *pendingTail1 = NULL;
    hp32 prevPoint;
    const hp32 down = {0, 0, -1};

    if (merge_projection(h0, h1, &c0, &c1)) {
        hp32 s = v_sub(c1, c0);
        hp64 normal = p_cross(down, s);
        hp64 t = p_cross64(s, normal);
        he *e = c0->edges, *start0 = NULL;
        if (e) {
            do {
                int64_t dot = p_dot64(v_sub(e->target, c0), normal);
                if (dot == 0 && p_dot64(v_sub(e->target, c0), t) > 0) {
                    if (!start0 || get_orientation(start0, e, s, down) == OR_CW) start0 = e;
                }
                e = e->next;
            } while (e != c0->edges);
        }
        e = c1->edges;
        he *start1 = NULL;
        if (e) {
            do {
                int64_t dot = p_dot64(v_sub(e->target, c1), normal);
                if (dot == 0 && p_dot64(v_sub(e->target, c1), t) > 0) {
                    if (!start1 || get_orientation(start1, e, s, down) == OR_CCW) start1 = e;
                }
                e = e->next;
            } while (e != c1->edges);
        }
        if (start0 || start1) {
            find_edge_for_coplanar_faces(c, c0, c1, &start0, &start1, NULL, NULL);
            if (start0) c0 = start0->target;
            if (start1) c1 = start1->target;
        }
        prevPoint = c1->p;
        prevPoint.z++;
    } else {
        prevPoint = c1->p;
        prevPoint.x++;
    }

    hv *first0 = c0, *first1 = c1;
    int firstRun = 1;
    for (;;) {
        if (c->fail) return;
        hp32 s = v_sub(c1, c0);
        hp32 r = p_sub(prevPoint, c0->p);
        hp64 rxs = p_cross(r, s);
        hp64 sxrxs = p_cross64(s, rxs);
        rat64 minCot0 = rat_make(0, 0), minCot1 = rat_make(0, 0);
        he *min0 = find_max_angle(c, 0, c0, s, rxs, sxrxs, &minCot0);
        he *min1 = find_max_angle(c, 1, c1, s, rxs, sxrxs, &minCot1);
        if (!min0 && !min1) {
            he *e = new_edge_pair(c, c0, c1);
            if (!e) return;
            link_edges(e, e);
            c0->edges = e;
            e = e->reverse;
            link_edges(e, e);
            c1->edges = e;
            return;
        } else {
            int cmp = !min0 ? 1 : !min1 ? -1 : rat_cmp(minCot0, minCot1);
            if (firstRun || ((cmp >= 0) ? !rat_is_neg_inf(minCot1) : !rat_is_neg_inf(minCot0))) {
                he *e = new_edge_pair(c, c0, c1);
                if (!e) return;
                if (pendingTail0) pendingTail0->prev = e;
                else pendingHead0 = e;
                e->next = pendingTail0;
                pendingTail0 = e;
                e = e->reverse;
                if (pendingTail1) pendingTail1->next = e;
                else pendingHead1 = e;
                e->prev = pendingTail1;
                pendingTail1 = e;
            }
            he *e0 = min0, *e1 = min1;
            if (cmp == 0) find_edge_for_coplanar_faces(c, c0, c1, &e0, &e1, NULL, NULL);
            if (cmp >= 0 && e1) {
                if (toPrev1) {
                    for (he *e = toPrev1->next, *n = NULL; e != min1; e = n) {
                        n = e->next;
                        remove_edge_pair(c, e);
                    }
                }
                if (pendingTail1) {
                    if (toPrev1) {
                        link_edges(toPrev1, pendingHead1);
                    } else {
                        link_edges(min1->prev, pendingHead1);
                        firstNew1 = pendingHead1;
                    }
                    link_edges(pendingTail1, min1);
                    pendingHead1 = NULL;
                    pendingTail1 = NULL;
                } else if (!toPrev1) {
                    firstNew1 = min1;
                }
                prevPoint = c1->p;
                c1 = e1->target;
                toPrev1 = e1->reverse;
            }
            if (cmp <= 0 && e0) {
                if (toPrev0) {
                    for (he *e = toPrev0->prev, *n = NULL; e != min0; e = n) {
                        n = e->prev;
                        remove_edge_pair(c, e);
                    }
                }
                if (pendingTail0) {
                    if (toPrev0) {
                        link_edges(pendingHead0, toPrev0);
                    } else {
                        link_edges(pendingHead0, min0->next);
                        firstNew0 = pendingHead0;
                    }
                    link_edges(min0, pendingTail0);
                    pendingHead0 = NULL;
                    pendingTail0 = NULL;
                } else if (!toPrev0) {
                    firstNew0 = min0;
                }
                prevPoint = c0->p;
                c0 = e0->target;
                toPrev0 = e0->reverse;
            }
        }
        if (c0 == first0 && c1 == first1) {
            if (toPrev0 == NULL) {
                link_edges(pendingHead0, pendingTail0);
                c0->edges = pendingTail0;
            } else {
                for (he *e = toPrev0->prev, *n = NULL; e != firstNew0; e = n) {
                    n = e->prev;
                    remove_edge_pair(c, e);
                }
                if (pendingTail0) {
                    link_edges(pendingHead0, toPrev0);
                    link_edges(firstNew0, pendingTail0);
                }
            }
            if (toPrev1 == NULL) {
                link_edges(pendingTail1, pendingHead1);
                c1->edges = pendingTail1;
            } else {
                for (he *e = toPrev1->next, *n = NULL; e != firstNew1; e = n) {
                    n = e->next;
                    remove_edge_pair(c, e);
                }
                if (pendingTail1) {
                    link_edges(toPrev1, pendingHead1);
                    link_edges(pendingTail1, firstNew1);
                }
            }
            return;
        }
        firstRun = 0;
    }
}

/* computeInternal (:1209-1324): hull of the sorted points [start, end) */
static void compute_internal(hctx *c, int start, int end, hhull *result) {
    int n = end - start;
    if (c->fail) return;
    if (n == 0) {
        result->minXy = result->maxXy = result->minYx = result->maxYx = NULL;
        return;
    }
    if (n == 2) {
        hv *v = &c->verts[start];
        hv *w = v + 1;
        if (!p_eq(v->p, w->p)) {
            int32_t dx = v->p.x - w->p.x;
            int32_t dy = v->p.y - w->p.y;
            if (dx == 0 && dy == 0) {
                if (v->p.z > w->p.z) { hv *t = w; w = v; v = t; }
                v->next = v;
                v->prev = v;
                result->minXy = result->maxXy = result->minYx = result->maxYx = v;
            } else {
                v->next = w; v->prev = w;
                w->next = v; w->prev = v;
                if (dx < 0 || (dx == 0 && dy < 0)) { result->minXy = v; result->maxXy = w; }
                else { result->minXy = w; result->maxXy = v; }
                if (dy < 0 || (dy == 0 && dx < 0)) { result->minYx = v; result->maxYx = w; }
                else { result->minYx = w; result->maxYx = v; }
            }
            he *e = new_edge_pair(c, v, w);
            if (!e) return;
            link_edges(e, e);
            v->edges = e;
            e = e->reverse;
            link_edges(e, e);
            w->edges = e;
            return;
        }
        /* two equal points: one vertex */
    }
    if (n <= 2) {
        hv *v = &c->verts[start];
        v->edges = NULL;
        v->next = v;
        v->prev = v;
        result->minXy = result->maxXy = result->minYx = result->maxYx = v;
        return;
    }
    int split0 = start + n / 2;
    hp32 p = c->verts[split0 - 1].p;
    int split1 = split0;
    while (split1 < end && p_eq(c->verts[split1].p, p)) split1++;
    compute_internal(c, start, split0, result);
    hhull hull1;
    compute_internal(c, split1, end, &hull1);
    if (c->fail) return;
    hull_merge(c, result, &hull1);
}

/* b3PointCmp (:1938-1941) and quickSortInternal (b3AlignedObjectArray.h:330-357) */
static int point_less(hp32 p, hp32 q) {
    return p.y < q.y || (p.y == q.y && (p.x < q.x || (p.x == q.x && p.z < q.z)));
}
static void quick_sort(hp32 *a, int lo, int hi) {
    int i = lo, j = hi;
    hp32 x = a[(lo + hi) / 2];
    do {
        while (point_less(a[i], x)) i++;
        while (point_less(x, a[j])) j--;
        if (i <= j) {
            hp32 t = a[i]; a[i] = a[j]; a[j] = t;
            i++;
            j--;
        }
    } while (i <= j);
    if (lo < j) quick_sort(a, lo, j);
    if (i < hi) quick_sort(a, i, hi);
}

static int max_axis3(const float *v) { return v[0] < v[1] ? (v[1] < v[2] ? 2 : 1) : (v[0] < v[2] ? 2 : 0); }
static int min_axis3(const float *v) { return v[0] < v[1] ? (v[0] < v[2] ? 0 : 2) : (v[1] < v[2] ? 1 : 2); }

/* Output of b3ConvexHullComputer::compute with shrink 0. */
typedef struct { int next, reverse, target; } hout_edge;
typedef struct {
    float *verts;  /* 3 per vertex */
    int nv;
    hout_edge *edges;
    int ne;
    int *faces;    /* one edge index per face */
    int nf;
} hout;

static void hout_free(hout *o) {
    free(o->verts);
    free(o->edges);
    free(o->faces);
    memset(o, 0, sizeof(*o));
}

/* returns 0 on success, -1 on allocation failure */
static int hull_compute(const float *xyz, int count, hout *out) {
    memset(out, 0, sizeof(*out));
    if (count <= 0) return 0;
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < count; i++)
        for (int k = 0; k < 3; k++) {
            float v = xyz[3 * i + k];
            if (v < mn[k]) mn[k] = v;  /* b3Vector3::setMin / setMax */
            if (mx[k] < v) mx[k] = v;
        }
    float s[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    int maxAxis = max_axis3(s), minAxis = min_axis3(s);
    if (minAxis == maxAxis) minAxis = (maxAxis + 1) % 3;
    int medAxis = 3 - maxAxis - minAxis;
    const float inv10216 = 1.0f / 10216.0f;  /* s /= 10216 multiplies by the reciprocal */
    for (int k = 0; k < 3; k++) s[k] = s[k] * inv10216;
    if (((medAxis + 1) % 3) != maxAxis)
        for (int k = 0; k < 3; k++) s[k] = s[k] * -1.0f;
    float scaling[3] = {s[0], s[1], s[2]};
    for (int k = 0; k < 3; k++)
        if (s[k] != 0) s[k] = 1.0f / s[k];
    float center[3];
    for (int k = 0; k < 3; k++) center[k] = (mn[k] + mx[k]) * 0.5f;

    hp32 *pts = (hp32 *)malloc(sizeof(hp32) * (size_t)count);
    if (!pts) return -1;
    for (int i = 0; i < count; i++) {
        float p[3];
        for (int k = 0; k < 3; k++) p[k] = (xyz[3 * i + k] - center[k]) * s[k];
        pts[i].x = (int32_t)p[medAxis];
        pts[i].y = (int32_t)p[maxAxis];
        pts[i].z = (int32_t)p[minAxis];
    }
    if (count > 1) quick_sort(pts, 0, count - 1);

    hctx c;
    memset(&c, 0, sizeof(c));
    c.chunk_cap = 6 * count + 16;
    c.verts = (hv *)calloc((size_t)count, sizeof(hv));
    if (!c.verts) { free(pts); return -1; }
    for (int i = 0; i < count; i++) {
        c.verts[i].p = pts[i];
        c.verts[i].copy = -1;
    }
    free(pts);
    c.merge_stamp = -3;
    hhull hull;
    compute_internal(&c, 0, count, &hull);
    int rc = c.fail ? -1 : 0;
    hv *vertexList = hull.minXy;

    /* output (:2640-2745): vertices in breadth-first order from vertexList; per vertex its edges
     * in ring order, each edge pair numbered when first met; faces traced through reverse->prev */
    int vcap = count, ecap = 16, fcap = 16;
    hv **old = NULL;
    if (!rc) {
        old = (hv **)malloc(sizeof(hv *) * (size_t)vcap);
        out->verts = (float *)malloc(sizeof(float) * 3 * (size_t)vcap);
        out->edges = (hout_edge *)malloc(sizeof(hout_edge) * (size_t)ecap);
        out->faces = (int *)malloc(sizeof(int) * (size_t)fcap);
        if (!old || !out->verts || !out->edges || !out->faces) rc = -1;
    }
    int nold = 0;
    if (!rc && vertexList) {
        vertexList->copy = nold;
        old[nold++] = vertexList;
    }
    int copied = 0;
    while (!rc && copied < nold) {
        hv *v = old[copied];
        float p[3];
        p[medAxis] = (float)v->p.x;
        p[maxAxis] = (float)v->p.y;
        p[minAxis] = (float)v->p.z;
        for (int k = 0; k < 3; k++) out->verts[3 * out->nv + k] = p[k] * scaling[k] + center[k];
        out->nv++;
        he *firstEdge = v->edges;
        if (firstEdge) {
            int firstCopy = -1, prevCopy = -1;
            he *e = firstEdge;
            do {
                if (e->copy < 0) {
                    if (out->ne + 2 > ecap) {
                        ecap *= 2;
                        hout_edge *ne = (hout_edge *)realloc(out->edges, sizeof(hout_edge) * (size_t)ecap);
                        if (!ne) { rc = -1; break; }
                        out->edges = ne;
                    }
                    int si = out->ne;
                    out->ne += 2;
                    e->copy = si;
                    e->reverse->copy = si + 1;
                    out->edges[si].reverse = 1;
                    out->edges[si + 1].reverse = -1;
                    int tv = e->target->copy;
                    if (tv < 0) {
                        tv = nold;
                        e->target->copy = tv;
                        old[nold++] = e->target;
                    }
                    out->edges[si].target = tv;
                    out->edges[si + 1].target = copied;
                }
                if (prevCopy >= 0) out->edges[e->copy].next = prevCopy - e->copy;
                else firstCopy = e->copy;
                prevCopy = e->copy;
                e = e->next;
            } while (e != firstEdge);
            if (rc) break;
            out->edges[firstCopy].next = prevCopy - firstCopy;
        }
        copied++;
    }
    for (int i = 0; !rc && i < copied; i++) {
        hv *v = old[i];
        he *firstEdge = v->edges;
        if (!firstEdge) continue;
        he *e = firstEdge;
        do {
            if (e->copy >= 0) {
                if (out->nf == fcap) {
                    fcap *= 2;
                    int *nf = (int *)realloc(out->faces, sizeof(int) * (size_t)fcap);
                    if (!nf) { rc = -1; break; }
                    out->faces = nf;
                }
                out->faces[out->nf++] = e->copy;
                he *f = e;
                do {
                    f->copy = -1;
                    f = f->reverse->prev;
                } while (f != e);
            }
            e = e->next;
        } while (e != firstEdge);
    }
    free(old);
    while (c.chunks) {
        edge_chunk *k = c.chunks;
        c.chunks = k->prev;
        free(k);
    }
    free(c.verts);
    if (rc) hout_free(out);
    return rc;
}

/* ------------------------------------------------------------------ float helpers (b3Vector3, scalar build) */
typedef struct { float x, y, z; } f3;
static f3 f3_make(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static f3 f3_sub(f3 a, f3 b) { return f3_make(a.x - b.x, a.y - b.y, a.z - b.z); }
static f3 f3_add(f3 a, f3 b) { return f3_make(a.x + b.x, a.y + b.y, a.z + b.z); }
static f3 f3_scale(f3 a, float s) { return f3_make(a.x * s, a.y * s, a.z * s); }
static float f3_dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static f3 f3_cross(f3 a, f3 b) { return f3_make(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
/* normalize(): *this /= length(), i.e. times 1 / sqrt(length2) */
static f3 f3_normalized(f3 a) { return f3_scale(a, 1.0f / sqrtf(f3_dot(a, a))); }
static f3 f3_at(const float *v, int i) { return f3_make(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }

/* b3PlaneSpace1 (b3Vector3.h:1184-1212) */
static void plane_space1(f3 n, f3 *p, f3 *q) {
    if (fabsf(n.z) > 0.7071067811865475244008443621048490f) {
        float a = n.y * n.y + n.z * n.z;
        float k = 1.0f / sqrtf(a);
        *p = f3_make(0.f, -n.z * k, n.y * k);
        *q = f3_make(a * k, -n.x * p->z, n.x * p->y);
    } else {
        float a = n.x * n.x + n.y * n.y;
        float k = 1.0f / sqrtf(a);
        *p = f3_make(-n.y * k, n.x * k, 0.f);
        *q = f3_make(-n.z * p->y, n.z * p->x, a * k);
    }
}

typedef struct { f3 p; int org; float angle; } gpoint;

/* b3AngleCompareFunc: angle, then distance to the anchor, then original index (a total order) */
static f3 g_anchor;
static int gpoint_cmp(const void *pa, const void *pb) {
    const gpoint *a = (const gpoint *)pa, *b = (const gpoint *)pb;
    if (a->angle != b->angle) return a->angle < b->angle ? -1 : 1;
    float al = f3_dot(f3_sub(a->p, g_anchor), f3_sub(a->p, g_anchor));
    float bl = f3_dot(f3_sub(b->p, g_anchor), f3_sub(b->p, g_anchor));
    if (al != bl) return al < bl ? -1 : 1;
    return a->org < b->org ? -1 : a->org > b->org ? 1 : 0;
}

/* b3GrahamScanConvexHull2D; returns the hull size written to hull[] */
static int graham_scan(gpoint *pts, int n, gpoint *hull, f3 normalAxis) {
    f3 axis0, axis1;
    plane_space1(normalAxis, &axis0, &axis1);
    int nh = 0;
    if (n <= 1) {
        for (int i = 0; i < n; i++) hull[nh++] = pts[0];
        return nh;
    }
    for (int i = 0; i < n; i++) {
        float projL = f3_dot(pts[i].p, axis0);
        float projR = f3_dot(pts[0].p, axis0);
        if (projL < projR) { gpoint t = pts[0]; pts[0] = pts[i]; pts[i] = t; }
    }
    pts[0].angle = -1e30f;
    for (int i = 1; i < n; i++) {
        f3 ar = f3_sub(pts[i].p, pts[0].p);
        pts[i].angle = f3_dot(f3_cross(axis0, ar), normalAxis) / sqrtf(f3_dot(ar, ar));
    }
    g_anchor = pts[0].p;
    qsort(pts + 1, (size_t)(n - 1), sizeof(gpoint), gpoint_cmp);
    int i;
    for (i = 0; i < 2; i++) hull[nh++] = pts[i];
    for (; i != n; i++) {
        int isConvex = 0;
        while (!isConvex && nh > 1) {
            f3 a = hull[nh - 2].p, b = hull[nh - 1].p;
            isConvex = f3_dot(f3_cross(f3_sub(a, b), f3_sub(a, pts[i].p)), normalAxis) > 0;
            if (!isConvex) nh--;
            else hull[nh++] = pts[i];
        }
    }
    return nh;
}

typedef struct { int *idx; int n; float plane[4]; } pface;

static int is_almost_zero(f3 v) {
    return !(fabsf(v.x) > 1e-6 || fabsf(v.y) > 1e-6 || fabsf(v.z) > 1e-6);
}

/* b3ConvexUtility::initializePolyhedralFeatures (merge = true) + initialize()'s unique edges +
 * registerConvexHullShape's vertex-mean local centre.  Outputs in caller buffers; counts4 in:
 * capacities (verts, faces, indices, edges), out: sizes.  Returns 0, 1 (a buffer too small) or
 * -1 (allocation failure). */
int oracle_hull(const float *xyz, int n, float *verts_out, float *planes_out, int *face_counts_out,
                int *indices_out, float *edges_out, float *center_out, int *counts4) {
    hout h;
    if (hull_compute(xyz, n, &h) != 0) return -1;
    const int nf = h.nf;
    pface *tmp = (pface *)calloc((size_t)(nf > 0 ? nf : 1), sizeof(pface));
    int *todo = (int *)malloc(sizeof(int) * (size_t)(nf > 0 ? nf : 1));
    int *group = (int *)malloc(sizeof(int) * (size_t)(nf > 0 ? nf : 1));
    pface *faces = (pface *)calloc((size_t)(nf > 0 ? nf : 1), sizeof(pface));
    int nfaces = 0, rc = 0;
    if (!tmp || !todo || !group || !faces) rc = -1;
    /* triangle (polygon) faces of the hull, normals from their first two edges (:47-98) */
    for (int i = 0; !rc && i < nf; i++) {
        const int first = h.faces[i];
        int e = first, cnt = 0;
        do {
            cnt++;
            int r = e + h.edges[e].reverse;
            e = r + h.edges[r].next;
        } while (e != first);
        tmp[i].idx = (int *)malloc(sizeof(int) * (size_t)cnt);
        if (!tmp[i].idx) { rc = -1; break; }
        f3 ed[2];
        int numEdges = 0;
        e = first;
        do {
            int r = e + h.edges[e].reverse;
            int src = h.edges[r].target, targ = h.edges[e].target;
            tmp[i].idx[tmp[i].n++] = src;
            f3 ne = f3_normalized(f3_sub(f3_at(h.verts, targ), f3_at(h.verts, src)));
            if (numEdges < 2) ed[numEdges++] = ne;
            e = r + h.edges[r].next;
        } while (e != first);
        f3 nrm = f3_make(0, 0, 0);
        float planeEq = 1e30f;
        if (numEdges == 2) nrm = f3_normalized(f3_cross(ed[0], ed[1]));
        for (int v = 0; v < tmp[i].n; v++) {
            float eq = f3_dot(f3_at(h.verts, tmp[i].idx[v]), nrm);
            if (planeEq > eq) planeEq = eq;
        }
        tmp[i].plane[0] = nrm.x;
        tmp[i].plane[1] = nrm.y;
        tmp[i].plane[2] = nrm.z;
        tmp[i].plane[3] = -planeEq;
    }
    /* coplanar welding (:100-244) */
    int ntodo = 0;
    for (int i = 0; !rc && i < nf; i++) todo[ntodo++] = i;
    while (!rc && ntodo) {
        int ng = 0;
        int refFace = todo[ntodo - 1];
        group[ng++] = refFace;
        ntodo--;
        f3 nA = f3_make(tmp[refFace].plane[0], tmp[refFace].plane[1], tmp[refFace].plane[2]);
        for (int j = ntodo - 1; j >= 0; j--) {
            int i = todo[j];
            f3 nB = f3_make(tmp[i].plane[0], tmp[i].plane[1], tmp[i].plane[2]);
            if (f3_dot(nA, nB) > 0.999f) {
                group[ng++] = i;
                /* b3AlignedObjectArray::remove (b3AlignedObjectArray.h:489-497): the first
                 * occurrence is swapped with the last element, then popped */
                for (int k = 0; k < ntodo; k++)
                    if (todo[k] == i) {
                        todo[k] = todo[ntodo - 1];
                        ntodo--;
                        break;
                    }
            }
        }
        int did_merge = 0;
        if (ng > 1) {
            int cap = 0;
            for (int g = 0; g < ng; g++) cap += tmp[group[g]].n;
            gpoint *org = (gpoint *)malloc(sizeof(gpoint) * (size_t)cap);
            gpoint *hull2 = (gpoint *)malloc(sizeof(gpoint) * (size_t)(2 * cap + 2));
            if (!org || !hull2) { free(org); free(hull2); rc = -1; break; }
            int norg = 0;
            f3 avg = f3_make(0, 0, 0);
            for (int g = 0; g < ng; g++) {
                const pface *f = &tmp[group[g]];
                avg = f3_add(avg, f3_make(f->plane[0], f->plane[1], f->plane[2]));
                for (int k = 0; k < f->n; k++) {
                    int o = f->idx[k], found = 0;
                    for (int q = 0; q < norg; q++)
                        if (org[q].org == o) { found = 1; break; }
                    if (!found) {
                        org[norg].p = f3_at(h.verts, o);
                        org[norg].org = o;
                        org[norg].angle = 0.f;
                        norg++;
                    }
                }
            }
            avg = f3_normalized(avg);
            int nh = graham_scan(org, norg, hull2, avg);
            pface comb;
            memcpy(comb.plane, tmp[group[0]].plane, sizeof(comb.plane));
            comb.idx = (int *)malloc(sizeof(int) * (size_t)(nh > 0 ? nh : 1));
            comb.n = 0;
            if (!comb.idx) { free(org); free(hull2); rc = -1; break; }
            for (int k = 0; k < nh; k++) {
                comb.idx[comb.n++] = hull2[k].org;
                for (int q = 0; q < norg; q++)
                    if (org[q].org == hull2[k].org) { org[q].org = -1; break; }
            }
            int reject = 0;
            for (int q = 0; q < norg && !reject; q++) {
                if (org[q].org == -1) continue;
                for (int j = 0; j < nf && !reject; j++) {
                    int in_group = 0;
                    for (int g = 0; g < ng; g++)
                        if (group[g] == j) { in_group = 1; break; }
                    if (in_group) continue;
                    for (int v = 0; v < tmp[j].n; v++)
                        if (tmp[j].idx[v] == org[q].org) { reject = 1; break; }
                }
            }
            free(org);
            free(hull2);
            if (!reject) {
                did_merge = 1;
                faces[nfaces++] = comb;
            } else {
                free(comb.idx);
            }
        }
        if (!did_merge) {
            for (int g = 0; g < ng; g++) {
                pface f = tmp[group[g]];
                f.idx = (int *)malloc(sizeof(int) * (size_t)(f.n > 0 ? f.n : 1));
                if (!f.idx) { rc = -1; break; }
                memcpy(f.idx, tmp[group[g]].idx, sizeof(int) * (size_t)f.n);
                faces[nfaces++] = f;
            }
        }
    }
    /* unique edge directions (initialize(), :329-375): v[min] - v[max] normalised, kept unless
     * parallel or anti-parallel to an earlier one within 1e-6 per component */
    int nidx = 0, nedges = 0, ecap = 16;
    f3 *edges = rc ? NULL : (f3 *)malloc(sizeof(f3) * (size_t)ecap);
    if (!rc && !edges) rc = -1;
    for (int i = 0; !rc && i < nfaces; i++) {
        nidx += faces[i].n;
        for (int j = 0; j < faces[i].n; j++) {
            int a = faces[i].idx[j], b = faces[i].idx[(j + 1) % faces[i].n];
            int v0 = a > b ? a : b, v1 = a > b ? b : a;
            f3 e = f3_normalized(f3_sub(f3_at(h.verts, v1), f3_at(h.verts, v0)));
            int found = 0;
            for (int p = 0; p < nedges; p++)
                if (is_almost_zero(f3_sub(edges[p], e)) || is_almost_zero(f3_add(edges[p], e))) { found = 1; break; }
            if (!found) {
                if (nedges == ecap) {
                    ecap *= 2;
                    f3 *ne = (f3 *)realloc(edges, sizeof(f3) * (size_t)ecap);
                    if (!ne) { rc = -1; break; }
                    edges = ne;
                }
                edges[nedges++] = e;
            }
        }
    }
    if (!rc) {
        int fits = counts4[0] >= h.nv && counts4[1] >= nfaces && counts4[2] >= nidx && counts4[3] >= nedges;
        counts4[0] = h.nv;
        counts4[1] = nfaces;
        counts4[2] = nidx;
        counts4[3] = nedges;
        if (!fits) {
            rc = 1;
        } else {
            memcpy(verts_out, h.verts, sizeof(float) * 3 * (size_t)h.nv);
            int off = 0;
            for (int i = 0; i < nfaces; i++) {
                memcpy(planes_out + 4 * i, faces[i].plane, sizeof(float) * 4);
                face_counts_out[i] = faces[i].n;
                memcpy(indices_out + off, faces[i].idx, sizeof(int) * (size_t)faces[i].n);
                off += faces[i].n;
            }
            for (int i = 0; i < nedges; i++) {
                edges_out[3 * i] = edges[i].x;
                edges_out[3 * i + 1] = edges[i].y;
                edges_out[3 * i + 2] = edges[i].z;
            }
            /* registerConvexHullShape (b3GpuNarrowPhase.cpp:326-331): localCenter = vertex mean */
            f3 cm = f3_make(0, 0, 0);
            for (int i = 0; i < h.nv; i++) cm = f3_add(cm, f3_at(h.verts, i));
            cm = f3_scale(cm, 1.f / (float)h.nv);
            center_out[0] = cm.x;
            center_out[1] = cm.y;
            center_out[2] = cm.z;
        }
    }
    free(edges);
    for (int i = 0; tmp && i < nf; i++) free(tmp[i].idx);
    for (int i = 0; faces && i < nfaces; i++) free(faces[i].idx);
    free(tmp);
    free(faces);
    free(todo);
    free(group);
    hout_free(&h);
    return rc;
}

/* ------------------------------------------------------------------ body registration */
/* b3Matrix3x3::setRotation(quaternion) (b3Matrix3x3.h:208-226) */
static void quat_to_mat(const float q[4], float m[3][3]) {
    float x = q[0], y = q[1], z = q[2], w = q[3];
    float d = x * x + y * y + z * z + w * w;
    float s = 2.0f / d;
    float xs = x * s, ys = y * s, zs = z * s;
    float wx = w * xs, wy = w * ys, wz = w * zs;
    float xx = x * xs, xy = x * ys, xz = x * zs;
    float yy = y * ys, yz = y * zs, zz = z * zs;
    m[0][0] = 1.0f - (yy + zz); m[0][1] = xy - wz; m[0][2] = xz + wy;
    m[1][0] = xy + wz; m[1][1] = 1.0f - (xx + zz); m[1][2] = yz - wx;
    m[2][0] = xz - wy; m[2][1] = yz + wx; m[2][2] = 1.0f - (xx + yy);
}

/* registerPhysicsInstance + registerRigidBody for one body: the body record (80 B layout of
 * b3RigidBodyData) and the inertia record (b3InertiaData, 96 B).  local_min / local_max: the
 * shape's local AABB.  Returns 0. */
int oracle_register_body(float mass, const float pos[3], const float orn[4], int collidable, const float local_min[3],
                         const float local_max[3], float *body_out, float *inertia_out) {
    float m[3][3];
    quat_to_mat(orn, m);
    /* b3TransformAabb(localMin, localMax, margin 0.01, t) (b3AabbUtil.h:146-159) */
    const float margin = 0.01f;
    f3 lmin = f3_make(local_min[0], local_min[1], local_min[2]);
    f3 lmax = f3_make(local_max[0], local_max[1], local_max[2]);
    f3 he = f3_scale(f3_sub(lmax, lmin), 0.5f);
    he = f3_add(he, f3_make(margin, margin, margin));
    f3 lc = f3_scale(f3_add(lmax, lmin), 0.5f);
    f3 center = f3_add(f3_make(f3_dot(f3_make(m[0][0], m[0][1], m[0][2]), lc),
                               f3_dot(f3_make(m[1][0], m[1][1], m[1][2]), lc),
                               f3_dot(f3_make(m[2][0], m[2][1], m[2][2]), lc)),
                       f3_make(pos[0], pos[1], pos[2]));
    f3 ext = f3_make(f3_dot(f3_make(fabsf(m[0][0]), fabsf(m[0][1]), fabsf(m[0][2])), he),
                     f3_dot(f3_make(fabsf(m[1][0]), fabsf(m[1][1]), fabsf(m[1][2])), he),
                     f3_dot(f3_make(fabsf(m[2][0]), fabsf(m[2][1]), fabsf(m[2][2])), he));
    f3 amin = f3_sub(center, ext), amax = f3_add(center, ext);

    memset(body_out, 0, 80);
    memcpy(body_out, pos, sizeof(float) * 3);
    memcpy(body_out + 4, orn, sizeof(float) * 4);
    memcpy(body_out + 16, &collidable, sizeof(int));
    body_out[17] = mass != 0.f ? 1.f / mass : 0.f;
    body_out[18] = 0.f; /* restitution */
    body_out[19] = 1.f; /* friction */
    memset(inertia_out, 0, 96);
    if (mass != 0.f) {
        /* the AABB box inertia with the full extent as "half extent" (b3GpuNarrowPhase.cpp:876-901) */
        f3 hx = f3_sub(amax, amin);
        float lx = 2.f * hx.x, ly = 2.f * hx.y, lz = 2.f * hx.z;
        float li[3] = {(mass / 12.0f) * (ly * ly + lz * lz), (mass / 12.0f) * (lx * lx + lz * lz),
                       (mass / 12.0f) * (lx * lx + ly * ly)};
        float inv[3] = {1.f / li[0], 1.f / li[1], 1.f / li[2]};
        /* m_initInvInertia: diag(inv), rows of 4 floats */
        inertia_out[12 + 0] = inv[0];
        inertia_out[12 + 5] = inv[1];
        inertia_out[12 + 10] = inv[2];
        /* m_invInertiaWorld = m.scaled(inv) * m.transpose() (b3Matrix3x3.h scaled :520, operator* :1040) */
        float sm[3][3], w[3][3];
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 3; k++) sm[r][k] = m[r][k] * inv[k];
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 3; k++) {
                /* (A * B)[r][k] = A.row(r) . B.col(k); B = m^T so B.col(k) = m.row(k) (tdotx/y/z) */
                w[r][k] = sm[r][0] * m[k][0] + sm[r][1] * m[k][1] + sm[r][2] * m[k][2];
            }
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 3; k++) inertia_out[4 * r + k] = w[r][k];
    }
    return 0;
}
