// Convex hull topology for registerConvexHullShape.
//
// The reference builds hull tables in two steps, and both are followed here so that a hull
// registered from the same points gets the reference's tables bit for bit (same vertex order,
// same faces in the same order with the same float planes, same unique edges):
//
//  1. b3ConvexHullComputer::compute (Bullet3Geometry/b3ConvexHullComputer.cpp): the points are
//     quantised onto a 10216-step integer grid spanning their bounding box (:1943-2062) and the
//     exact hull is built by Kniemeyer's divide and conquer after Preparata and Hong: sort by
//     (y, x, z), split, hull both halves, join the x/y projections (:1024-1207) and wrap the band
//     of faces between the halves with a max-angle search (:1651-1936, :1390-1649).  Its output
//     lists the vertices breadth first from the final hull's start vertex and the faces in the
//     order their first edges are met (:2625-2745).  That order decides which of two welded
//     near-coplanar triangles gives a merged face its plane, so the algorithm is followed step by
//     step; all of it is integer arithmetic (64-bit, with 128-bit products to compare ratios).
//  2. b3ConvexUtility::initializePolyhedralFeatures (Bullet3Collision/NarrowPhaseCollision/
//     b3ConvexUtility.cpp:26-246): per face a float normal from its first two edges and the plane
//     constant -min(v.n) (:47-98), welding of faces whose normals are within 0.999 with a 2-D
//     Graham scan (:100-244, Bullet3Geometry/b3GrahamScan2dConvexHull.h), and the unique edge
//     directions (:319-375).
//
// Representation here: vertices and half-edges live in flat arrays addressed by index (edge
// pairs allocated together, a free list for removed pairs), not in pointer-linked pools; the
// float post-processing uses plain float3 arithmetic in the reference's operation order (the
// library is built without FMA contraction).  Host code only; no GPU is touched.
#include "hull.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace b3g {

namespace {

// ------------------------------------------------------------------ exact integer hull
struct I3 {
    int32_t x, y, z;
    bool operator==(const I3& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct L3 {
    int64_t x, y, z;
};
inline I3 operator-(I3 a, I3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline L3 cross(I3 a, I3 b) {
    return {(int64_t)a.y * b.z - (int64_t)a.z * b.y, (int64_t)a.z * b.x - (int64_t)a.x * b.z,
            (int64_t)a.x * b.y - (int64_t)a.y * b.x};
}
inline L3 cross(I3 a, L3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline int64_t dot(I3 a, I3 b) { return (int64_t)a.x * b.x + (int64_t)a.y * b.y + (int64_t)a.z * b.z; }
inline int64_t dot(I3 a, L3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline int64_t dot(L3 a, L3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// a ratio n/d kept as sign and magnitudes; d == 0 is +-infinity (or undefined when n == 0 too)
struct Ratio {
    uint64_t n = 0, d = 0;
    int sign = 0;
    Ratio() = default;
    Ratio(int64_t num, int64_t den) {
        sign = num > 0 ? 1 : num < 0 ? -1 : 0;
        n = num >= 0 ? (uint64_t)num : (uint64_t)(-num);
        if (den < 0) {
            sign = -sign;
            d = (uint64_t)(-den);
        } else {
            d = (uint64_t)den;
        }
    }
    bool undefined() const { return sign == 0 && d == 0; }
    bool minus_infinity() const { return sign < 0 && d == 0; }
    int compare(const Ratio& b) const {
        if (sign != b.sign) return sign - b.sign;
        if (sign == 0) return 0;
        const unsigned __int128 l = (unsigned __int128)n * b.d, r = (unsigned __int128)d * b.n;
        return sign * (l < r ? -1 : l > r ? 1 : 0);
    }
};

constexpr int NIL = -1;

class IntegerHull {
public:
    struct Vtx {
        I3 p;
        int ring_next = NIL, ring_prev = NIL;  // projection ring of the partial hull
        int edge = NIL;                        // one outgoing half-edge
        int out = -1;                          // output index
    };
    struct HalfEdge {
        int next, prev;  // ring of half-edges leaving the same vertex
        int target;      // vertex index
        int stamp;       // merge stamp at creation; output index while extracting
    };
    struct Part {        // a partial hull: its extreme vertices in x/y and y/x order
        int min_xy = NIL, max_xy = NIL, min_yx = NIL, max_yx = NIL;
    };

    std::vector<Vtx> v;
    std::vector<HalfEdge> e;  // half-edge 2k and 2k+1 are each other's reverse
    std::vector<int> free_pairs;
    int stamp = -3;

    static int rev(int h) { return h ^ 1; }
    I3 d(int a, int b) const { return v[a].p - v[b].p; }

    int new_pair(int from, int to) {
        int k;
        if (!free_pairs.empty()) {
            k = free_pairs.back();
            free_pairs.pop_back();
        } else {
            k = (int)e.size() / 2;
            e.resize(e.size() + 2);
        }
        e[2 * k] = HalfEdge{NIL, NIL, to, stamp};
        e[2 * k + 1] = HalfEdge{NIL, NIL, from, stamp};
        return 2 * k;
    }
    void link(int a, int b) {
        e[a].next = b;
        e[b].prev = a;
    }
    void remove_pair(int h) {
        const int r = rev(h);
        int n = e[h].next;
        if (n != h) {
            e[n].prev = e[h].prev;
            e[e[h].prev].next = n;
            v[e[r].target].edge = n;
        } else {
            v[e[r].target].edge = NIL;
        }
        n = e[r].next;
        if (n != r) {
            e[n].prev = e[r].prev;
            e[e[r].prev].next = n;
            v[e[h].target].edge = n;
        } else {
            v[e[h].target].edge = NIL;
        }
        free_pairs.push_back(h >> 1);
    }

    enum Turn { TURN_NONE, TURN_CW, TURN_CCW };

    // orientation of half-edge b relative to half-edge a around their common source vertex
    Turn turn(int a, int b, I3 s, I3 t) const {
        if (e[a].next == b) {
            if (e[a].prev == b) {
                const L3 n = cross(t, s);
                const int src = e[rev(b)].target;
                const L3 m = cross(d(e[a].target, src), d(e[b].target, src));
                return dot(n, m) > 0 ? TURN_CCW : TURN_CW;
            }
            return TURN_CCW;
        }
        return e[a].prev == b ? TURN_CW : TURN_NONE;
    }

    // edge of `from` that makes the largest angle with the wrap plane (smallest cotangent)
    int max_angle_edge(bool ccw, int from, I3 s, L3 rxs, L3 sxrxs, Ratio& best) const {
        int pick = NIL;
        const int first = v[from].edge;
        if (first == NIL) return NIL;
        int h = first;
        do {
            if (e[h].stamp > stamp) {
                const I3 t = d(e[h].target, from);
                const Ratio cot(dot(t, sxrxs), dot(t, rxs));
                if (!cot.undefined()) {
                    int c;
                    if (pick == NIL) {
                        best = cot;
                        pick = h;
                    } else if ((c = cot.compare(best)) < 0) {
                        best = cot;
                        pick = h;
                    } else if (c == 0 && ccw == (turn(pick, h, s, t) == TURN_CCW)) {
                        pick = h;
                    }
                }
            }
            h = e[h].next;
        } while (h != first);
        return pick;
    }

    // advances the wrap over faces coplanar with the current bridge (c0, c1)
    void advance_coplanar(int c0, int c1, int& h0, int& h1) const {
        const int start0 = h0, start1 = h1;
        I3 et0 = start0 != NIL ? v[e[start0].target].p : v[c0].p;
        I3 et1 = start1 != NIL ? v[e[start1].target].p : v[c1].p;
        const I3 s = v[c1].p - v[c0].p;
        const L3 normal = cross(v[e[start0 != NIL ? start0 : start1].target].p - v[c0].p, s);
        const int64_t dist = dot(v[c0].p, normal);
        const L3 perp = cross(s, normal);

        int64_t reach0 = dot(et0, perp);
        if (h0 != NIL) {
            for (;;) {
                const int h = e[rev(h0)].prev;
                const I3 q = v[e[h].target].p;
                if (dot(q, normal) < dist || e[h].stamp == stamp) break;
                const int64_t r = dot(q, perp);
                if (r <= reach0) break;
                reach0 = r;
                h0 = h;
                et0 = q;
            }
        }
        int64_t reach1 = dot(et1, perp);
        if (h1 != NIL) {
            for (;;) {
                const int h = e[rev(h1)].next;
                const I3 q = v[e[h].target].p;
                if (dot(q, normal) < dist || e[h].stamp == stamp) break;
                const int64_t r = dot(q, perp);
                if (r <= reach1) break;
                reach1 = r;
                h1 = h;
                et1 = q;
            }
        }
        int64_t dx = reach1 - reach0;
        if (dx > 0) {
            for (;;) {
                const int64_t dy = dot(et1 - et0, s);
                if (h0 != NIL) {
                    const int f0 = rev(e[h0].next);
                    if (e[f0].stamp > stamp) {
                        const I3 q = v[e[f0].target].p;
                        const int64_t dx0 = dot(q - et0, perp), dy0 = dot(q - et0, s);
                        if (dx0 == 0 ? dy0 < 0 : (dx0 < 0 && Ratio(dy0, dx0).compare(Ratio(dy, dx)) >= 0)) {
                            et0 = q;
                            dx = dot(et1 - et0, perp);
                            h0 = h0 == start0 ? NIL : f0;
                            continue;
                        }
                    }
                }
                if (h1 != NIL) {
                    const int f1 = e[rev(h1)].next;
                    if (e[f1].stamp > stamp) {
                        const I3 q = v[e[f1].target].p;
                        const I3 d1 = q - et1;
                        if (dot(d1, normal) == 0) {
                            const int64_t dx1 = dot(d1, perp), dy1 = dot(d1, s), dxn = dot(q - et0, perp);
                            if (dxn > 0 &&
                                (dx1 == 0 ? dy1 < 0 : (dx1 < 0 && Ratio(dy1, dx1).compare(Ratio(dy, dx)) > 0))) {
                                h1 = f1;
                                et1 = q;
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
                const int64_t dy = dot(et1 - et0, s);
                if (h1 != NIL) {
                    const int f1 = rev(e[h1].prev);
                    if (e[f1].stamp > stamp) {
                        const I3 q = v[e[f1].target].p;
                        const int64_t dx1 = dot(q - et1, perp), dy1 = dot(q - et1, s);
                        if (dx1 == 0 ? dy1 > 0 : (dx1 < 0 && Ratio(dy1, dx1).compare(Ratio(dy, dx)) <= 0)) {
                            et1 = q;
                            dx = dot(et1 - et0, perp);
                            h1 = h1 == start1 ? NIL : f1;
                            continue;
                        }
                    }
                }
                if (h0 != NIL) {
                    const int f0 = e[rev(h0)].prev;
                    if (e[f0].stamp > stamp) {
                        const I3 q = v[e[f0].target].p;
                        const I3 d0 = q - et0;
                        if (dot(d0, normal) == 0) {
                            const int64_t dx0 = dot(d0, perp), dy0 = dot(d0, s), dxn = dot(et1 - q, perp);
                            if (dxn < 0 &&
                                (dx0 == 0 ? dy0 > 0 : (dx0 < 0 && Ratio(dy0, dx0).compare(Ratio(dy, dx)) < 0))) {
                                h0 = f0;
                                et0 = q;
                                dx = dxn;
                                continue;
                            }
                        }
                    }
                }
                break;
            }
        }
    }

    // joins the projection rings of two parts separated along x; false when the right part is a
    // vertical segment right above the left part's last point (no bridge in the projection)
    bool join_projections(Part& a, Part& b, int& c0, int& c1) {
        int v0 = a.max_yx, v1 = b.min_yx;
        if (v[v0].p.x == v[v1].p.x && v[v0].p.y == v[v1].p.y) {
            const int v1p = v[v1].ring_prev;
            if (v1p == v1) {
                c0 = v0;
                if (v[v1].edge != NIL) v1 = e[v[v1].edge].target;
                c1 = v1;
                return false;
            }
            const int v1n = v[v1].ring_next;
            v[v1p].ring_next = v1n;
            v[v1n].ring_prev = v1p;
            const I3 pn = v[v1n].p, pp = v[v1p].p;
            if (v1 == b.min_xy) b.min_xy = (pn.x < pp.x || (pn.x == pp.x && pn.y < pp.y)) ? v1n : v1p;
            if (v1 == b.max_xy) b.max_xy = (pn.x > pp.x || (pn.x == pp.x && pn.y > pp.y)) ? v1n : v1p;
        }
        v0 = a.max_xy;
        v1 = b.max_xy;
        int v00 = NIL, v10 = NIL;
        int32_t sg = 1;
        for (int side = 0; side <= 1; side++) {
            auto fwd0 = [&](int x) { return side ? v[x].ring_next : v[x].ring_prev; };
            auto bwd0 = [&](int x) { return side ? v[x].ring_prev : v[x].ring_next; };
            int32_t dx = (v[v1].p.x - v[v0].p.x) * sg;
            if (dx > 0) {
                for (;;) {
                    const int32_t dy = v[v1].p.y - v[v0].p.y;
                    const int w0 = fwd0(v0);
                    if (w0 != v0) {
                        const int32_t dx0 = (v[w0].p.x - v[v0].p.x) * sg, dy0 = v[w0].p.y - v[v0].p.y;
                        if (dy0 <= 0 && (dx0 == 0 || (dx0 < 0 && (int64_t)dy0 * dx <= (int64_t)dy * dx0))) {
                            v0 = w0;
                            dx = (v[v1].p.x - v[v0].p.x) * sg;
                            continue;
                        }
                    }
                    const int w1 = side ? v[v1].ring_next : v[v1].ring_prev;
                    if (w1 != v1) {
                        const int32_t dx1 = (v[w1].p.x - v[v1].p.x) * sg, dy1 = v[w1].p.y - v[v1].p.y;
                        const int32_t dxn = (v[w1].p.x - v[v0].p.x) * sg;
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
                    const int32_t dy = v[v1].p.y - v[v0].p.y;
                    const int w1 = side ? v[v1].ring_prev : v[v1].ring_next;
                    if (w1 != v1) {
                        const int32_t dx1 = (v[w1].p.x - v[v1].p.x) * sg, dy1 = v[w1].p.y - v[v1].p.y;
                        if (dy1 >= 0 && (dx1 == 0 || (dx1 < 0 && (int64_t)dy1 * dx <= (int64_t)dy * dx1))) {
                            v1 = w1;
                            dx = (v[v1].p.x - v[v0].p.x) * sg;
                            continue;
                        }
                    }
                    const int w0 = bwd0(v0);
                    if (w0 != v0) {
                        const int32_t dx0 = (v[w0].p.x - v[v0].p.x) * sg, dy0 = v[w0].p.y - v[v0].p.y;
                        const int32_t dxn = (v[v1].p.x - v[w0].p.x) * sg;
                        if (dxn < 0 && dy0 > 0 && (dx0 == 0 || (dx0 < 0 && (int64_t)dy0 * dx < (int64_t)dy * dx0))) {
                            v0 = w0;
                            dx = dxn;
                            continue;
                        }
                    }
                    break;
                }
            } else {
                const int32_t x = v[v0].p.x;
                int32_t y0 = v[v0].p.y;
                int w0 = v0, t;
                while ((t = fwd0(w0)) != v0 && v[t].p.x == x && v[t].p.y <= y0) {
                    w0 = t;
                    y0 = v[t].p.y;
                }
                v0 = w0;
                int32_t y1 = v[v1].p.y;
                int w1 = v1;
                while ((t = side ? v[w1].ring_prev : v[w1].ring_next) != v1 && v[t].p.x == x && v[t].p.y >= y1) {
                    w1 = t;
                    y1 = v[t].p.y;
                }
                v1 = w1;
            }
            if (side == 0) {
                v00 = v0;
                v10 = v1;
                v0 = a.min_xy;
                v1 = b.min_xy;
                sg = -1;
            }
        }
        v[v0].ring_prev = v1;
        v[v1].ring_next = v0;
        v[v00].ring_next = v10;
        v[v10].ring_prev = v00;
        if (v[b.min_xy].p.x < v[a.min_xy].p.x) a.min_xy = b.min_xy;
        if (v[b.max_xy].p.x >= v[a.max_xy].p.x) a.max_xy = b.max_xy;
        a.max_yx = b.max_yx;
        c0 = v00;
        c1 = v10;
        return true;
    }

    // wraps the band of faces joining part a and part b (the result is left in a)
    void join(Part& a, Part& b) {
        if (b.max_xy == NIL) return;
        if (a.max_xy == NIL) {
            a = b;
            return;
        }
        stamp--;
        int c0 = NIL, c1 = NIL;
        int toPrev0 = NIL, firstNew0 = NIL, head0 = NIL, tail0 = NIL;
        int toPrev1 = NIL, firstNew1 = NIL, head1 = NIL, tail1 = NIL;
        I3 prevPoint;
        const I3 down{0, 0, -1};
        if (join_projections(a, b, c0, c1)) {
            const I3 s = v[c1].p - v[c0].p;
            const L3 normal = cross(down, s);
            const L3 t = cross(s, normal);
            int start0 = NIL, start1 = NIL;
            for (int k = 0; k < 2; k++) {
                const int c = k == 0 ? c0 : c1;
                int& start = k == 0 ? start0 : start1;
                const Turn want = k == 0 ? TURN_CW : TURN_CCW;
                const int first = v[c].edge;
                if (first == NIL) continue;
                int h = first;
                do {
                    const I3 q = d(e[h].target, c);
                    if (dot(q, normal) == 0 && dot(q, t) > 0 && (start == NIL || turn(start, h, s, down) == want))
                        start = h;
                    h = e[h].next;
                } while (h != first);
            }
            if (start0 != NIL || start1 != NIL) {
                advance_coplanar(c0, c1, start0, start1);
                if (start0 != NIL) c0 = e[start0].target;
                if (start1 != NIL) c1 = e[start1].target;
            }
            prevPoint = v[c1].p;
            prevPoint.z++;
        } else {
            prevPoint = v[c1].p;
            prevPoint.x++;
        }
        const int first0 = c0, first1 = c1;
        bool firstRun = true;
        for (;;) {
            const I3 s = v[c1].p - v[c0].p;
            const I3 r = prevPoint - v[c0].p;
            const L3 rxs = cross(r, s);
            const L3 sxrxs = cross(s, rxs);
            Ratio cot0, cot1;
            const int min0 = max_angle_edge(false, c0, s, rxs, sxrxs, cot0);
            const int min1 = max_angle_edge(true, c1, s, rxs, sxrxs, cot1);
            if (min0 == NIL && min1 == NIL) {
                const int h = new_pair(c0, c1);
                link(h, h);
                v[c0].edge = h;
                link(rev(h), rev(h));
                v[c1].edge = rev(h);
                return;
            }
            const int cmp = min0 == NIL ? 1 : min1 == NIL ? -1 : cot0.compare(cot1);
            if (firstRun || (cmp >= 0 ? !cot1.minus_infinity() : !cot0.minus_infinity())) {
                // the new bridge edge joins the pending chains on both sides
                const int h = new_pair(c0, c1);
                if (tail0 != NIL) e[tail0].prev = h;
                else head0 = h;
                e[h].next = tail0;
                tail0 = h;
                const int hr = rev(h);
                if (tail1 != NIL) e[tail1].next = hr;
                else head1 = hr;
                e[hr].prev = tail1;
                tail1 = hr;
            }
            int e0 = min0, e1 = min1;
            if (cmp == 0) advance_coplanar(c0, c1, e0, e1);
            if (cmp >= 0 && e1 != NIL) {
                if (toPrev1 != NIL)
                    for (int h = e[toPrev1].next, n; h != min1; h = n) {
                        n = e[h].next;
                        remove_pair(h);
                    }
                if (tail1 != NIL) {
                    if (toPrev1 != NIL) {
                        link(toPrev1, head1);
                    } else {
                        link(e[min1].prev, head1);
                        firstNew1 = head1;
                    }
                    link(tail1, min1);
                    head1 = tail1 = NIL;
                } else if (toPrev1 == NIL) {
                    firstNew1 = min1;
                }
                prevPoint = v[c1].p;
                c1 = e[e1].target;
                toPrev1 = rev(e1);
            }
            if (cmp <= 0 && e0 != NIL) {
                if (toPrev0 != NIL)
                    for (int h = e[toPrev0].prev, n; h != min0; h = n) {
                        n = e[h].prev;
                        remove_pair(h);
                    }
                if (tail0 != NIL) {
                    if (toPrev0 != NIL) {
                        link(head0, toPrev0);
                    } else {
                        link(head0, e[min0].next);
                        firstNew0 = head0;
                    }
                    link(min0, tail0);
                    head0 = tail0 = NIL;
                } else if (toPrev0 == NIL) {
                    firstNew0 = min0;
                }
                prevPoint = v[c0].p;
                c0 = e[e0].target;
                toPrev0 = rev(e0);
            }
            if (c0 == first0 && c1 == first1) {
                if (toPrev0 == NIL) {
                    link(head0, tail0);
                    v[c0].edge = tail0;
                } else {
                    for (int h = e[toPrev0].prev, n; h != firstNew0; h = n) {
                        n = e[h].prev;
                        remove_pair(h);
                    }
                    if (tail0 != NIL) {
                        link(head0, toPrev0);
                        link(firstNew0, tail0);
                    }
                }
                if (toPrev1 == NIL) {
                    link(tail1, head1);
                    v[c1].edge = tail1;
                } else {
                    for (int h = e[toPrev1].next, n; h != firstNew1; h = n) {
                        n = e[h].next;
                        remove_pair(h);
                    }
                    if (tail1 != NIL) {
                        link(toPrev1, head1);
                        link(tail1, firstNew1);
                    }
                }
                return;
            }
            firstRun = false;
        }
    }

    // hull of the sorted vertices [lo, hi)
    void build(int lo, int hi, Part& out) {
        const int n = hi - lo;
        if (n == 0) {
            out = Part();
            return;
        }
        if (n == 2 && !(v[lo].p == v[lo + 1].p)) {
            int a = lo, b = lo + 1;
            const int32_t dx = v[a].p.x - v[b].p.x, dy = v[a].p.y - v[b].p.y;
            if (dx == 0 && dy == 0) {
                if (v[a].p.z > v[b].p.z) std::swap(a, b);
                v[a].ring_next = v[a].ring_prev = a;
                out.min_xy = out.max_xy = out.min_yx = out.max_yx = a;
            } else {
                v[a].ring_next = v[a].ring_prev = b;
                v[b].ring_next = v[b].ring_prev = a;
                const bool a_first_x = dx < 0 || (dx == 0 && dy < 0);
                const bool a_first_y = dy < 0 || (dy == 0 && dx < 0);
                out.min_xy = a_first_x ? a : b;
                out.max_xy = a_first_x ? b : a;
                out.min_yx = a_first_y ? a : b;
                out.max_yx = a_first_y ? b : a;
            }
            const int h = new_pair(a, b);
            link(h, h);
            v[a].edge = h;
            link(rev(h), rev(h));
            v[b].edge = rev(h);
            return;
        }
        if (n <= 2) {  // one point, or two equal ones
            v[lo].edge = NIL;
            v[lo].ring_next = v[lo].ring_prev = lo;
            out.min_xy = out.max_xy = out.min_yx = out.max_yx = lo;
            return;
        }
        const int mid = lo + n / 2;
        int right = mid;
        while (right < hi && v[right].p == v[mid - 1].p) right++;  // duplicates of the split point
        build(lo, mid, out);
        Part other;
        build(right, hi, other);
        join(out, other);
    }
};

// in-place sort by (y, x, z): b3AlignedObjectArray::quickSortInternal with b3PointCmp (equal
// points are interchangeable, so any order among them gives the same hull)
inline bool point_before(const I3& p, const I3& q) {
    return p.y < q.y || (p.y == q.y && (p.x < q.x || (p.x == q.x && p.z < q.z)));
}

// ------------------------------------------------------------------ float post-processing
struct F3 {
    float x, y, z;
};
inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 fcross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// b3Vector3::normalize: times the reciprocal of the length
inline F3 unit(F3 a) { return a * (1.0f / std::sqrt(fdot(a, a))); }

// b3PlaneSpace1 (Bullet3Common/b3Vector3.h:1184-1212)
void plane_space(F3 n, F3& p, F3& q) {
    if (std::fabs(n.z) > 0.70710678f) {
        const float a = n.y * n.y + n.z * n.z, k = 1.0f / std::sqrt(a);
        p = {0.f, -n.z * k, n.y * k};
        q = {a * k, -n.x * p.z, n.x * p.y};
    } else {
        const float a = n.x * n.x + n.y * n.y, k = 1.0f / std::sqrt(a);
        p = {-n.y * k, n.x * k, 0.f};
        q = {-n.z * p.y, n.z * p.x, a * k};
    }
}

struct FlatPoint {
    F3 p;
    int org;
    float angle;
};

// 2-D hull of the points of a welded face group around `axis`: anchor with the smallest
// projection on the plane's first axis, points by angle, then distance, then index (a total
// order), back-tracking scan (b3GrahamScanConvexHull2D)
std::vector<FlatPoint> flat_hull(std::vector<FlatPoint> pts, F3 axis) {
    F3 a0, a1;
    plane_space(axis, a0, a1);
    std::vector<FlatPoint> hull;
    if (pts.size() <= 1) {
        for (size_t i = 0; i < pts.size(); i++) hull.push_back(pts[0]);
        return hull;
    }
    for (size_t i = 0; i < pts.size(); i++)
        if (fdot(pts[i].p, a0) < fdot(pts[0].p, a0)) std::swap(pts[0], pts[i]);
    pts[0].angle = -1e30f;
    for (size_t i = 1; i < pts.size(); i++) {
        const F3 ar = pts[i].p - pts[0].p;
        pts[i].angle = fdot(fcross(a0, ar), axis) / std::sqrt(fdot(ar, ar));
    }
    const F3 anchor = pts[0].p;
    std::sort(pts.begin() + 1, pts.end(), [&](const FlatPoint& a, const FlatPoint& b) {
        if (a.angle != b.angle) return a.angle < b.angle;
        const float al = fdot(a.p - anchor, a.p - anchor), bl = fdot(b.p - anchor, b.p - anchor);
        if (al != bl) return al < bl;
        return a.org < b.org;
    });
    size_t i = 0;
    for (; i < 2; i++) hull.push_back(pts[i]);
    for (; i != pts.size(); i++) {
        bool convex = false;
        while (!convex && hull.size() > 1) {
            const F3 a = hull[hull.size() - 2].p, b = hull[hull.size() - 1].p;
            convex = fdot(fcross(a - b, a - pts[i].p), axis) > 0;
            if (convex)
                hull.push_back(pts[i]);
            else
                hull.pop_back();
        }
    }
    return hull;
}

struct Polygon {
    std::vector<int> idx;
    float plane[4];
};

}  // namespace

int build_hull(const float* verts, int stride_bytes, int num_verts, const float scaling[3], HullTables& out) {
    out = HullTables();
    if (num_verts < 1 || verts == nullptr) return 1;
    const unsigned char* base = reinterpret_cast<const unsigned char*>(verts);
    std::vector<F3> in(num_verts);
    for (int i = 0; i < num_verts; i++) {
        const float* p = reinterpret_cast<const float*>(base + (size_t)i * stride_bytes);
        const float sx = scaling ? scaling[0] : 1.f, sy = scaling ? scaling[1] : 1.f, sz = scaling ? scaling[2] : 1.f;
        in[i] = {p[0] * sx, p[1] * sy, p[2] * sz};
    }
    // quantisation: axes ranked by extent; the grid step is the extent / 10216, negated so that
    // (med, max, min) stays a right-handed frame
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (const F3& p : in) {
        const float c[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) {
            if (c[k] < lo[k]) lo[k] = c[k];
            if (hi[k] < c[k]) hi[k] = c[k];
        }
    }
    float step[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    const int maxAxis = step[0] < step[1] ? (step[1] < step[2] ? 2 : 1) : (step[0] < step[2] ? 2 : 0);
    int minAxis = step[0] < step[1] ? (step[0] < step[2] ? 0 : 2) : (step[1] < step[2] ? 1 : 2);
    if (minAxis == maxAxis) minAxis = (maxAxis + 1) % 3;
    const int medAxis = 3 - maxAxis - minAxis;
    const float inv_grid = 1.0f / 10216.0f;
    for (int k = 0; k < 3; k++) step[k] = step[k] * inv_grid;
    if ((medAxis + 1) % 3 != maxAxis)
        for (int k = 0; k < 3; k++) step[k] = step[k] * -1.0f;
    float inv_step[3], center[3];
    for (int k = 0; k < 3; k++) {
        inv_step[k] = step[k] != 0 ? 1.0f / step[k] : step[k];
        center[k] = (lo[k] + hi[k]) * 0.5f;
    }
    IntegerHull H;
    H.v.resize(num_verts);
    std::vector<I3> q(num_verts);
    for (int i = 0; i < num_verts; i++) {
        const float c[3] = {in[i].x, in[i].y, in[i].z};
        float g[3];
        for (int k = 0; k < 3; k++) g[k] = (c[k] - center[k]) * inv_step[k];
        q[i] = I3{(int32_t)g[medAxis], (int32_t)g[maxAxis], (int32_t)g[minAxis]};
    }
    std::sort(q.begin(), q.end(), point_before);
    for (int i = 0; i < num_verts; i++) H.v[i].p = q[i];
    H.e.reserve(6 * (size_t)num_verts + 16);
    IntegerHull::Part whole;
    H.build(0, num_verts, whole);

    // vertices breadth first from the start vertex; each vertex's half-edges in ring order, a
    // pair numbered when first met (output half-edge 2k leaves the vertex that numbered it)
    struct OutEdge {
        int next, reverse, target;
    };
    std::vector<int> order;
    std::vector<OutEdge> oe;
    std::vector<int> ofaces;
    std::vector<F3> V;
    if (whole.min_xy != NIL) {
        H.v[whole.min_xy].out = 0;
        order.push_back(whole.min_xy);
    }
    for (size_t k = 0; k < order.size(); k++) {
        const int vi = order[k];
        const I3 p = H.v[vi].p;
        float c[3];
        c[medAxis] = (float)p.x;
        c[maxAxis] = (float)p.y;
        c[minAxis] = (float)p.z;
        V.push_back(F3{c[0] * step[0] + center[0], c[1] * step[1] + center[1], c[2] * step[2] + center[2]});
        const int first = H.v[vi].edge;
        if (first == NIL) continue;
        int firstOut = -1, prevOut = -1, h = first;
        do {
            if (H.e[h].stamp < 0) {
                const int o = (int)oe.size();
                oe.push_back(OutEdge{0, 1, 0});
                oe.push_back(OutEdge{0, -1, (int)k});
                H.e[h].stamp = o;
                H.e[IntegerHull::rev(h)].stamp = o + 1;
                const int t = H.e[h].target;
                if (H.v[t].out < 0) {
                    H.v[t].out = (int)order.size();
                    order.push_back(t);
                }
                oe[o].target = H.v[t].out;
            }
            if (prevOut >= 0)
                oe[H.e[h].stamp].next = prevOut - H.e[h].stamp;
            else
                firstOut = H.e[h].stamp;
            prevOut = H.e[h].stamp;
            h = H.e[h].next;
        } while (h != first);
        oe[firstOut].next = prevOut - firstOut;
    }
    for (size_t k = 0; k < order.size(); k++) {
        const int first = H.v[order[k]].edge;
        if (first == NIL) continue;
        int h = first;
        do {
            if (H.e[h].stamp >= 0) {  // a face not traced yet: trace it through reverse->prev
                ofaces.push_back(H.e[h].stamp);
                int f = h;
                do {
                    H.e[f].stamp = -1;
                    f = H.e[IntegerHull::rev(f)].prev;
                } while (f != h);
            }
            h = H.e[h].next;
        } while (h != first);
    }
    if (ofaces.empty()) return 1;  // collinear or fewer than three distinct points: no face

    // faces with float planes from their first two edges
    std::vector<Polygon> tri(ofaces.size());
    for (size_t i = 0; i < ofaces.size(); i++) {
        F3 ed[2];
        int ned = 0;
        int x = ofaces[i];
        do {
            const int r = x + oe[x].reverse;
            const int src = oe[r].target, dst = oe[x].target;
            tri[i].idx.push_back(src);
            const F3 dir = unit(V[dst] - V[src]);
            if (ned < 2) ed[ned++] = dir;
            x = r + oe[r].next;
        } while (x != ofaces[i]);
        const F3 n = ned == 2 ? unit(fcross(ed[0], ed[1])) : F3{0, 0, 0};
        float m = 1e30f;
        for (int vi : tri[i].idx) {
            const float eq = fdot(V[vi], n);
            if (m > eq) m = eq;
        }
        tri[i].plane[0] = n.x;
        tri[i].plane[1] = n.y;
        tri[i].plane[2] = n.z;
        tri[i].plane[3] = -m;
    }

    // welding of near-coplanar faces; groups are formed from the back of the to-do list, whose
    // removals swap the removed entry with the last one (b3AlignedObjectArray::remove)
    std::vector<Polygon> faces;
    std::vector<int> todo(tri.size());
    for (size_t i = 0; i < tri.size(); i++) todo[i] = (int)i;
    while (!todo.empty()) {
        std::vector<int> group{todo.back()};
        todo.pop_back();
        const Polygon& ref = tri[group[0]];
        const F3 nA{ref.plane[0], ref.plane[1], ref.plane[2]};
        for (int j = (int)todo.size() - 1; j >= 0; j--) {
            const int i = todo[j];
            if (fdot(nA, F3{tri[i].plane[0], tri[i].plane[1], tri[i].plane[2]}) > 0.999f) {
                group.push_back(i);
                auto it = std::find(todo.begin(), todo.end(), i);
                *it = todo.back();
                todo.pop_back();
            }
        }
        bool merged = false;
        if (group.size() > 1) {
            std::vector<FlatPoint> pts;
            F3 avg{0, 0, 0};
            for (int g : group) {
                avg = avg + F3{tri[g].plane[0], tri[g].plane[1], tri[g].plane[2]};
                for (int vi : tri[g].idx)
                    if (std::none_of(pts.begin(), pts.end(), [&](const FlatPoint& f) { return f.org == vi; }))
                        pts.push_back(FlatPoint{V[vi], vi, 0.f});
            }
            const std::vector<FlatPoint> outline = flat_hull(pts, unit(avg));
            Polygon joined;
            std::copy(tri[group[0]].plane, tri[group[0]].plane + 4, joined.plane);
            for (const FlatPoint& f : outline) {
                joined.idx.push_back(f.org);
                for (FlatPoint& p : pts)
                    if (p.org == f.org) {
                        p.org = -1;
                        break;
                    }
            }
            // a point left inside the outline that another face still uses vetoes the merge
            bool veto = false;
            for (const FlatPoint& p : pts) {
                if (p.org == -1) continue;
                for (size_t j = 0; j < tri.size() && !veto; j++) {
                    if (std::find(group.begin(), group.end(), (int)j) != group.end()) continue;
                    veto = std::find(tri[j].idx.begin(), tri[j].idx.end(), p.org) != tri[j].idx.end();
                }
                if (veto) break;
            }
            if (!veto) {
                merged = true;
                faces.push_back(joined);
            }
        }
        if (!merged)
            for (int g : group) faces.push_back(tri[g]);
    }

    // unique edge directions: v[min] - v[max] normalised, unless parallel or anti-parallel to
    // an earlier one within 1e-6 per component
    std::vector<F3> edges;
    auto tiny = [](F3 a) { return !(std::fabs(a.x) > 1e-6 || std::fabs(a.y) > 1e-6 || std::fabs(a.z) > 1e-6); };
    for (const Polygon& f : faces) {
        const int n = (int)f.idx.size();
        for (int j = 0; j < n; j++) {
            const int a = f.idx[j], b = f.idx[(j + 1) % n];
            const F3 dir = unit(V[std::min(a, b)] - V[std::max(a, b)]);
            if (std::none_of(edges.begin(), edges.end(), [&](F3 u) { return tiny(u - dir) || tiny(u + dir); }))
                edges.push_back(dir);
        }
    }

    for (const F3& p : V) out.vertices.insert(out.vertices.end(), {p.x, p.y, p.z});
    for (const Polygon& f : faces) {
        out.planes.insert(out.planes.end(), f.plane, f.plane + 4);
        out.face_counts.push_back((int)f.idx.size());
        out.indices.insert(out.indices.end(), f.idx.begin(), f.idx.end());
    }
    for (const F3& d : edges) out.edges.insert(out.edges.end(), {d.x, d.y, d.z});
    // local centre = vertex mean (b3GpuNarrowPhase.cpp:326-331)
    F3 c{0, 0, 0};
    for (const F3& p : V) c = c + p;
    c = c * (1.f / (float)V.size());
    out.center[0] = c.x;
    out.center[1] = c.y;
    out.center[2] = c.z;
    return 0;
}

}  // namespace b3g
