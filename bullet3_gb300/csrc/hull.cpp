// Convex hull topology for registerConvexHullShape.
//
// The reference builds hull topology with b3ConvexHullComputer (exact integer
// arithmetic) followed by b3ConvexUtility::initializePolyhedralFeatures
// (Bullet3Collision/NarrowPhaseCollision/b3ConvexUtility.cpp:26-246): face normals from the
// first two edges of each face (:67-81), plane constant = -min(v.n) (:88-96), coplanar
// face welding with a 0.999 normal threshold and a 2-D Graham scan (:100-244, Graham scan in
// Bullet3Geometry/b3GrahamScan2dConvexHull.h), and the unique-edge table (:291-345).
//
// Here the hull itself is an incremental 3-D hull in double precision (own design, one
// triangle fan per added point); the post-processing follows the reference's rules so that
// the face planes, face polygons and unique edges carry the same meaning (and, for
// non-degenerate inputs, the same geometry).  Host code only; no GPU is touched.
#include "hull.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <unordered_map>
#include <vector>

namespace b3g {

namespace {

struct D3 {
    double x, y, z;
};
static inline D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct Tri {
    int v[3];
    D3 n;       // unnormalised outward normal
    double d;   // n.x + d = 0 on the plane
    bool alive;
};

// float3 helpers that follow the reference's float arithmetic for the post-processing
struct F3 {
    float x, y, z;
};
static inline F3 fsub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline F3 fadd(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline F3 fscale(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline F3 fcross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline F3 fnormalize(F3 a) {
    float l = std::sqrt(fdot(a, a));
    float inv = 1.0f / l;
    return fscale(a, inv);
}

// b3PlaneSpace1 (Bullet3Common/b3Vector3.h:1184-1212)
static void plane_space(F3 n, F3& p, F3& q) {
    if (std::fabs(n.z) > 0.70710678f) {
        float a = n.y * n.y + n.z * n.z;
        float k = 1.0f / std::sqrt(a);
        p = {0.f, -n.z * k, n.y * k};
        q = {a * k, -n.x * p.z, n.x * p.y};
    } else {
        float a = n.x * n.x + n.y * n.y;
        float k = 1.0f / std::sqrt(a);
        p = {-n.y * k, n.x * k, 0.f};
        q = {-n.z * p.y, n.z * p.x, a * k};
    }
}

struct GPoint {
    F3 p;
    int org;
    float angle;
};

// 2-D convex hull of coplanar points around normalAxis; same anchor choice, angle key,
// tie-breaks and back-tracking rule as b3GrahamScanConvexHull2D.
static void graham_scan(std::vector<GPoint>& pts, std::vector<GPoint>& hull, F3 normalAxis) {
    F3 axis0, axis1;
    plane_space(normalAxis, axis0, axis1);
    if (pts.size() <= 1) {
        for (size_t i = 0; i < pts.size(); i++) hull.push_back(pts[0]);
        return;
    }
    for (size_t i = 0; i < pts.size(); i++) {
        float projL = fdot(pts[i].p, axis0);
        float projR = fdot(pts[0].p, axis0);
        if (projL < projR) std::swap(pts[0], pts[i]);
    }
    pts[0].angle = -1e30f;
    for (size_t i = 1; i < pts.size(); i++) {
        F3 ar = fsub(pts[i].p, pts[0].p);
        pts[i].angle = fdot(fcross(axis0, ar), normalAxis) / std::sqrt(fdot(ar, ar));
    }
    const F3 anchor = pts[0].p;
    std::sort(pts.begin() + 1, pts.end(), [&](const GPoint& a, const GPoint& b) {
        if (a.angle != b.angle) return a.angle < b.angle;
        F3 da = fsub(a.p, anchor), db = fsub(b.p, anchor);
        float al = fdot(da, da), bl = fdot(db, db);
        if (al != bl) return al < bl;
        return a.org < b.org;
    });
    size_t i = 0;
    for (; i < 2; i++) hull.push_back(pts[i]);
    for (; i != pts.size(); i++) {
        bool isConvex = false;
        while (!isConvex && hull.size() > 1) {
            const F3 a = hull[hull.size() - 2].p;
            const F3 b = hull[hull.size() - 1].p;
            isConvex = fdot(fcross(fsub(a, b), fsub(a, pts[i].p)), normalAxis) > 0;
            if (!isConvex)
                hull.pop_back();
            else
                hull.push_back(pts[i]);
        }
    }
}

struct PolyFace {
    std::vector<int> idx;
    float plane[4];
};

}  // namespace

int build_hull(const float* verts, int stride_bytes, int num_verts, const float scaling[3], HullTables& out) {
    out = HullTables();
    if (num_verts < 4 || verts == nullptr) return 1;
    std::vector<F3> inF(num_verts);
    const unsigned char* base = reinterpret_cast<const unsigned char*>(verts);
    for (int i = 0; i < num_verts; i++) {
        const float* v = reinterpret_cast<const float*>(base + (size_t)i * stride_bytes);
        float sx = scaling ? scaling[0] : 1.f, sy = scaling ? scaling[1] : 1.f, sz = scaling ? scaling[2] : 1.f;
        inF[i] = {v[0] * sx, v[1] * sy, v[2] * sz};
    }
    // Input quantisation of b3ConvexHullComputer (Bullet3Geometry/b3ConvexHullComputer.cpp:1943-2035,
    // output :2078-2085): the bounding box is mapped onto a 10216-step integer grid per axis
    // (truncation toward zero) and hull vertices are returned as q * scaling + center.  The hull is
    // then computed exactly on the integer coordinates (all orientation tests fit in a double).
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < num_verts; i++) {
        const float p[3] = {inF[i].x, inF[i].y, inF[i].z};
        for (int k = 0; k < 3; k++) {
            mn[k] = std::min(mn[k], p[k]);
            mx[k] = std::max(mx[k], p[k]);
        }
    }
    float s[3], inv_s[3], center[3];
    const float step = 1.0f / 10216.0f;
    for (int k = 0; k < 3; k++) {
        s[k] = (mx[k] - mn[k]) * step;
        inv_s[k] = s[k] != 0.f ? 1.0f / s[k] : 0.f;
        center[k] = (mn[k] + mx[k]) * 0.5f;
    }
    std::vector<std::array<int, 3>> Q(num_verts);
    for (int i = 0; i < num_verts; i++) {
        const float p[3] = {inF[i].x, inF[i].y, inF[i].z};
        for (int k = 0; k < 3; k++) Q[i][k] = (int)((p[k] - center[k]) * inv_s[k]);
    }
    // unique quantised points (duplicates collapse to the first occurrence)
    std::vector<int> uniq;
    uniq.reserve(num_verts);
    for (int i = 0; i < num_verts; i++) {
        bool dup = false;
        for (int j : uniq)
            if (Q[j] == Q[i]) {
                dup = true;
                break;
            }
        if (!dup) uniq.push_back(i);
    }
    const int n = (int)uniq.size();
    if (n < 4) return 1;
    std::vector<D3> P(n);
    for (int i = 0; i < n; i++) P[i] = {(double)Q[uniq[i]][0], (double)Q[uniq[i]][1], (double)Q[uniq[i]][2]};
    const double eps = 0.0;  // exact integer geometry
    auto dequant = [&](int i) {
        const std::array<int, 3>& q = Q[uniq[i]];
        return F3{(float)q[0] * s[0] + center[0], (float)q[1] * s[1] + center[1], (float)q[2] * s[2] + center[2]};
    };

    // initial tetrahedron: extreme points
    int i0 = 0, i1 = -1, i2 = -1, i3 = -1;
    double best = -1;
    for (int i = 1; i < n; i++) {
        D3 d = dsub(P[i], P[i0]);
        double l = ddot(d, d);
        if (l > best) { best = l; i1 = i; }
    }
    if (best <= 0) return 1;
    best = -1;
    for (int i = 0; i < n; i++) {
        D3 c = dcross(dsub(P[i1], P[i0]), dsub(P[i], P[i0]));
        double l = ddot(c, c);
        if (l > best) { best = l; i2 = i; }
    }
    if (best <= 0) return 1;
    D3 n012 = dcross(dsub(P[i1], P[i0]), dsub(P[i2], P[i0]));
    best = -1;
    double sgn = 0;
    for (int i = 0; i < n; i++) {
        double v = ddot(n012, dsub(P[i], P[i0]));
        if (std::fabs(v) > best) { best = std::fabs(v); i3 = i; sgn = v; }
    }
    if (best <= 0) return 1;

    std::vector<Tri> tris;
    auto add_tri = [&](int a, int b, int c) {
        Tri t;
        t.v[0] = a; t.v[1] = b; t.v[2] = c;
        t.n = dcross(dsub(P[b], P[a]), dsub(P[c], P[a]));
        t.d = -ddot(t.n, P[a]);
        t.alive = true;
        tris.push_back(t);
    };
    // orient so that normals point away from i3
    if (sgn > 0) {
        add_tri(i0, i2, i1);
        add_tri(i0, i1, i3);
        add_tri(i1, i2, i3);
        add_tri(i2, i0, i3);
    } else {
        add_tri(i0, i1, i2);
        add_tri(i0, i3, i1);
        add_tri(i1, i3, i2);
        add_tri(i2, i3, i0);
    }
    std::vector<char> used(n, 0);
    used[i0] = used[i1] = used[i2] = used[i3] = 1;

    // directed edge -> triangle
    std::unordered_map<uint64_t, int> edge_owner;
    auto key = [](int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; };
    for (int t = 0; t < (int)tris.size(); t++)
        for (int e = 0; e < 3; e++) edge_owner[key(tris[t].v[e], tris[t].v[(e + 1) % 3])] = t;

    // points farthest-first relative to the initial hull keep coplanar extensions stable
    std::vector<int> order;
    for (int i = 0; i < n; i++)
        if (!used[i]) order.push_back(i);

    std::vector<int> visible;
    std::vector<std::pair<int, int>> horizon;
    for (int pi : order) {
        visible.clear();
        for (int t = 0; t < (int)tris.size(); t++) {
            if (!tris[t].alive) continue;
            // exact: integer coordinates below 2^15, every product below 2^53
            double dist = ddot(tris[t].n, P[pi]) + tris[t].d;
            if (dist > eps) visible.push_back(t);
        }
        if (visible.empty()) continue;
        std::vector<char> isvis(tris.size(), 0);
        for (int t : visible) isvis[t] = 1;
        horizon.clear();
        for (int t : visible) {
            for (int e = 0; e < 3; e++) {
                int a = tris[t].v[e], b = tris[t].v[(e + 1) % 3];
                auto it = edge_owner.find(key(b, a));
                if (it == edge_owner.end() || !isvis[it->second]) horizon.push_back({a, b});
            }
        }
        for (int t : visible) {
            tris[t].alive = false;
            for (int e = 0; e < 3; e++) {
                uint64_t k = key(tris[t].v[e], tris[t].v[(e + 1) % 3]);
                auto it = edge_owner.find(k);
                if (it != edge_owner.end() && it->second == t) edge_owner.erase(it);
            }
        }
        for (auto& h : horizon) {
            int t = (int)tris.size();
            add_tri(h.first, h.second, pi);
            for (int e = 0; e < 3; e++) edge_owner[key(tris[t].v[e], tris[t].v[(e + 1) % 3])] = t;
        }
        used[pi] = 1;
    }

    // hull vertices, in input order
    std::vector<int> remap(n, -1);
    std::vector<char> onhull(n, 0);
    for (auto& t : tris)
        if (t.alive)
            for (int e = 0; e < 3; e++) onhull[t.v[e]] = 1;
    std::vector<F3> V;
    for (int i = 0; i < n; i++)
        if (onhull[i]) {
            remap[i] = (int)V.size();
            V.push_back(dequant(i));
        }

    // triangle faces with the reference's float plane construction
    std::vector<PolyFace> tmpFaces;
    for (auto& t : tris) {
        if (!t.alive) continue;
        PolyFace f;
        for (int e = 0; e < 3; e++) f.idx.push_back(remap[t.v[e]]);
        F3 e0 = fnormalize(fsub(V[f.idx[1]], V[f.idx[0]]));
        F3 e1 = fnormalize(fsub(V[f.idx[2]], V[f.idx[1]]));
        F3 nrm = fnormalize(fcross(e0, e1));
        float planeEq = 1e30f;
        for (int v : f.idx) {
            float eq = fdot(V[v], nrm);
            if (planeEq > eq) planeEq = eq;
        }
        f.plane[0] = nrm.x; f.plane[1] = nrm.y; f.plane[2] = nrm.z; f.plane[3] = -planeEq;
        tmpFaces.push_back(f);
    }

    // coplanar welding (b3ConvexUtility.cpp:100-244)
    std::vector<PolyFace> faces;
    const float faceWeldThreshold = 0.999f;
    std::vector<int> todo;
    for (int i = 0; i < (int)tmpFaces.size(); i++) todo.push_back(i);
    while (!todo.empty()) {
        std::vector<int> group;
        int refFace = todo.back();
        group.push_back(refFace);
        todo.pop_back();
        F3 nA = {tmpFaces[refFace].plane[0], tmpFaces[refFace].plane[1], tmpFaces[refFace].plane[2]};
        for (int j = (int)todo.size() - 1; j >= 0; j--) {
            int i = todo[j];
            F3 nB = {tmpFaces[i].plane[0], tmpFaces[i].plane[1], tmpFaces[i].plane[2]};
            if (fdot(nA, nB) > faceWeldThreshold) {
                group.push_back(i);
                todo.erase(std::find(todo.begin(), todo.end(), i));
            }
        }
        bool did_merge = false;
        if (group.size() > 1) {
            std::vector<GPoint> orgpoints;
            F3 avg = {0, 0, 0};
            for (int gi : group) {
                const PolyFace& f = tmpFaces[gi];
                avg = fadd(avg, F3{f.plane[0], f.plane[1], f.plane[2]});
                for (int orgIndex : f.idx) {
                    bool found = false;
                    for (auto& op : orgpoints)
                        if (op.org == orgIndex) { found = true; break; }
                    if (!found) orgpoints.push_back(GPoint{V[orgIndex], orgIndex, 0.f});
                }
            }
            PolyFace combined;
            for (int k = 0; k < 4; k++) combined.plane[k] = tmpFaces[group[0]].plane[k];
            std::vector<GPoint> hull2;
            avg = fnormalize(avg);
            graham_scan(orgpoints, hull2, avg);
            for (auto& hp : hull2) {
                combined.idx.push_back(hp.org);
                for (auto& op : orgpoints)
                    if (op.org == hp.org) { op.org = -1; break; }
            }
            bool reject = false;
            for (auto& op : orgpoints) {
                if (op.org == -1) continue;
                for (int j = 0; j < (int)tmpFaces.size() && !reject; j++) {
                    if (std::find(group.begin(), group.end(), j) != group.end()) continue;
                    for (int v : tmpFaces[j].idx)
                        if (v == op.org) { reject = true; break; }
                }
                if (reject) break;
            }
            if (!reject) {
                did_merge = true;
                faces.push_back(combined);
            }
        }
        if (!did_merge)
            for (int gi : group) faces.push_back(tmpFaces[gi]);
    }

    // unique edges (b3ConvexUtility.cpp:291-345): direction v[min] - v[max], normalised,
    // kept unless parallel or anti-parallel within 1e-6 per component to an earlier edge
    std::vector<F3> edges;
    for (auto& f : faces) {
        int nv = (int)f.idx.size();
        for (int j = 0; j < nv; j++) {
            int a = f.idx[j], b = f.idx[(j + 1) % nv];
            int v0 = std::max(a, b), v1 = std::min(a, b);
            F3 e = fnormalize(fsub(V[v1], V[v0]));
            bool found = false;
            for (auto& u : edges) {
                F3 d1 = fsub(u, e), d2 = fadd(u, e);
                bool z1 = !(std::fabs(d1.x) > 1e-6f || std::fabs(d1.y) > 1e-6f || std::fabs(d1.z) > 1e-6f);
                bool z2 = !(std::fabs(d2.x) > 1e-6f || std::fabs(d2.y) > 1e-6f || std::fabs(d2.z) > 1e-6f);
                if (z1 || z2) { found = true; break; }
            }
            if (!found) edges.push_back(e);
        }
    }

    for (auto& v : V) {
        out.vertices.push_back(v.x);
        out.vertices.push_back(v.y);
        out.vertices.push_back(v.z);
    }
    for (auto& f : faces) {
        for (int k = 0; k < 4; k++) out.planes.push_back(f.plane[k]);
        out.face_counts.push_back((int)f.idx.size());
        for (int v : f.idx) out.indices.push_back(v);
    }
    for (auto& e : edges) {
        out.edges.push_back(e.x);
        out.edges.push_back(e.y);
        out.edges.push_back(e.z);
    }
    // local centre = vertex mean (b3GpuNarrowPhase.cpp:324-329)
    F3 c = {0, 0, 0};
    for (auto& v : V) c = fadd(c, v);
    c = fscale(c, 1.f / (float)V.size());
    out.center[0] = c.x; out.center[1] = c.y; out.center[2] = c.z;
    return 0;
}

}  // namespace b3g
