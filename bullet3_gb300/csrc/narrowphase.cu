// Narrowphase: contact manifolds (b3Contact4Data, up to 4 points) for every overlapping pair.
//
// Reference functions restated (paths relative to the reference's src/):
//   hull-hull     b3ContactConvexConvexSAT          Bullet3Collision/NarrowPhaseCollision/shared/b3ContactConvexConvexSAT.h:403
//                 b3FindSeparatingAxis              .../shared/b3FindSeparatingAxis.h:55-195 (face axes of A, of B, exact edge x edge)
//                 b3ClipHullAgainstHull/b3ClipFace  .../shared/b3ContactConvexConvexSAT.h:20-259 (minDist -1, maxDist 0)
//                 b3ReduceContacts                  .../shared/b3ReduceContacts.h:4-87
//   plane-hull    computeContactPlaneConvex         Bullet3OpenCL/NarrowphaseCollision/b3ConvexHullContact.cpp:1272-1395
//   sphere-hull   computeContactSphereConvex        Bullet3OpenCL/NarrowphaseCollision/b3ConvexHullContact.cpp:2323-2470
//   sphere-sphere primitiveContactsKernel           Bullet3OpenCL/NarrowphaseCollision/kernels/primitiveContacts.cl:926-972
//   plane-sphere  computeContactPlaneSphere         same file :729-790
// A/B roles per shape pair follow the reference's dispatch (b3ConvexHullContact.cpp:2655-2735):
// the sphere / plane is always body A, the hull body B; hull-hull and sphere-sphere use the
// pair order (lower body index = A).
//
// GB300 design: pairs are bucketed by shape combination; the primitive cases run one thread
// per pair; hull-hull runs one warp per pair -- lanes split the face and edge-edge axes,
// vertex reads are warp-broadcast, the axis choice is a (depth, axis index) warp arg-min
// (first minimum wins, as in the sequential loop), clipping polygons live in shared memory.
// Each manifold is written to the slot of its pair; a scan over per-pair flags gives the
// manifold order (= pair order), so the contact list is deterministic.
#include <cfloat>

#include "common.cuh"
#include "world_internal.h"

namespace b3g {

static constexpr int NP_THREADS = 256;
static constexpr int CLIP_CAP = 64;

struct NPArgs {
    const b3gBody* bodies;
    const b3gCollidable* cols;
    const b3gHull* hulls;
    const uint32_t* face_dup;  // per hull: faces whose SAT axis repeats an earlier face's
    const b3gFace* faces;
    const int* indices;
    const b3gFloat4* verts;
    const b3gFloat4* edges;
    const b3gPair* pairs;
    const int* type_list;
    const int* type_count;
    b3gContact4* slots;
    int* flags;
    unsigned int* status;
    unsigned short friction_cmp;
    // compounds
    const b3gChildShape* children;
    const b3gAabb* local_aabbs;
    // concave meshes
    const b3gAabb* aabbs;  // world AABBs by body
    const b3gBvhInfo* bvh_infos;
    const b3gBvhNode* bvh_nodes;
};

__device__ __forceinline__ v3 ld3(const b3gFloat4* p) {
    float4 a = __ldg(reinterpret_cast<const float4*>(p));
    return mk3(a.x, a.y, a.z);
}
__device__ __forceinline__ float4 ldf4(const b3gFloat4* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ int sgn_index(const b3gBody* bodies, int i) { return bodies[i].invMass == 0.f ? -i : i; }

__device__ __forceinline__ void write_header(b3gContact4& c, const NPArgs& a, int bodyA, int bodyB, v3 n, int np) {
    c.worldNormalOnB = b3gFloat4{n.x, n.y, n.z, (float)np};
    c.restitutionCmp = 0;
    c.frictionCmp = a.friction_cmp;
    c.batchIdx = 0;
    c.bodyA = sgn_index(a.bodies, bodyA);
    c.bodyB = sgn_index(a.bodies, bodyB);
    c.childIndexA = -1;
    c.childIndexB = -1;
    c.unused1 = 0;
    c.unused2 = 0;
}

// b3ReduceContacts / extractManifoldSequentialGlobal: deepest point + extremes along +-u, +-v.
// p: xyz + w = depth. idx receives 4 indices (pre-set to 0,1,2,3 by the caller's convention).
__device__ int reduce_contacts(const float4* p, int n, v3 nearNormal, int idx[4]) {
    idx[0] = 0; idx[1] = 1; idx[2] = 2; idx[3] = 3;
    if (n == 0) return 0;
    if (n <= 4) return n;
    if (n > 64) n = 64;
    float cx = 0.f, cy = 0.f, cz = 0.f;
    for (int i = 0; i < n; i++) {
        cx = cx + p[i].x;
        cy = cy + p[i].y;
        cz = cz + p[i].z;
    }
    float inv = 1.0f / (float)n;
    cx = cx * inv; cy = cy * inv; cz = cz * inv;
    v3 center = mk3(cx, cy, cz);
    v3 aVector = mk3(p[0].x, p[0].y, p[0].z) - center;
    v3 u = cross3(nearNormal, aVector);
    v3 v = cross3(nearNormal, u);
    u = normalize3(u);
    v = normalize3(v);
    float minW = FLT_MAX;
    int minIndex = -1;
    float m0 = FLT_MIN, m1 = FLT_MIN, m2 = FLT_MIN, m3 = FLT_MIN;
    v3 nu = -u, nv = -v;
    for (int ie = 0; ie < n; ie++) {
        if (p[ie].w < minW) {
            minW = p[ie].w;
            minIndex = ie;
        }
        v3 r = mk3(p[ie].x, p[ie].y, p[ie].z) - center;
        float f;
        f = dot3(u, r);
        if (f < m0) { m0 = f; idx[0] = ie; }
        f = dot3(nu, r);
        if (f < m1) { m1 = f; idx[1] = ie; }
        f = dot3(v, r);
        if (f < m2) { m2 = f; idx[2] = ie; }
        f = dot3(nv, r);
        if (f < m3) { m3 = f; idx[3] = ie; }
    }
    if (idx[0] != minIndex && idx[1] != minIndex && idx[2] != minIndex && idx[3] != minIndex) idx[0] = minIndex;
    return 4;
}

// ------------------------------------------------------------------ plane (A) vs hull (B)
// computeContactPlaneConvex (b3ConvexHullContact.cpp:1272-1395) for a hull at pose (posB, ornB):
// the points below the plane (reduced to 4), returns their count; nWorld = the plane's world normal
__device__ int plane_hull_points(const NPArgs& a, int bodyA, const b3gHull& hull, v3 posB, quat ornB, float4* pts,
                                 int idx[4], v3& nWorld) {
    const b3gBody& BA = a.bodies[bodyA];
    const b3gCollidable colA = a.cols[BA.collidableIdx];
    v3 posA = f4v3(BA.pos);
    quat ornA = f4q(BA.quat);
    float4 pe = ldf4(&a.faces[colA.shapeIndex].plane);
    v3 planeNormal = mk3(pe.x, pe.y, pe.z);
    float planeConstant = pe.w;
    m33 RA = qmat(ornA), RB = qmat(ornB);
    v3 planeNormalWorld = qrotq(ornA, planeNormal);
    // planeInConvex = inverse(convexWorld) * planeTransform: basis RB^T * RA (b3Transform order)
    v3 planeNormalInConvex = mmul(mmul33(mtrans(RB), RA), -planeNormal);
    int numPoints = 0;
    float maxDot = -1e30f;
    for (int i = 0; i < hull.numVertices; i++) {
        v3 vtx = ld3(&a.verts[hull.vertexOffset + i]);
        float curDot = dot3(vtx, planeNormalInConvex);
        if (curDot > maxDot) {
            maxDot = curDot;
            if (numPoints == 64) numPoints--;
        }
        if (numPoints < 64) {
            v3 vtxWorld = mmul(RB, vtx) + posB;
            v3 vtxInPlane = xform_inv(RA, posA, vtxWorld);
            float dist = dot3(planeNormal, vtxInPlane) - planeConstant;
            if (dist < 0.f) {
                pts[numPoints] = make_float4(vtxWorld.x, vtxWorld.y, vtxWorld.z, dist);
                numPoints++;
            }
        }
    }
    nWorld = planeNormalWorld;
    return reduce_contacts(pts, numPoints, planeNormalInConvex, idx);
}

__device__ void plane_hull(const NPArgs& a, int pairIdx, int bodyA, int bodyB) {
    const b3gBody& BB = a.bodies[bodyB];
    const b3gHull hull = a.hulls[a.cols[BB.collidableIdx].shapeIndex];
    float4 pts[64];
    int idx[4];
    v3 planeNormalWorld;
    const int nred = plane_hull_points(a, bodyA, hull, f4v3(BB.pos), f4q(BB.quat), pts, idx, planeNormalWorld);
    if (nred > 0) {
        b3gContact4& c = a.slots[pairIdx];
        write_header(c, a, bodyA, bodyB, -planeNormalWorld, nred);
        for (int i = 0; i < nred; i++) {
            float4 q = pts[idx[i]];
            c.worldPosB[i] = b3gFloat4{q.x, q.y, q.z, q.w};
        }
        a.flags[pairIdx] = 1;
    }
}

// ------------------------------------------------------------------ plane (A) vs sphere (B)
__device__ void plane_sphere(const NPArgs& a, int pairIdx, int bodyA, int bodyB) {
    const b3gBody& BA = a.bodies[bodyA];
    const b3gBody& BB = a.bodies[bodyB];
    float4 pe = ldf4(&a.faces[a.cols[BA.collidableIdx].shapeIndex].plane);
    float radius = a.cols[BB.collidableIdx].radius;
    v3 posA = f4v3(BA.pos), posB = f4v3(BB.pos);
    quat ornA = f4q(BA.quat), ornB = f4q(BB.quat);
    v3 n = mk3(pe.x, pe.y, pe.z);
    float planeConstant = pe.w;
    m33 RA = qmat(ornA), RB = qmat(ornB);
    // sphere point nearest the plane, expressed in the plane frame:
    // vtx1 = (RB^T RA)(-n) * r ; vtxInPlane = RA^T (RB vtx1 + posB - posA)
    v3 vtx1 = mtmul(RB, mmul(RA, -n)) * radius;
    v3 vtxInPlane = mtmul(RA, (mmul(RB, vtx1) + posB) - posA);
    float distance = dot3(n, vtxInPlane) - planeConstant;
    if (distance < 0.f) {
        v3 projected = vtxInPlane - distance * n;
        v3 world = mmul(RA, projected) + posA;
        v3 normalOnSurfaceB = mmul(RA, n);
        v3 pOnB = world + normalOnSurfaceB * distance;
        b3gContact4& c = a.slots[pairIdx];
        write_header(c, a, bodyA, bodyB, -normalOnSurfaceB, 1);
        c.worldPosB[0] = b3gFloat4{pOnB.x, pOnB.y, pOnB.z, distance};
        a.flags[pairIdx] = 1;
    }
}

// ------------------------------------------------------------------ sphere (A) vs hull (B)
__device__ bool point_in_polygon(v3 p, const b3gFace& face, const b3gFloat4* base, const int* indices, v3& out) {
    v3 plane = mk3(face.plane.x, face.plane.y, face.plane.z);
    if (face.numIndices < 2) return false;
    v3 b = ld3(&base[indices[face.indexOffset + face.numIndices - 1]]);
    for (int i = 0; i < face.numIndices; i++) {
        v3 a = b;
        b = ld3(&base[indices[face.indexOffset + i]]);
        v3 ab = b - a;
        v3 ap = p - a;
        v3 v = cross3(ab, plane);
        if (dot3(ap, v) > 0.f) {
            float ab_m2 = dot3(ab, ab);
            float rt = ab_m2 != 0.f ? dot3(ab, ap) / ab_m2 : 0.f;
            if (rt <= 0.f)
                out = a;
            else if (rt >= 1.f)
                out = b;
            else {
                float s = 1.f - rt;
                out = mk3(s * a.x + rt * b.x, s * a.y + rt * b.y, s * a.z + rt * b.z);
            }
            return false;
        }
    }
    return true;
}

__device__ void sphere_hull(const NPArgs& a, int pairIdx, int bodyA, int bodyB) {
    const b3gBody& BA = a.bodies[bodyA];
    const b3gBody& BB = a.bodies[bodyB];
    float radius = a.cols[BA.collidableIdx].radius;
    v3 spherePos1 = f4v3(BA.pos);
    v3 pos = f4v3(BB.pos);
    m33 R = qmat(f4q(BB.quat));
    v3 spherePos = xform_inv(R, pos, spherePos1);
    const b3gHull hull = a.hulls[a.cols[BB.collidableIdx].shapeIndex];
    v3 closest = mk3(0, 0, 0);
    float minDist = -1000000.f;
    bool bCollide = true;
    v3 localHitNormal = mk3(0, 0, 0);
    const b3gFloat4* base = &a.verts[hull.vertexOffset];
    for (int f = 0; f < hull.numFaces; f++) {
        const b3gFace face = a.faces[hull.faceOffset + f];
        v3 n = mk3(face.plane.x, face.plane.y, face.plane.z);
        float dist = dot3(n, spherePos) + face.plane.w;
        v3 pntReturn = spherePos - dist * n;
        if (dist > radius) {
            bCollide = false;
            break;
        }
        if (dist > 0.f) {
            v3 out;
            bool inPoly = point_in_polygon(spherePos, face, base, a.indices, out);
            if (inPoly) {
                if (dist > minDist) {
                    minDist = dist;
                    closest = pntReturn;
                    localHitNormal = n;
                }
            } else {
                v3 tmp = spherePos - out;
                float l2 = dot3(tmp, tmp);
                if (l2 < radius * radius) {
                    dist = sqrtf(l2);
                    if (dist > minDist) {
                        minDist = dist;
                        closest = out;
                        float inv = 1.0f / dist;  // b3Vector3 operator/ scales by the reciprocal
                        localHitNormal = mk3(tmp.x * inv, tmp.y * inv, tmp.z * inv);
                    }
                } else {
                    bCollide = false;
                    break;
                }
            }
        } else {
            if (dist > minDist) {
                minDist = dist;
                closest = pntReturn;
                localHitNormal = n;
            }
        }
    }
    if (bCollide && minDist > -10000.f) {
        v3 normalOnSurfaceB = mmul(R, localHitNormal);
        v3 pOnB = mmul(R, closest) + pos;
        float actualDepth = minDist - radius;
        if (actualDepth < 0.f) {
            b3gContact4& c = a.slots[pairIdx];
            write_header(c, a, bodyA, bodyB, normalOnSurfaceB, 1);
            c.worldPosB[0] = b3gFloat4{pOnB.x, pOnB.y, pOnB.z, actualDepth};
            a.flags[pairIdx] = 1;
        }
    }
}

// ------------------------------------------------------------------ sphere vs sphere
__device__ void sphere_sphere(const NPArgs& a, int pairIdx, int bodyA, int bodyB) {
    const b3gBody& BA = a.bodies[bodyA];
    const b3gBody& BB = a.bodies[bodyB];
    float rA = a.cols[BA.collidableIdx].radius, rB = a.cols[BB.collidableIdx].radius;
    v3 posA = f4v3(BA.pos), posB = f4v3(BB.pos);
    v3 diff = posA - posB;
    float len = sqrtf(dot3(diff, diff));
    if (len <= (rA + rB)) {
        float dist = len - (rA + rB);
        v3 n = mk3(1.f, 0.f, 0.f);
        if (len > 0.00001f) n = mk3(diff.x / len, diff.y / len, diff.z / len);
        v3 cp = posB + n * rB;
        b3gContact4& c = a.slots[pairIdx];
        write_header(c, a, bodyA, bodyB, n, 1);
        c.worldPosB[0] = b3gFloat4{cp.x, cp.y, cp.z, dist};
        a.flags[pairIdx] = 1;
    }
}

__device__ __forceinline__ int shape_type(const NPArgs& a, int body) { return a.cols[a.bodies[body].collidableIdx].shapeType; }

// All four primitive pair types (plane-hull, sphere-hull, sphere-sphere, plane-sphere) in one
// launch: work item t walks the concatenation of the four type lists.
__global__ void __launch_bounds__(NP_THREADS) k_primitive_pairs(NPArgs a, int max_pairs) {
    const int c1 = a.type_count[PT_PLANE_HULL], c2 = a.type_count[PT_SPHERE_HULL],
              c3 = a.type_count[PT_SPHERE_SPHERE], c4 = a.type_count[PT_PLANE_SPHERE];
    const int n = c1 + c2 + c3 + c4;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int type, k;
        if (t < c1) { type = PT_PLANE_HULL; k = t; }
        else if (t < c1 + c2) { type = PT_SPHERE_HULL; k = t - c1; }
        else if (t < c1 + c2 + c3) { type = PT_SPHERE_SPHERE; k = t - c1 - c2; }
        else { type = PT_PLANE_SPHERE; k = t - c1 - c2 - c3; }
        int p = a.type_list[(size_t)type * max_pairs + k];
        b3gPair pr = a.pairs[p];
        int A = pr.x, B = pr.y;
        int ta = shape_type(a, A);
        if (type == PT_PLANE_HULL) {
            if (ta == B3G_SHAPE_PLANE) plane_hull(a, p, A, B);
            else plane_hull(a, p, B, A);
        } else if (type == PT_PLANE_SPHERE) {
            if (ta == B3G_SHAPE_PLANE) plane_sphere(a, p, A, B);
            else plane_sphere(a, p, B, A);
        } else if (type == PT_SPHERE_HULL) {
            if (ta == B3G_SHAPE_SPHERE) sphere_hull(a, p, A, B);
            else sphere_hull(a, p, B, A);
        } else if (type == PT_SPHERE_SPHERE) {
            sphere_sphere(a, p, A, B);
        }
    }
}

// ------------------------------------------------------------------ hull vs hull, one warp per pair
struct AxisBest {
    float d;
    int idx;
};
__device__ __forceinline__ AxisBest warp_argmin(AxisBest x) {
    for (int o = 16; o; o >>= 1) {
        float od = __shfl_xor_sync(0xffffffffu, x.d, o);
        int oi = __shfl_xor_sync(0xffffffffu, x.idx, o);
        if (od < x.d || (od == x.d && oi < x.idx)) {
            x.d = od;
            x.idx = oi;
        }
    }
    return x;
}
__device__ __forceinline__ AxisBest warp_argmax(AxisBest x) {
    for (int o = 16; o; o >>= 1) {
        float od = __shfl_xor_sync(0xffffffffu, x.d, o);
        int oi = __shfl_xor_sync(0xffffffffu, x.idx, o);
        if (od > x.d || (od == x.d && oi < x.idx)) {
            x.d = od;
            x.idx = oi;
        }
    }
    return x;
}

// b3ProjectAxis: project the hull's local vertices on the axis rotated into its frame.
__device__ __forceinline__ void project(const b3gFloat4* verts, int nv, v3 pos, quat orn, v3 dir, float& mn,
                                        float& mx) {
    v3 localDir = qrotq(qconj(orn), dir);
    float offset = dot3(pos, dir);
    mn = FLT_MAX;
    mx = -FLT_MAX;
    for (int i = 0; i < nv; i++) {
        float dp = dot3(ld3(&verts[i]), localDir);
        if (dp < mn) mn = dp;
        if (dp > mx) mx = dp;
    }
    if (mn > mx) {
        float t = mn; mn = mx; mx = t;
    }
    mn = mn + offset;
    mx = mx + offset;
}

// Face axes k that repeat an earlier face axis of the same hull (exactly opposite normals): the
// same axis after the sign flip and the same overlap, so they can never be the first minimum and
// never separate where the earlier one did not.
__device__ __forceinline__ bool dup_face_axis(int k, int nfA, uint32_t dupA, uint32_t dupB) {
    if (k < nfA) return k < 32 && ((dupA >> k) & 1u);
    const int f = k - nfA;
    return f < 32 && ((dupB >> f) & 1u);
}

// Axis k of the SAT sequence: faces of A, faces of B, then edges (e0 of A major, e1 of B minor).
// Returns false when the edge cross product is almost zero (axis skipped).
__device__ __forceinline__ bool sat_axis(int k, const b3gHull& hA, const b3gHull& hB, const b3gFace* faces,
                                         const b3gFloat4* edges, quat qA, quat qB, v3 deltaC2, v3& axis) {
    if (k < hA.numFaces) {
        v3 n = ld3(&faces[hA.faceOffset + k].plane);
        axis = qrotq(qA, n);
    } else if (k < hA.numFaces + hB.numFaces) {
        v3 n = ld3(&faces[hB.faceOffset + (k - hA.numFaces)].plane);
        axis = qrotq(qB, n);
    } else {
        int e = k - hA.numFaces - hB.numFaces;
        int e0 = e / hB.numUniqueEdges, e1 = e - e0 * hB.numUniqueEdges;
        v3 w0 = qrotq(qA, ld3(&edges[hA.uniqueEdgesOffset + e0]));
        v3 w1 = qrotq(qB, ld3(&edges[hB.uniqueEdgesOffset + e1]));
        v3 c = cross3(w0, w1);
        // b3IsAlmostZero compares |c| against the double 1e-6
        if (!((double)fabsf(c.x) > 1e-6 || (double)fabsf(c.y) > 1e-6 || (double)fabsf(c.z) > 1e-6)) return false;
        axis = normalize3(c);
    }
    if (dot3(deltaC2, axis) < 0.f) axis = -axis;
    return true;
}

// Sutherland-Hodgman clip of a polygon against one plane (b3ClipFace)
__device__ int clip_face(const float4* in, int nin, v3 n, float eq, float4* out, unsigned int* status) {
    if (nin < 2) return 0;
    int nout = 0;
    float4 first = in[nin - 1];
    float ds = dot3(n, mk3(first.x, first.y, first.z)) + eq;
    for (int ve = 0; ve < nin; ve++) {
        float4 end = in[ve];
        float de = dot3(n, mk3(end.x, end.y, end.z)) + eq;
        if (ds < 0.f) {
            if (de < 0.f) {
                if (nout < CLIP_CAP) out[nout++] = end; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
            } else {
                float t = ds * 1.f / (ds - de);
                float4 l = make_float4(first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                                       first.z + (end.z - first.z) * t, 0.f);
                if (nout < CLIP_CAP) out[nout++] = l; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
            }
        } else {
            if (de < 0.f) {
                float t = ds * 1.f / (ds - de);
                float4 l = make_float4(first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                                       first.z + (end.z - first.z) * t, 0.f);
                if (nout < CLIP_CAP) out[nout++] = l; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
                if (nout < CLIP_CAP) out[nout++] = end; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
            }
        }
        first = end;
        ds = de;
    }
    return nout;
}

static constexpr int HH_WARPS = 4;

__global__ void __launch_bounds__(HH_WARPS * 32) k_hull_hull(NPArgs a, int max_pairs) {
    __shared__ float4 s_poly[HH_WARPS][2][CLIP_CAP];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int n = a.type_count[PT_HULL_HULL];
    const int* list = a.type_list + (size_t)PT_HULL_HULL * max_pairs;
    const int nwarps = gridDim.x * HH_WARPS;
    for (int t = blockIdx.x * HH_WARPS + wib; t < n; t += nwarps) {
        const int p = list[t];
        const b3gPair pr = a.pairs[p];
        const int iA = pr.x, iB = pr.y;
        const b3gBody& BA = a.bodies[iA];
        const b3gBody& BB = a.bodies[iB];
        const b3gHull hA = a.hulls[a.cols[BA.collidableIdx].shapeIndex];
        const b3gHull hB = a.hulls[a.cols[BB.collidableIdx].shapeIndex];
        const v3 posA = f4v3(BA.pos), posB = f4v3(BB.pos);
        const quat qA = f4q(BA.quat), qB = f4q(BB.quat);
        const m33 RA = qmat(qA), RB = qmat(qB);
        const v3 c0 = mmul(RA, f4v3(hA.localCenter)) + posA;
        const v3 c1 = mmul(RB, f4v3(hB.localCenter)) + posB;
        const v3 deltaC2 = c0 - c1;
        const int naxes = hA.numFaces + hB.numFaces + hA.numUniqueEdges * hB.numUniqueEdges;
        const int nfaces = hA.numFaces + hB.numFaces;
        const uint32_t dupA = __ldg(&a.face_dup[a.cols[BA.collidableIdx].shapeIndex]);
        const uint32_t dupB = __ldg(&a.face_dup[a.cols[BB.collidableIdx].shapeIndex]);
        AxisBest best{FLT_MAX, 0x7fffffff};
        bool separated = false;
        const b3gFloat4* vA = &a.verts[hA.vertexOffset];
        const b3gFloat4* vB = &a.verts[hB.vertexOffset];
        // 32 axes per round; a separating axis found by any lane ends the test (the pair has no
        // contact whichever axis separates it, so the reference's early return gives the same result)
        for (int k0 = 0; k0 < naxes; k0 += 32) {
            const int k = k0 + lane;
            v3 axis;
            if (k < naxes && !(k < nfaces && dup_face_axis(k, hA.numFaces, dupA, dupB)) &&
                sat_axis(k, hA, hB, a.faces, a.edges, qA, qB, deltaC2, axis)) {
                float min0, max0, min1, max1;
                project(vA, hA.numVertices, posA, qA, axis, min0, max0);
                project(vB, hB.numVertices, posB, qB, axis, min1, max1);
                if (max0 < min1 || max1 < min0) {
                    separated = true;
                } else {
                    float d0 = max0 - min1, d1 = max1 - min0;
                    float depth = d0 < d1 ? d0 : d1;
                    if (depth < best.d || (depth == best.d && k < best.idx)) {
                        best.d = depth;
                        best.idx = k;
                    }
                }
            }
            if (__any_sync(0xffffffffu, separated)) break;
        }
        if (__any_sync(0xffffffffu, separated)) continue;
        best = warp_argmin(best);
        if (best.idx == 0x7fffffff) continue;  // no usable axis (degenerate)
        v3 sep;
        sat_axis(best.idx, hA, hB, a.faces, a.edges, qA, qB, deltaC2, sep);
        if (dot3(-deltaC2, sep) > 0.0f) sep = -sep;

        // b3ClipHullHullSingle clips with the orientation round-tripped through a b3Transform
        // (setRotation then getRotation, b3ContactConvexConvexSAT.h:315-330)
        const quat cA = quat_from_mat(RA), cB = quat_from_mat(RB);
        const m33 CA = qmat(cA), CB = qmat(cB);
        // incident face of B: max dot(world normal, sep), first max wins
        AxisBest fb{-FLT_MAX, 0x7fffffff};
        for (int f = lane; f < hB.numFaces; f += 32) {
            float d = dot3(qrotq(cB, ld3(&a.faces[hB.faceOffset + f].plane)), sep);
            if (d > fb.d || (d == fb.d && f < fb.idx)) { fb.d = d; fb.idx = f; }
        }
        fb = warp_argmax(fb);
        // reference face of A: min dot(world normal, sep), first min wins
        AxisBest fa{FLT_MAX, 0x7fffffff};
        for (int f = lane; f < hA.numFaces; f += 32) {
            float d = dot3(qrotq(cA, ld3(&a.faces[hA.faceOffset + f].plane)), sep);
            if (d < fa.d || (d == fa.d && f < fa.idx)) { fa.d = d; fa.idx = f; }
        }
        fa = warp_argmin(fa);
        if (fb.idx == 0x7fffffff || fa.idx == 0x7fffffff) continue;

        if (lane == 0) {
            float4* pin = s_poly[wib][0];
            float4* pout = s_poly[wib][1];
            const b3gFace polyB = a.faces[hB.faceOffset + fb.idx];
            int nin = 0;
            for (int e = 0; e < polyB.numIndices && e < CLIP_CAP; e++) {
                v3 w = mmul(CB, ld3(&vB[a.indices[polyB.indexOffset + e]])) + posB;
                pin[nin++] = make_float4(w.x, w.y, w.z, 0.f);
            }
            const b3gFace polyA = a.faces[hA.faceOffset + fa.idx];
            const v3 planeNormalA = mk3(polyA.plane.x, polyA.plane.y, polyA.plane.z);
            const v3 worldPlaneAnormal1 = qrotq(cA, planeNormalA);
            const int nva = polyA.numIndices;
            for (int e0 = 0; e0 < nva; e0++) {
                v3 va = ld3(&vA[a.indices[polyA.indexOffset + e0]]);
                v3 vb = ld3(&vA[a.indices[polyA.indexOffset + ((e0 + 1) % nva)]]);
                v3 worldEdge0 = qrotq(cA, va - vb);
                v3 planeNormalWS1 = -cross3(worldEdge0, worldPlaneAnormal1);
                v3 worldA1 = mmul(CA, va) + posA;
                float planeEqWS1 = -dot3(worldA1, planeNormalWS1);
                int nout = clip_face(pin, nin, planeNormalWS1, planeEqWS1, pout, a.status);
                float4* tmp = pout; pout = pin; pin = tmp;
                nin = nout;
            }
            // keep points behind the reference face; depth clamped at minDist=-1, kept if <= maxDist=0
            const float planeEqWS = polyA.plane.w - dot3(worldPlaneAnormal1, posA);
            int ncont = 0;
            for (int i = 0; i < nin; i++) {
                float depth = dot3(worldPlaneAnormal1, mk3(pin[i].x, pin[i].y, pin[i].z)) + planeEqWS;
                if (depth <= -1.0f) depth = -1.0f;
                if (depth <= 0.0f) pout[ncont++] = make_float4(pin[i].x, pin[i].y, pin[i].z, depth);
            }
            if (ncont > 0) {
                int idx[4];
                int np = reduce_contacts(pout, ncont, sep, idx);
                b3gContact4& c = a.slots[p];
                write_header(c, a, iA, iB, sep, np);
                for (int q = 0; q < np; q++) {
                    float4 v = pout[idx[q]];
                    c.worldPosB[q] = b3gFloat4{v.x, v.y, v.z, v.w};
                }
                a.flags[p] = 1;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ hull vs hull, one thread per pair
// For small hulls (every face <= SMALL_FACE_VERTS vertices): the sequential form of the same
// SAT -- axes in reference order, return at the first separating axis (b3FindSeparatingAxis
// returns false there) -- then the same clip and reduction.  Bit-identical to the warp path.
static constexpr int SMALL_CLIP = 2 * B3G_SMALL_FACE_VERTS;

__global__ void __launch_bounds__(NP_THREADS, 3) k_hull_hull_small(NPArgs a, int max_pairs) {
    const int n = a.type_count[PT_HULL_HULL_SMALL];
    const int* list = a.type_list + (size_t)PT_HULL_HULL_SMALL * max_pairs;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int p = list[t];
        const b3gPair pr = a.pairs[p];
        const int iA = pr.x, iB = pr.y;
        const b3gBody& BA = a.bodies[iA];
        const b3gBody& BB = a.bodies[iB];
        const b3gHull hA = a.hulls[a.cols[BA.collidableIdx].shapeIndex];
        const b3gHull hB = a.hulls[a.cols[BB.collidableIdx].shapeIndex];
        const v3 posA = f4v3(BA.pos), posB = f4v3(BB.pos);
        const quat qA = f4q(BA.quat), qB = f4q(BB.quat);
        const m33 RA = qmat(qA), RB = qmat(qB);
        const v3 deltaC2 = (mmul(RA, f4v3(hA.localCenter)) + posA) - (mmul(RB, f4v3(hB.localCenter)) + posB);
        const b3gFloat4* vA = &a.verts[hA.vertexOffset];
        const b3gFloat4* vB = &a.verts[hB.vertexOffset];
        const int naxes = hA.numFaces + hB.numFaces + hA.numUniqueEdges * hB.numUniqueEdges;
        const int nfaces = hA.numFaces + hB.numFaces;
        const uint32_t dupA = __ldg(&a.face_dup[a.cols[BA.collidableIdx].shapeIndex]);
        const uint32_t dupB = __ldg(&a.face_dup[a.cols[BB.collidableIdx].shapeIndex]);
        float dmin = FLT_MAX;
        v3 sep = mk3(0.f, 0.f, 0.f);
        bool separated = false;
        for (int k = 0; k < naxes; k++) {
            v3 axis;
            if (k < nfaces && dup_face_axis(k, hA.numFaces, dupA, dupB)) continue;
            if (!sat_axis(k, hA, hB, a.faces, a.edges, qA, qB, deltaC2, axis)) continue;
            float min0, max0, min1, max1;
            project(vA, hA.numVertices, posA, qA, axis, min0, max0);
            project(vB, hB.numVertices, posB, qB, axis, min1, max1);
            if (max0 < min1 || max1 < min0) {
                separated = true;
                break;
            }
            float d0 = max0 - min1, d1 = max1 - min0;
            float depth = d0 < d1 ? d0 : d1;
            if (depth < dmin) {
                dmin = depth;
                sep = axis;
            }
        }
        if (separated || dmin == FLT_MAX) continue;
        if (dot3(-deltaC2, sep) > 0.0f) sep = -sep;
        const quat cA = quat_from_mat(RA), cB = quat_from_mat(RB);
        const m33 CA = qmat(cA), CB = qmat(cB);
        int fbi = -1, fai = -1;
        float dmax = -FLT_MAX, dmn = FLT_MAX;
        for (int f = 0; f < hB.numFaces; f++) {
            float d = dot3(qrotq(cB, ld3(&a.faces[hB.faceOffset + f].plane)), sep);
            if (d > dmax) { dmax = d; fbi = f; }
        }
        for (int f = 0; f < hA.numFaces; f++) {
            float d = dot3(qrotq(cA, ld3(&a.faces[hA.faceOffset + f].plane)), sep);
            if (d < dmn) { dmn = d; fai = f; }
        }
        if (fbi < 0 || fai < 0) continue;
        float4 buf0[SMALL_CLIP], buf1[SMALL_CLIP];
        float4* pin = buf0;
        float4* pout = buf1;
        const b3gFace polyB = a.faces[hB.faceOffset + fbi];
        int nin = 0;
        for (int e = 0; e < polyB.numIndices && e < SMALL_CLIP; e++) {
            v3 w = mmul(CB, ld3(&vB[a.indices[polyB.indexOffset + e]])) + posB;
            pin[nin++] = make_float4(w.x, w.y, w.z, 0.f);
        }
        const b3gFace polyA = a.faces[hA.faceOffset + fai];
        const v3 worldPlaneAnormal1 = qrotq(cA, mk3(polyA.plane.x, polyA.plane.y, polyA.plane.z));
        const int nva = polyA.numIndices;
        for (int e0 = 0; e0 < nva; e0++) {
            v3 va = ld3(&vA[a.indices[polyA.indexOffset + e0]]);
            v3 vb = ld3(&vA[a.indices[polyA.indexOffset + ((e0 + 1) % nva)]]);
            v3 worldEdge0 = qrotq(cA, va - vb);
            v3 planeNormalWS1 = -cross3(worldEdge0, worldPlaneAnormal1);
            v3 worldA1 = mmul(CA, va) + posA;
            float planeEqWS1 = -dot3(worldA1, planeNormalWS1);
            // a convex polygon clipped by one plane gains at most one vertex: nin + 1 <= SMALL_CLIP
            int nout = 0;
            if (nin >= 2) {
                float4 first = pin[nin - 1];
                float ds = dot3(planeNormalWS1, mk3(first.x, first.y, first.z)) + planeEqWS1;
                for (int ve = 0; ve < nin; ve++) {
                    float4 end = pin[ve];
                    float de = dot3(planeNormalWS1, mk3(end.x, end.y, end.z)) + planeEqWS1;
                    if (ds < 0.f) {
                        if (de < 0.f) {
                            if (nout < SMALL_CLIP) pout[nout++] = end;
                        } else {
                            float tt = ds * 1.f / (ds - de);
                            if (nout < SMALL_CLIP)
                                pout[nout++] = make_float4(first.x + (end.x - first.x) * tt,
                                                           first.y + (end.y - first.y) * tt,
                                                           first.z + (end.z - first.z) * tt, 0.f);
                        }
                    } else if (de < 0.f) {
                        float tt = ds * 1.f / (ds - de);
                        if (nout < SMALL_CLIP)
                            pout[nout++] = make_float4(first.x + (end.x - first.x) * tt,
                                                       first.y + (end.y - first.y) * tt,
                                                       first.z + (end.z - first.z) * tt, 0.f);
                        if (nout < SMALL_CLIP) pout[nout++] = end;
                    }
                    first = end;
                    ds = de;
                }
            }
            float4* tmp = pout; pout = pin; pin = tmp;
            nin = nout;
        }
        const float planeEqWS = polyA.plane.w - dot3(worldPlaneAnormal1, posA);
        int ncont = 0;
        for (int i = 0; i < nin; i++) {
            float depth = dot3(worldPlaneAnormal1, mk3(pin[i].x, pin[i].y, pin[i].z)) + planeEqWS;
            if (depth <= -1.0f) depth = -1.0f;
            if (depth <= 0.0f) pout[ncont++] = make_float4(pin[i].x, pin[i].y, pin[i].z, depth);
        }
        if (ncont > 0) {
            int idx[4];
            int np = reduce_contacts(pout, ncont, sep, idx);
            b3gContact4& c = a.slots[p];
            write_header(c, a, iA, iB, sep, np);
            for (int q = 0; q < np; q++) {
                float4 v = pout[idx[q]];
                c.worldPosB[q] = b3gFloat4{v.x, v.y, v.z, v.w};
            }
            a.flags[p] = 1;
        }
    }
}

// manifold list in pair order + pair.z = manifold index + point count
__global__ void k_manifold_list(const int* __restrict__ flags, const int* __restrict__ cidx,
                                const int* __restrict__ d_nslots, const int* __restrict__ d_np,
                                const b3gContact4* __restrict__ slots, b3gPair* __restrict__ pairs,
                                int* __restrict__ manifold_pair, int* __restrict__ num_points) {
    const int ns = *d_nslots, np = *d_np;  // slots: the pairs', then the compound child pairs'
    int local = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ns; p += gridDim.x * blockDim.x) {
        if (flags[p]) {
            int m = cidx[p];
            manifold_pair[m] = p;
            if (p < np) pairs[p].z = m;
            local += (int)slots[p].worldNormalOnB.w;
        }
    }
    for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(num_points, local);
}

__global__ void k_compact_contacts(const int* __restrict__ d_nc, const int* __restrict__ manifold_pair,
                                   const b3gContact4* __restrict__ slots, b3gContact4* __restrict__ out) {
    const int nc = *d_nc;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nc; m += gridDim.x * blockDim.x)
        out[m] = slots[manifold_pair[m]];
}

// ------------------------------------------------------------------ compound shapes
// A pair with a compound (SHAPE_COMPOUND_OF_CONVEX_HULLS) expands into child pairs in (pair, child
// of A, child of B) order -- the set of findCompoundPairsKernel (b3ConvexHullContact.cpp:1419-1775):
// compound-compound the children whose world AABBs overlap (the reference walks quantized child
// BVHs, whose conservative boxes add only child pairs that cannot touch), compound against another
// shape every child.  Each child pair has its own manifold slot after the pair slots.

// child pose: newPos = b3QuatRotate(orn, childPos) + pos, newOrn = b3QuatMul(orn, childOrn)
// (processCompoundPairsKernel, b3ConvexHullContact.cpp:1813-1829)
__device__ __forceinline__ void child_pose(const b3gBody& b, const b3gChildShape& ch, v3& pos, quat& orn) {
    const quat q = f4q(b.quat);
    pos = qrotq(q, f4v3(ch.childPosition)) + f4v3(b.pos);
    orn = qmul(q, f4q(ch.childOrientation));
}

__device__ __forceinline__ bool aabb_overlap(v3 amn, v3 amx, v3 bmn, v3 bmx) {
    return amn.x <= bmx.x && bmn.x <= amx.x && amn.y <= bmx.y && bmn.y <= amx.y && amn.z <= bmx.z && bmn.z <= amx.z;
}

// the child pairs of pair p: counted (out == nullptr), or written at out[0..cap)
__device__ int compound_child_pairs(const NPArgs& a, int p, int4* out, int cap) {
    const b3gPair pr = a.pairs[p];
    const int A = pr.x, B = pr.y;
    const b3gBody& BA = a.bodies[A];
    const b3gBody& BB = a.bodies[B];
    const b3gCollidable cA = a.cols[BA.collidableIdx], cB = a.cols[BB.collidableIdx];
    const bool compA = cA.shapeType == B3G_SHAPE_COMPOUND, compB = cB.shapeType == B3G_SHAPE_COMPOUND;
    if (!compA && !compB) return 0;
    if (BA.invMass == 0.f && BB.invMass == 0.f) return 0;  // findCompoundPairsKernel :1446
    int n = 0;
    if (compA && compB) {
        for (int i = 0; i < cA.numChildShapes; i++) {
            const b3gChildShape chA = a.children[cA.shapeIndex + i];
            v3 pA, mnA, mxA;
            quat qA;
            child_pose(BA, chA, pA, qA);
            transform_aabb(a.local_aabbs[chA.shapeIndex], pA, qA, 0.f, mnA, mxA);
            for (int k = 0; k < cB.numChildShapes; k++) {
                const b3gChildShape chB = a.children[cB.shapeIndex + k];
                v3 pB, mnB, mxB;
                quat qB;
                child_pose(BB, chB, pB, qB);
                transform_aabb(a.local_aabbs[chB.shapeIndex], pB, qB, 0.f, mnB, mxB);
                if (!aabb_overlap(mnA, mxA, mnB, mxB)) continue;
                if (out && n < cap) out[n] = make_int4(A, B, cA.shapeIndex + i, cB.shapeIndex + k);
                n++;
            }
        }
    } else if (compA) {
        for (int i = 0; i < cA.numChildShapes; i++) {
            if (out && n < cap) out[n] = make_int4(A, B, cA.shapeIndex + i, -1);
            n++;
        }
    } else {
        for (int k = 0; k < cB.numChildShapes; k++) {
            if (out && n < cap) out[n] = make_int4(A, B, -1, cB.shapeIndex + k);
            n++;
        }
    }
    return n;
}

__global__ void k_compound_count(NPArgs a, const int* __restrict__ d_np, int* __restrict__ counts) {
    const int np = *d_np;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        counts[p] = compound_child_pairs(a, p, nullptr, 0);
}

// an expansion's total clamped to its capacity (the overflow flag beyond it)
__global__ void k_clamp_total(int* __restrict__ d_total, int cap, unsigned int* __restrict__ status) {
    const int total = *d_total;
    if (total > cap) atomicOr(status, B3G_FLAG_CONTACT_OVERFLOW);
    *d_total = total < cap ? total : cap;
}

// manifold slots: the pairs', the compound child pairs', the concave triangle-convex pairs'
__global__ void k_slot_total(const int* __restrict__ d_np, const int* __restrict__ d_J, const int* __restrict__ d_K,
                             int* __restrict__ d_slots) {
    *d_slots = *d_np + (d_J ? *d_J : 0) + (d_K ? *d_K : 0);
}

__global__ void k_compound_expand(NPArgs a, const int* __restrict__ d_np, const int* __restrict__ offsets,
                                  int4* __restrict__ child_pairs, int cap) {
    const int np = *d_np;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int o = offsets[p];
        if (o < cap) compound_child_pairs(a, p, child_pairs + o, cap - o);
    }
}

// findSeparatingAxis (b3ConvexHullContact.cpp:562-700): face normals of A, of B, edge-edge axes,
// returning at the first separating axis; sep = the smallest overlap's axis, pointing from B to A
__device__ bool find_sep_full(const NPArgs& a, const b3gHull& hA, const b3gHull& hB, v3 posA, quat qA, v3 posB,
                              quat qB, v3& sep) {
    const v3 deltaC2 = (mmul(qmat(qA), f4v3(hA.localCenter)) + posA) - (mmul(qmat(qB), f4v3(hB.localCenter)) + posB);
    const b3gFloat4* vA = &a.verts[hA.vertexOffset];
    const b3gFloat4* vB = &a.verts[hB.vertexOffset];
    float dmin = FLT_MAX;
    for (int i = 0; i < hA.numFaces + hB.numFaces; i++) {
        v3 n = i < hA.numFaces ? qrotq(qA, ld3(&a.faces[hA.faceOffset + i].plane))
                               : qrotq(qB, ld3(&a.faces[hB.faceOffset + (i - hA.numFaces)].plane));
        if (dot3(deltaC2, n) < 0.f) n = -n;
        float min0, max0, min1, max1;
        project(vA, hA.numVertices, posA, qA, n, min0, max0);
        project(vB, hB.numVertices, posB, qB, n, min1, max1);
        if (max0 < min1 || max1 < min0) return false;
        const float d0 = max0 - min1, d1 = max1 - min0;
        const float d = d0 < d1 ? d0 : d1;
        if (d < dmin) { dmin = d; sep = n; }
    }
    for (int e0 = 0; e0 < hA.numUniqueEdges; e0++) {
        const v3 w0 = qrotq(qA, ld3(&a.edges[hA.uniqueEdgesOffset + e0]));
        for (int e1 = 0; e1 < hB.numUniqueEdges; e1++) {
            const v3 w1 = qrotq(qB, ld3(&a.edges[hB.uniqueEdgesOffset + e1]));
            v3 c = cross3(w0, w1);
            if (!((double)fabsf(c.x) > 1e-6 || (double)fabsf(c.y) > 1e-6 || (double)fabsf(c.z) > 1e-6)) continue;
            c = normalize3(c);
            if (dot3(deltaC2, c) < 0.f) c = -c;
            float min0, max0, min1, max1;
            project(vA, hA.numVertices, posA, qA, c, min0, max0);
            project(vB, hB.numVertices, posB, qB, c, min1, max1);
            if (max0 < min1 || max1 < min0) return false;
            const float d0 = max0 - min1, d1 = max1 - min0;
            const float d = d0 < d1 ? d0 : d1;
            if (d < dmin) { dmin = d; sep = c; }
        }
    }
    if (dmin == FLT_MAX) return false;
    if (dot3(-deltaC2, sep) > 0.0f) sep = -sep;
    return true;
}

// One child pair per thread (slot = pair count + child pair index): every slot's flag cleared, and
// computeContactPlaneCompound (b3ConvexHullContact.cpp:2182-2321) for a plane against a child.
// Two hulls are k_compound_hull_hull's; compound children against spheres give nothing.
__global__ void __launch_bounds__(NP_THREADS, 2) k_compound_contacts(NPArgs a, const int* __restrict__ d_np,
                                                                     const int* __restrict__ d_J,
                                                                     const int4* __restrict__ child_pairs) {
    const int P = *d_np, J = *d_J;
    const unsigned short fr07 = (unsigned short)(0.7f * 0xffff);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < J; j += gridDim.x * blockDim.x) {
        const int slot = P + j;
        a.flags[slot] = 0;
        const int4 cp = child_pairs[j];
        const b3gBody& BA = a.bodies[cp.x];
        const b3gBody& BB = a.bodies[cp.y];
        v3 posA = f4v3(BA.pos), posB = f4v3(BB.pos);
        quat qA = f4q(BA.quat), qB = f4q(BB.quat);
        int colA = BA.collidableIdx, colB = BB.collidableIdx;
        if (cp.z >= 0) {
            const b3gChildShape ch = a.children[cp.z];
            colA = ch.shapeIndex;
            child_pose(BA, ch, posA, qA);
        }
        if (cp.w >= 0) {
            const b3gChildShape ch = a.children[cp.w];
            colB = ch.shapeIndex;
            child_pose(BB, ch, posB, qB);
        }
        const b3gCollidable cA = a.cols[colA], cB = a.cols[colB];
        b3gContact4& c = a.slots[slot];
        // two hulls: k_compound_hull_hull, a warp per child pair
        if (cA.shapeType == B3G_SHAPE_CONVEX_HULL && cB.shapeType == B3G_SHAPE_CONVEX_HULL) continue;
        {
            // a plane against a child: the plane body first in the manifold, the child's hull at its pose
            int plane = -1, comp = -1, child = -1;
            v3 pos;
            quat q;
            if (cA.shapeType == B3G_SHAPE_PLANE && cB.shapeType == B3G_SHAPE_CONVEX_HULL && cp.w >= 0) {
                plane = cp.x; comp = cp.y; child = cp.w; pos = posB; q = qB;
            } else if (cB.shapeType == B3G_SHAPE_PLANE && cA.shapeType == B3G_SHAPE_CONVEX_HULL && cp.z >= 0) {
                plane = cp.y; comp = cp.x; child = cp.z; pos = posA; q = qA;
            }
            if (plane < 0) continue;
            float4 pts[64];
            int idx[4];
            v3 nWorld;
            const int hull = a.cols[a.children[child].shapeIndex].shapeIndex;
            const int nred = plane_hull_points(a, plane, a.hulls[hull], pos, q, pts, idx, nWorld);
            if (nred > 0) {
                write_header(c, a, plane, comp, -nWorld, nred);
                c.frictionCmp = fr07;
                c.batchIdx = j;
                c.childIndexB = child;
                for (int i = 0; i < nred; i++) {
                    const float4 qq = pts[idx[i]];
                    c.worldPosB[i] = b3gFloat4{qq.x, qq.y, qq.z, qq.w};
                }
                a.flags[slot] = 1;
            }
        }
    }
}

// Two hulls of a child pair, one warp per child pair (slot = pair count + child pair index):
// processCompoundPairsKernel + clipCompoundsHullHullKernel (b3ConvexHullContact.cpp:1777-2022).
// The reference runs findSeparatingAxis(A, B), findSeparatingAxis(B, A) and
// findSeparatingAxisEdgeEdge(A, B) in turn and keeps the axis the last one leaves.  The second
// pass tests the first pass's axes, each exactly negated (negation is exact and x - y = -(y - x)),
// with the same overlaps, so it separates exactly when the first does; the edge pass recomputes
// the first pass's edge overlaps.  So one pass over the faces of A, the faces of B and the edge
// axes decides the separation and keeps the first minimum of the edge axes, the contact normal;
// only when no edge axis is usable (every cross product almost zero) does the second pass's face
// minimum stand, computed then as the reference computes it.  Clipped at the child poses with
// minDist -1e30 and maxDist 0, reduced against -sep, friction 0.7.
static constexpr int CH_WARPS = 4;

// (80 registers, 6 CTAs an SM: measured 10% faster than 128 registers at 4 despite a few spills)
__global__ void __launch_bounds__(CH_WARPS * 32, 6) k_compound_hull_hull(NPArgs a, const int* __restrict__ d_np,
                                                                     const int* __restrict__ d_J,
                                                                     const int4* __restrict__ child_pairs) {
    __shared__ float4 s_poly[CH_WARPS][2][CLIP_CAP];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int P = *d_np, J = *d_J;
    const unsigned short fr07 = (unsigned short)(0.7f * 0xffff);
    for (int j = blockIdx.x * CH_WARPS + wib; j < J; j += gridDim.x * CH_WARPS) {
        const int4 cp = child_pairs[j];
        const b3gBody& BA = a.bodies[cp.x];
        const b3gBody& BB = a.bodies[cp.y];
        v3 posA = f4v3(BA.pos), posB = f4v3(BB.pos);
        quat qA = f4q(BA.quat), qB = f4q(BB.quat);
        int colA = BA.collidableIdx, colB = BB.collidableIdx;
        if (cp.z >= 0) {
            const b3gChildShape ch = a.children[cp.z];
            colA = ch.shapeIndex;
            child_pose(BA, ch, posA, qA);
        }
        if (cp.w >= 0) {
            const b3gChildShape ch = a.children[cp.w];
            colB = ch.shapeIndex;
            child_pose(BB, ch, posB, qB);
        }
        const b3gCollidable cA = a.cols[colA], cB = a.cols[colB];
        if (cA.shapeType != B3G_SHAPE_CONVEX_HULL || cB.shapeType != B3G_SHAPE_CONVEX_HULL) continue;
        const b3gHull hA = a.hulls[cA.shapeIndex], hB = a.hulls[cB.shapeIndex];
        const v3 deltaC2 =
            (mmul(qmat(qA), f4v3(hA.localCenter)) + posA) - (mmul(qmat(qB), f4v3(hB.localCenter)) + posB);
        const int nfaces = hA.numFaces + hB.numFaces;
        const int naxes = nfaces + hA.numUniqueEdges * hB.numUniqueEdges;
        const uint32_t dupA = __ldg(&a.face_dup[cA.shapeIndex]);
        const uint32_t dupB = __ldg(&a.face_dup[cB.shapeIndex]);
        const b3gFloat4* vA = &a.verts[hA.vertexOffset];
        const b3gFloat4* vB = &a.verts[hB.vertexOffset];
        AxisBest best{FLT_MAX, 0x7fffffff};  // edge axes only
        bool separated = false;
        for (int k0 = 0; k0 < naxes; k0 += 32) {
            const int k = k0 + lane;
            v3 axis;
            if (k < naxes && !(k < nfaces && dup_face_axis(k, hA.numFaces, dupA, dupB)) &&
                sat_axis(k, hA, hB, a.faces, a.edges, qA, qB, deltaC2, axis)) {
                float min0, max0, min1, max1;
                project(vA, hA.numVertices, posA, qA, axis, min0, max0);
                project(vB, hB.numVertices, posB, qB, axis, min1, max1);
                if (max0 < min1 || max1 < min0) {
                    separated = true;
                } else if (k >= nfaces) {
                    const float d0 = max0 - min1, d1 = max1 - min0;
                    const float dist = d0 < d1 ? d0 : d1;
                    if (dist < best.d || (dist == best.d && k < best.idx)) {
                        best.d = dist;
                        best.idx = k;
                    }
                }
            }
            if (__any_sync(0xffffffffu, separated)) break;
        }
        if (__any_sync(0xffffffffu, separated)) continue;
        best = warp_argmin(best);
        v3 sep;
        if (best.idx != 0x7fffffff) {
            sat_axis(best.idx, hA, hB, a.faces, a.edges, qA, qB, deltaC2, sep);
        } else if (!find_sep_full(a, hB, hA, posB, qB, posA, qA, sep)) {
            continue;
        }
        if (dot3(-deltaC2, sep) > 0.0f) sep = -sep;  // findSeparatingAxisEdgeEdge's last step

        // clipHullAgainstHull (b3ConvexHullContact.cpp:939-1044): incident face of B (first max of
        // dot(world normal, sep)), reference face of A (first min)
        AxisBest fb{-FLT_MAX, 0x7fffffff};
        for (int f = lane; f < hB.numFaces; f += 32) {
            const float d = dot3(qrotq(qB, ld3(&a.faces[hB.faceOffset + f].plane)), sep);
            if (d > fb.d || (d == fb.d && fb.idx != 0x7fffffff && f < fb.idx)) { fb.d = d; fb.idx = f; }
        }
        fb = warp_argmax(fb);
        AxisBest fa{FLT_MAX, 0x7fffffff};
        for (int f = lane; f < hA.numFaces; f += 32) {
            const float d = dot3(qrotq(qA, ld3(&a.faces[hA.faceOffset + f].plane)), sep);
            if (d < fa.d || (d == fa.d && fa.idx != 0x7fffffff && f < fa.idx)) { fa.d = d; fa.idx = f; }
        }
        fa = warp_argmin(fa);
        if (fb.idx == 0x7fffffff || fa.idx == 0x7fffffff) continue;

        if (lane == 0) {
            float4* pin = s_poly[wib][0];
            float4* pout = s_poly[wib][1];
            const m33 RA = qmat(qA), RB = qmat(qB);
            const b3gFace polyB = a.faces[hB.faceOffset + fb.idx];
            int nin = 0;
            for (int e = 0; e < polyB.numIndices && e < CLIP_CAP; e++) {
                const v3 w = mmul(RB, ld3(&vB[a.indices[polyB.indexOffset + e]])) + posB;
                pin[nin++] = make_float4(w.x, w.y, w.z, 0.f);
            }
            const b3gFace polyA = a.faces[hA.faceOffset + fa.idx];
            const v3 planeNormalA = mk3(polyA.plane.x, polyA.plane.y, polyA.plane.z);
            const int nva = polyA.numIndices;
            for (int e0 = 0; e0 < nva; e0++) {
                const v3 va = ld3(&vA[a.indices[polyA.indexOffset + e0]]);
                const v3 vb = ld3(&vA[a.indices[polyA.indexOffset + ((e0 + 1) % nva)]]);
                const v3 worldEdge0 = qrotq(qA, va - vb);
                const v3 worldPlaneAnormal1 = qrotq(qA, planeNormalA);
                const v3 planeNormalWS1 = -cross3(worldEdge0, worldPlaneAnormal1);
                const v3 worldA1 = mmul(RA, va) + posA;
                const float planeEqWS1 = -dot3(worldA1, planeNormalWS1);
                const int nout = clip_face(pin, nin, planeNormalWS1, planeEqWS1, pout, a.status);
                float4* t = pout;
                pout = pin;
                pin = t;
                nin = nout;
            }
            const v3 planeNormalWS = qrotq(qA, planeNormalA);
            const float planeEqWS = polyA.plane.w - dot3(planeNormalWS, posA);
            int np = 0;
            for (int i = 0; i < nin; i++) {
                float depth = dot3(planeNormalWS, mk3(pin[i].x, pin[i].y, pin[i].z)) + planeEqWS;
                if (depth <= -1e30f) depth = -1e30f;
                if (np < CLIP_CAP && depth <= 0.0f) pout[np++] = make_float4(pin[i].x, pin[i].y, pin[i].z, depth);
            }
            if (np > 0) {
                int idx[4];
                const int nred = reduce_contacts(pout, np, -sep, idx);
                const int slot = P + j;
                b3gContact4& c = a.slots[slot];
                write_header(c, a, cp.x, cp.y, sep, nred);
                c.frictionCmp = fr07;
                c.batchIdx = j;
                c.childIndexA = cp.z;
                c.childIndexB = cp.w;
                for (int i = 0; i < nred; i++) {
                    const float4 q = pout[idx[i]];
                    c.worldPosB[i] = b3gFloat4{q.x, q.y, q.z, q.w};
                }
                a.flags[slot] = 1;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ concave meshes
// A pair whose first body is a concave mesh and whose second is a hull or a compound expands into
// triangle-convex pairs (b3BvhTraversal, shared/b3BvhTraversal.h:11-111): the triangles whose
// quantized leaf box overlaps the other body's world AABB quantized into the mesh's BVH bounds
// (as the reference does, in the mesh's own frame: meshes stay at the identity pose), with every
// child of a compound; in (pair, triangle, child) order, the BVH's depth-first order being the
// triangle order.  Static-static pairs are skipped.

// b3QuantizeWithClamp (shared/b3QuantizedBvhNodeData.h:42-60)
__device__ __forceinline__ void quantize_clamp(unsigned short out[3], const float p[3], bool isMax,
                                               const b3gBvhInfo& bi) {
    const float mn[3] = {bi.aabbMin.x, bi.aabbMin.y, bi.aabbMin.z};
    const float mx[3] = {bi.aabbMax.x, bi.aabbMax.y, bi.aabbMax.z};
    const float q[3] = {bi.quantization.x, bi.quantization.y, bi.quantization.z};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float c = p[k];
        if (c < mn[k]) c = mn[k];
        if (mx[k] < c) c = mx[k];
        const float v = (c - mn[k]) * q[k];
        out[k] = isMax ? (unsigned short)(((unsigned short)(v + 1.f)) | 1) : (unsigned short)(((unsigned short)v) & 0xfffe);
    }
}

// the triangle-convex pairs of pair p: counted (out == nullptr), or written at out[0..cap)
__device__ int concave_tri_pairs(const NPArgs& a, int p, int4* out, int cap) {
    const b3gPair pr = a.pairs[p];
    const int A = pr.x, B = pr.y;
    const b3gBody& BA = a.bodies[A];
    const b3gBody& BB = a.bodies[B];
    if (BA.invMass == 0.f && BB.invMass == 0.f) return 0;
    const b3gCollidable cA = a.cols[BA.collidableIdx];
    if (cA.shapeType != B3G_SHAPE_CONCAVE_TRIMESH) return 0;
    const b3gCollidable cB = a.cols[BB.collidableIdx];
    if (cB.shapeType != B3G_SHAPE_CONVEX_HULL && cB.shapeType != B3G_SHAPE_SPHERE && cB.shapeType != B3G_SHAPE_COMPOUND)
        return 0;
    const bool comp = cB.shapeType == B3G_SHAPE_COMPOUND;
    const int nch = comp ? cB.numChildShapes : 1;
    const b3gBvhInfo bi = a.bvh_infos[cA.numChildShapes];
    const b3gAabb box = a.aabbs[B];
    unsigned short qmn[3], qmx[3];
    quantize_clamp(qmn, box.minv, false, bi);
    quantize_clamp(qmx, box.maxv, true, bi);
    const int4* nodes = reinterpret_cast<const int4*>(a.bvh_nodes + bi.nodeOffset);
    int n = 0, cur = 0;
    while (cur < bi.numNodes) {
        const int4 raw = __ldg(&nodes[cur]);
        const unsigned short nmn0 = (unsigned short)(raw.x & 0xffff), nmn1 = (unsigned short)((unsigned)raw.x >> 16);
        const unsigned short nmn2 = (unsigned short)(raw.y & 0xffff), nmx0 = (unsigned short)((unsigned)raw.y >> 16);
        const unsigned short nmx1 = (unsigned short)(raw.z & 0xffff), nmx2 = (unsigned short)((unsigned)raw.z >> 16);
        const int e = raw.w;
        // b3TestQuantizedAabbAgainstQuantizedAabbSlow (shared/b3QuantizedBvhNodeData.h:62-85)
        const bool ov = !(qmn[0] > nmx0 || qmx[0] < nmn0 || qmn[1] > nmx1 || qmx[1] < nmn1 || qmn[2] > nmx2 ||
                          qmx[2] < nmn2);
        const bool leaf = e >= 0;
        if (ov && leaf) {
            for (int c = 0; c < nch; c++) {
                if (out && n < cap) out[n] = make_int4(A, B, e, comp ? cB.shapeIndex + c : 0);
                n++;
            }
        }
        cur += (ov || leaf) ? 1 : -e;
    }
    return n;
}

__global__ void k_concave_count(NPArgs a, const int* __restrict__ d_np, int* __restrict__ counts) {
    const int np = *d_np;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        counts[p] = concave_tri_pairs(a, p, nullptr, 0);
}

__global__ void k_concave_expand(NPArgs a, const int* __restrict__ d_np, const int* __restrict__ offsets,
                                 int4* __restrict__ tri_pairs, int cap) {
    const int np = *d_np;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int o = offsets[p];
        if (o < cap) concave_tri_pairs(a, p, tri_pairs + o, cap - o);
    }
}

// clipFaceGlobal (shared/b3ClipFaces.h:20-61): as clip_face, but a polygon of one vertex is
// clipped too (the reference has no lower bound on the input)
__device__ int clip_face_global(const float4* in, int nin, v3 n, float eq, float4* out, unsigned int* status) {
    if (nin < 1) return 0;
    int nout = 0;
    float4 first = in[nin - 1];
    float ds = dot3(n, mk3(first.x, first.y, first.z)) + eq;
    for (int ve = 0; ve < nin; ve++) {
        const float4 end = in[ve];
        const float de = dot3(n, mk3(end.x, end.y, end.z)) + eq;
        if (ds < 0.f) {
            if (de < 0.f) {
                if (nout < CLIP_CAP) out[nout++] = end; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
            } else {
                const float t = ds * 1.f / (ds - de);
                const float4 l = make_float4(first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                                             first.z + (end.z - first.z) * t, 0.f);
                if (nout < CLIP_CAP) out[nout++] = l; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
            }
        } else if (de < 0.f) {
            const float t = ds * 1.f / (ds - de);
            const float4 l = make_float4(first.x + (end.x - first.x) * t, first.y + (end.y - first.y) * t,
                                         first.z + (end.z - first.z) * t, 0.f);
            if (nout < CLIP_CAP) out[nout++] = l; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
            if (nout < CLIP_CAP) out[nout++] = end; else atomicOr(status, B3G_FLAG_CLIP_OVERFLOW);
        }
        first = end;
        ds = de;
    }
    return nout;
}

// A triangle as the reference's five-face prism (b3FindConcaveSeparatingAxisKernel,
// shared/b3FindConcaveSatAxis.h:506-797): its 3 vertices; faces 0 front (the mesh face's plane), 1
// back (negated), 2..4 the edge planes normalize(n x (v[prev] - v[i])); unique edges v1 - v0,
// v2 - v1, v0 - v2; local centre (v0 + v1 + v2) / 3.
struct TriPrism {
    v3 v[3];
    v3 n[5];
    v3 e[3];
    v3 center;
};

__device__ __forceinline__ void tri_prism(const NPArgs& a, const b3gHull& mesh, int t, TriPrism& P) {
    const b3gFace face = a.faces[mesh.faceOffset + t];
    v3 lc = mk3(0.f, 0.f, 0.f);
    for (int i = 0; i < 3; i++) {
        P.v[i] = ld3(&a.verts[mesh.vertexOffset + a.indices[face.indexOffset + i]]);
        lc = lc + P.v[i];
    }
    const v3 normal = mk3(face.plane.x, face.plane.y, face.plane.z);
    P.n[0] = normal;
    P.n[1] = -normal;
    int prev = 2;
    for (int i = 0; i < 3; i++) {
        P.n[2 + i] = normalize3(cross3(normal, P.v[prev] - P.v[i]));
        prev = i;
    }
    P.e[0] = P.v[1] - P.v[0];
    P.e[1] = P.v[2] - P.v[1];
    P.e[2] = P.v[0] - P.v[2];
    P.center = lc * (1.f / 3.f);
}

// b3Project over the prism's 3 vertices
__device__ __forceinline__ void project_tri(const TriPrism& P, v3 pos, quat orn, v3 dir, float& mn, float& mx) {
    const v3 localDir = qrotq(qconj(orn), dir);
    const float offset = dot3(pos, dir);
    mn = FLT_MAX;
    mx = -FLT_MAX;
    for (int i = 0; i < 3; i++) {
        const float dp = dot3(P.v[i], localDir);
        if (dp < mn) mn = dp;
        if (dp > mx) mx = dp;
    }
    if (mn > mx) {
        const float t = mn; mn = mx; mx = t;
    }
    mn = mn + offset;
    mx = mx + offset;
}

// SAT axis k of a triangle-convex pair, in the reference's order: the prism's 5 faces, the hull's
// faces, then the edge pairs (prism edge major); false when the edge cross product is almost zero
__device__ __forceinline__ bool concave_axis(int k, const TriPrism& P, const b3gHull& hB, const NPArgs& a, quat qA,
                                             quat qB, v3 D, v3& axis) {
    if (k < 5) {
        axis = qrotq(qA, P.n[k]);
    } else if (k < 5 + hB.numFaces) {
        axis = qrotq(qB, ld3(&a.faces[hB.faceOffset + (k - 5)].plane));
    } else {
        const int e = k - 5 - hB.numFaces;
        const int e0 = e / hB.numUniqueEdges, e1 = e - e0 * hB.numUniqueEdges;
        const v3 w0 = qrotq(qA, P.e[e0]);
        const v3 w1 = qrotq(qB, ld3(&a.edges[hB.uniqueEdgesOffset + e1]));
        const v3 c = cross3(w0, w1);
        if (!((double)fabsf(c.x) > 1e-6 || (double)fabsf(c.y) > 1e-6 || (double)fabsf(c.z) > 1e-6)) return false;
        axis = normalize3(c);
    }
    if (dot3(D, axis) < 0.f) axis = -axis;
    return true;
}

// computeContactSphereTriangle (kernels/primitiveContacts.cl:1163-1302, run by
// findConcaveSphereContactsKernel :1319-1370): the sphere centre in the mesh's frame; the
// triangle's plane turned towards it; a contact on the face when the centre's projection is inside
// the triangle (pointInTriangle), else the nearest point of an edge within the radius (the last such
// edge, segmentSqrDistance); one point at most the radius deep, the sphere as body A, childIndexB
// the triangle
__device__ bool concave_sphere(const NPArgs& a, const b3gHull& mesh, int4 cp, int index, b3gContact4& c) {
    const b3gBody& BM = a.bodies[cp.x];
    const b3gBody& BS = a.bodies[cp.y];
    const float radius = a.cols[BS.collidableIdx].radius;
    const b3gFace face = a.faces[mesh.faceOffset + cp.z];
    v3 tv[3];
    for (int i = 0; i < 3; i++) tv[i] = ld3(&a.verts[mesh.vertexOffset + a.indices[face.indexOffset + i]]);
    const v3 pos = f4v3(BM.pos);
    const quat q = f4q(BM.quat), qi = qconj(q);
    const v3 centre = qrotq(qi, f4v3(BS.pos)) + qrotq(qi, -pos);
    v3 normal = normalize3(cross3(tv[1] - tv[0], tv[2] - tv[0]));
    float dist = dot3(centre - tv[0], normal);
    if (dist < 0.f) {
        dist = dist * -1.f;
        normal = normal * -1.f;
    }
    bool has = false;
    v3 cpt = mk3(0.f, 0.f, 0.f);
    if (dist < radius) {
        const v3 e1 = tv[1] - tv[0], e2 = tv[2] - tv[1], e3 = tv[0] - tv[2];
        const float r1 = dot3(cross3(e1, normal), centre - tv[0]);
        const float r2 = dot3(cross3(e2, normal), centre - tv[1]);
        const float r3 = dot3(cross3(e3, normal), centre - tv[2]);
        if ((r1 > 0.f && r2 > 0.f && r3 > 0.f) || (r1 <= 0.f && r2 <= 0.f && r3 <= 0.f)) {
            has = true;
            cpt = centre - normal * dist;
        } else {
            const float rr = radius * radius;
            for (int i = 0; i < 3; i++) {
                const v3 from = tv[i], to = tv[(i + 1) % 3];
                v3 diff = centre - from;
                const v3 v = to - from;
                float t = dot3(v, diff);
                if (t > 0.f) {
                    const float vv = dot3(v, v);
                    if (t < vv) {
                        t = t / vv;
                        diff = diff - t * v;
                    } else {
                        t = 1.f;
                        diff = diff - v;
                    }
                } else {
                    t = 0.f;
                }
                if (dot3(diff, diff) < rr) {
                    has = true;
                    cpt = from + t * v;
                }
            }
        }
    }
    if (!has) return false;
    const v3 toc = centre - cpt;
    const float md = sqrtf(dot3(toc, toc));
    if (!(md > FLT_EPSILON)) return false;
    const float depth = md - radius;
    const v3 n1 = qrotq(q, -normalize3(toc));
    const v3 pB = qrotq(q, cpt) + pos;
    if (!(depth <= 0.f) || !(dot3(n1, n1) > FLT_EPSILON)) return false;
    write_header(c, a, cp.y, cp.x, -n1, 1);
    c.frictionCmp = (unsigned short)(0.7f * 0xffff);
    c.batchIdx = index;
    c.childIndexB = cp.z;
    c.worldPosB[0] = b3gFloat4{pB.x, pB.y, pB.z, depth};
    return true;
}

// One warp per triangle-convex pair (slot = pairs + compound child pairs + its index):
// b3FindConcaveSeparatingAxisKernel, then b3FindClippingFaces (shared/b3FindConcaveSatAxis.h:421-504),
// clipFacesAndFindContactsKernel (shared/b3ClipFaces.h:67-177) and b3NewContactReductionKernel
// (shared/b3NewContactReduction.h:88-177).  The reference's three passes (the prism's faces, the
// hull's faces, the edge pairs) share one running minimum and orient every axis towards the
// triangle, so the normal is the first minimum over the whole sequence; every pass returns at a
// separating axis.  Clipped with minDist -1e30 and maxDist 0.02, reduced against -sep, friction
// 0.7, no child indices (the reference stores -1 for both).
static constexpr int CC_WARPS = 4;

// (80 registers, 6 CTAs an SM, as k_compound_hull_hull)
__global__ void __launch_bounds__(CC_WARPS * 32, 6) k_concave_contacts(NPArgs a, const int* __restrict__ d_np,
                                                                   const int* __restrict__ d_J,
                                                                   const int* __restrict__ d_K,
                                                                   const int4* __restrict__ tri_pairs) {
    __shared__ float4 s_poly[CC_WARPS][2][CLIP_CAP];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int base = *d_np + (d_J ? *d_J : 0), K = *d_K;
    const unsigned short fr07 = (unsigned short)(0.7f * 0xffff);
    for (int k = blockIdx.x * CC_WARPS + wib; k < K; k += gridDim.x * CC_WARPS) {
        const int slot = base + k;
        if (lane == 0) a.flags[slot] = 0;
        const int4 cp = tri_pairs[k];
        const b3gBody& BA = a.bodies[cp.x];
        const b3gBody& BB = a.bodies[cp.y];
        const b3gHull mesh = a.hulls[a.cols[BA.collidableIdx].shapeIndex];
        if (a.cols[BB.collidableIdx].shapeType == B3G_SHAPE_SPHERE) {
            if (lane == 0 && concave_sphere(a, mesh, cp, k, a.slots[slot])) a.flags[slot] = 1;
            continue;
        }
        TriPrism P;
        tri_prism(a, mesh, cp.z, P);
        // the triangle's local AABB against the other body's world AABB
        {
            const b3gAabb box = a.aabbs[cp.y];
            float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
            for (int i = 0; i < 3; i++) {
                const float c[3] = {P.v[i].x, P.v[i].y, P.v[i].z};
                for (int q = 0; q < 3; q++) {
                    if (c[q] < lo[q]) lo[q] = c[q];
                    if (hi[q] < c[q]) hi[q] = c[q];
                }
            }
            bool ov = true;
            for (int q = 0; q < 3; q++)
                if (lo[q] > box.maxv[q] || hi[q] < box.minv[q]) ov = false;
            if (!ov) continue;
        }
        const v3 posA = f4v3(BA.pos);
        const quat qA = f4q(BA.quat);
        v3 posB = f4v3(BB.pos);
        quat qB = f4q(BB.quat);
        // b3TransformPoint of the host code is b3Transform's (the quaternion's rotation matrix): for
        // the child pose, the centres and the clipping faces' vertices
        int colB = BB.collidableIdx;
        if (a.cols[colB].shapeType == B3G_SHAPE_COMPOUND) {
            const b3gChildShape ch = a.children[cp.w];
            colB = ch.shapeIndex;
            posB = mmul(qmat(qB), f4v3(ch.childPosition)) + posB;
            qB = qmul(qB, f4q(ch.childOrientation));
        }
        const b3gHull hB = a.hulls[a.cols[colB].shapeIndex];
        const m33 RA = qmat(qA), RB = qmat(qB);
        const v3 c0 = mmul(RA, P.center) + posA;
        const v3 c1 = mmul(RB, f4v3(hB.localCenter)) + posB;
        const v3 D = c0 - c1;
        const b3gFloat4* vB = &a.verts[hB.vertexOffset];
        const int naxes = 5 + hB.numFaces + 3 * hB.numUniqueEdges;
        AxisBest best{FLT_MAX, 0x7fffffff};
        bool separated = false;
        for (int k0 = 0; k0 < naxes; k0 += 32) {
            const int ax = k0 + lane;
            v3 axis;
            if (ax < naxes && concave_axis(ax, P, hB, a, qA, qB, D, axis)) {
                float min0, max0, min1, max1;
                project_tri(P, posA, qA, axis, min0, max0);
                project(vB, hB.numVertices, posB, qB, axis, min1, max1);
                if (max0 < min1 || max1 < min0) {
                    separated = true;
                } else {
                    const float d0 = max0 - min1, d1 = max1 - min0;
                    const float d = d0 < d1 ? d0 : d1;
                    if (d < best.d || (d == best.d && ax < best.idx)) {
                        best.d = d;
                        best.idx = ax;
                    }
                }
            }
            if (__any_sync(0xffffffffu, separated)) break;
        }
        if (__any_sync(0xffffffffu, separated)) continue;
        best = warp_argmin(best);
        if (best.idx == 0x7fffffff) continue;
        v3 sep;
        concave_axis(best.idx, P, hB, a, qA, qB, D, sep);

        // b3FindClippingFaces: the hull's face most along sep (first max), the prism's face most
        // against it (first min)
        AxisBest fb{-FLT_MAX, 0x7fffffff};
        for (int f = lane; f < hB.numFaces; f += 32) {
            const float d = dot3(qrotq(qB, ld3(&a.faces[hB.faceOffset + f].plane)), sep);
            if (d > fb.d || (d == fb.d && fb.idx != 0x7fffffff && f < fb.idx)) { fb.d = d; fb.idx = f; }
        }
        fb = warp_argmax(fb);
        if (fb.idx == 0x7fffffff) continue;

        if (lane == 0) {
            int fa = -1;
            float dmn = FLT_MAX;
            v3 nA = mk3(0.f, 0.f, 0.f);
            for (int f = 0; f < 5; f++) {
                const v3 wn = qrotq(qA, P.n[f]);
                const float d = dot3(wn, sep);
                if (d < dmn) { dmn = d; fa = f; nA = wn; }
            }
            if (fa >= 0) {
                // the prism face's vertices: front 0 1 2, back 2 1 0, edge plane 2 + i: i, prev(i)
                int ia[3], na;
                if (fa == 0) { ia[0] = 0; ia[1] = 1; ia[2] = 2; na = 3; }
                else if (fa == 1) { ia[0] = 2; ia[1] = 1; ia[2] = 0; na = 3; }
                else { const int i = fa - 2; ia[0] = i; ia[1] = i == 0 ? 2 : i - 1; na = 2; }
                v3 wA[3];
                for (int i = 0; i < na; i++) wA[i] = mmul(RA, P.v[ia[i]]) + posA;
                float4* pin = s_poly[wib][0];
                float4* pout = s_poly[wib][1];
                const b3gFace polyB = a.faces[hB.faceOffset + fb.idx];
                int nin = 0;
                for (int e = 0; e < polyB.numIndices && e < CLIP_CAP; e++) {
                    const v3 w = mmul(RB, ld3(&vB[a.indices[polyB.indexOffset + e]])) + posB;
                    pin[nin++] = make_float4(w.x, w.y, w.z, 0.f);
                }
                for (int e0 = 0; e0 < na; e0++) {
                    const v3 aw = wA[e0], bw = wA[(e0 + 1) % na];
                    const v3 pn = -cross3(aw - bw, nA);
                    const float eq = -dot3(aw, pn);
                    const int nout = clip_face_global(pin, nin, pn, eq, pout, a.status);
                    float4* t = pout;
                    pout = pin;
                    pin = t;
                    nin = nout;
                }
                const float eqA = -dot3(nA, wA[0]);
                int np = 0;
                for (int i = 0; i < nin; i++) {
                    float depth = dot3(nA, mk3(pin[i].x, pin[i].y, pin[i].z)) + eqA;
                    if (depth <= -1e30f) depth = -1e30f;
                    if (depth <= 0.02f) pout[np++] = make_float4(pin[i].x, pin[i].y, pin[i].z, depth);
                }
                if (np > 0) {
                    int idx[4];
                    const int nred = reduce_contacts(pout, np, -sep, idx);
                    b3gContact4& c = a.slots[slot];
                    write_header(c, a, cp.x, cp.y, sep, nred);
                    c.frictionCmp = fr07;
                    c.batchIdx = k;
                    for (int i = 0; i < nred; i++) {
                        const float4 q = pout[idx[i]];
                        c.worldPosB[i] = b3gFloat4{q.x, q.y, q.z, q.w};
                    }
                    a.flags[slot] = 1;
                }
            }
        }
        __syncwarp();
    }
}

static NPArgs make_args(DeviceState& d, unsigned short friction_cmp) {
    NPArgs a;
    a.bodies = d.bodies;
    a.cols = d.collidables;
    a.hulls = d.hulls;
    a.face_dup = d.hull_face_dup;
    a.faces = d.faces;
    a.indices = d.indices;
    a.verts = d.vertices;
    a.edges = d.edges;
    a.pairs = d.pairs;
    a.type_list = d.type_lists;
    a.type_count = d.counters->type_count;
    a.slots = d.contact_slots;
    a.flags = d.contact_flag;
    a.status = &d.counters->status;
    a.friction_cmp = friction_cmp;
    a.children = d.children;
    a.local_aabbs = d.local_aabbs;
    a.aabbs = d.aabbs;
    a.bvh_infos = d.bvh_infos;
    a.bvh_nodes = d.bvh_nodes;
    return a;
}

unsigned short friction_to_cmp(float f) {
    if (f < 0.f) f = 0.f;
    if (f > 1.f) f = 1.f;
    return (unsigned short)(f * 65535.0f);
}

int launch_contacts(DeviceState& d, float friction, cudaStream_t s) {
    NPArgs a = make_args(d, friction_to_cmp(friction));
    int grid = d.num_sms * 4;
    k_primitive_pairs<<<grid, NP_THREADS, 0, s>>>(a, d.max_pairs);
    k_hull_hull_small<<<d.num_sms * d.tune.narrow_blocks_per_sm, NP_THREADS, 0, s>>>(a, d.max_pairs);
    k_hull_hull<<<d.num_sms * 16, HH_WARPS * 32, 0, s>>>(a, d.max_pairs);
    long long ll = 0;
    int* d_np = &d.counters->pad[0];
    int* d_slots = d_np;
    int launches = 0;
    int* d_J = nullptr;
    if (d.num_children > 0) {
        // compound pairs: child-pair counts, their scan (total in pad[4]) clamped to capacity, the
        // child pairs, their manifolds (the flags cleared and plane-child pairs, then hull-hull
        // child pairs a warp each)
        d_J = &d.counters->pad[4];
        k_compound_count<<<grid, NP_THREADS, 0, s>>>(a, d_np, d.child_count);
        exclusive_scan_i32(d.prim, d.child_count, d.child_offset, d_np, d_J, d.scan_scratch, s, &ll);
        k_clamp_total<<<1, 1, 0, s>>>(d_J, d.max_child_pairs, &d.counters->status);
        k_compound_expand<<<grid, NP_THREADS, 0, s>>>(a, d_np, d.child_offset, d.child_pairs, d.max_child_pairs);
        k_compound_contacts<<<grid, NP_THREADS, 0, s>>>(a, d_np, d_J, d.child_pairs);
        k_compound_hull_hull<<<d.num_sms * 16, CH_WARPS * 32, 0, s>>>(a, d_np, d_J, d.child_pairs);
        launches += 5;
    }
    int* d_K = nullptr;
    if (d.num_meshes > 0) {
        // concave-mesh pairs: triangle-convex pair counts, their scan (total in pad[6]) clamped to
        // capacity, the triangle-convex pairs, their manifolds a warp each
        d_K = &d.counters->pad[6];
        k_concave_count<<<grid, NP_THREADS, 0, s>>>(a, d_np, d.concave_count);
        exclusive_scan_i32(d.prim, d.concave_count, d.concave_offset, d_np, d_K, d.scan_scratch, s, &ll);
        k_clamp_total<<<1, 1, 0, s>>>(d_K, d.max_concave_pairs, &d.counters->status);
        k_concave_expand<<<grid, NP_THREADS, 0, s>>>(a, d_np, d.concave_offset, d.concave_pairs, d.max_concave_pairs);
        k_concave_contacts<<<d.num_sms * 16, CC_WARPS * 32, 0, s>>>(a, d_np, d_J, d_K, d.concave_pairs);
        launches += 4;
    }
    if (d_J || d_K) {
        d_slots = &d.counters->pad[7];
        k_slot_total<<<1, 1, 0, s>>>(d_np, d_J, d_K, d_slots);
        launches++;
    }
    exclusive_scan_i32(d.prim, d.contact_flag, d.contact_index, d_slots, &d.counters->num_contacts, d.scan_scratch,
                       s, &ll);
    k_manifold_list<<<grid, NP_THREADS, 0, s>>>(d.contact_flag, d.contact_index, d_slots, d_np, d.contact_slots,
                                                d.pairs, d.manifold_pair, &d.counters->num_points);
    return 1 + 2 + 1 + launches + (int)ll;
}

int launch_compact_contacts(DeviceState& d, cudaStream_t s) {
    k_compact_contacts<<<d.num_sms * 4, NP_THREADS, 0, s>>>(&d.counters->num_contacts, d.manifold_pair,
                                                            d.contact_slots, d.contacts_compact);
    return 1;
}

}  // namespace b3g
