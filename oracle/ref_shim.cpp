// ref_shim.cpp -- C entry points into the REFERENCE's own CPU code, compiled in place from the
// reference sources by oracle/build_ref.sh into oracle/_ref/libb3ref.so.  TEST INFRASTRUCTURE
// ONLY: it generates the golden vectors under tests/golden/ and pins the plain-C oracle
// (oracle/b3oracle.c) to the reference; nothing in the product loads it.
//
// Functions wrapped (paths relative to the reference project's src/):
//   b3ConvexUtility::initializePolyhedralFeatures   Bullet3Collision/NarrowPhaseCollision/b3ConvexUtility.cpp:26
//   b3TransformAabb2                                Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h:24
//   b3DynamicBvhBroadphase + b3TestAabbAgainstAabb  Bullet3Collision/BroadPhaseCollision/b3DynamicBvhBroadphase.cpp
//   b3ContactConvexConvexSAT                        Bullet3Collision/NarrowPhaseCollision/shared/b3ContactConvexConvexSAT.h:403
//   computeContactPlaneConvex / SphereConvex        Bullet3OpenCL/NarrowphaseCollision/b3ConvexHullContact.cpp:1272, :2323
//   b3PgsJacobiSolver::solveGroup                   Bullet3Dynamics/ConstraintSolver/b3PgsJacobiSolver.cpp:170
//   integrateSingleTransform                        Bullet3Dynamics/shared/b3IntegrateTransforms.h:5
//   registerPhysicsInstance / registerRigidBody     Bullet3OpenCL/RigidBody/b3GpuRigidBodyPipeline.cpp:603, b3GpuNarrowPhase.cpp:816
//   b3GpuRaycast::castRaysHost                      Bullet3OpenCL/Raycast/b3GpuRaycast.cpp:175-247
//   b3Point2PointConstraint / b3FixedConstraint     Bullet3Dynamics/ConstraintSolver/b3Point2PointConstraint.cpp, b3FixedConstraint.cpp
//     through b3PgsJacobiSolver::solveGroup         (joints only, no contacts)
//   processCompoundPairsKernel + clipCompoundsHullHullKernel, computeContactPlaneCompound
//                                                   Bullet3OpenCL/NarrowphaseCollision/b3ConvexHullContact.cpp:1777-2022, :2182
//   registerConcaveMesh's BVH (b3OptimizedBvh)      Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.cpp:521-613
//   b3BvhTraversal, b3FindConcaveSeparatingAxisKernel, clipFacesAndFindContactsKernel,
//   b3NewContactReductionKernel                     Bullet3Collision/NarrowPhaseCollision/shared/ (host twins)
#include <algorithm>
#include <cstring>
#include <vector>

#include "Bullet3Common/b3AlignedObjectArray.h"
#include "Bullet3Common/b3Vector3.h"
#include "Bullet3Common/b3Quaternion.h"
#include "Bullet3Common/b3Matrix3x3.h"
#include "Bullet3Common/b3Transform.h"
#include "Bullet3Geometry/b3AabbUtil.h"
#include "Bullet3Common/shared/b3Int4.h"
#include "Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h"
#include "Bullet3Collision/BroadPhaseCollision/b3DynamicBvhBroadphase.h"
#include "Bullet3Collision/NarrowPhaseCollision/b3ConvexUtility.h"
#include "Bullet3Collision/NarrowPhaseCollision/b3Contact4.h"
#include "Bullet3Collision/NarrowPhaseCollision/shared/b3RigidBodyData.h"
#include "Bullet3Collision/NarrowPhaseCollision/shared/b3Collidable.h"
#include "Bullet3Collision/NarrowPhaseCollision/shared/b3ConvexPolyhedronData.h"
#include "Bullet3Collision/NarrowPhaseCollision/shared/b3ContactConvexConvexSAT.h"
#include "Bullet3Dynamics/ConstraintSolver/b3PgsJacobiSolver.h"
#include "Bullet3OpenCL/NarrowphaseCollision/b3BvhInfo.h"
#include "Bullet3OpenCL/NarrowphaseCollision/b3OptimizedBvh.h"
#include "Bullet3OpenCL/NarrowphaseCollision/b3TriangleIndexVertexArray.h"
#include "Bullet3Dynamics/ConstraintSolver/b3ContactSolverInfo.h"
#include "Bullet3Dynamics/ConstraintSolver/b3Point2PointConstraint.h"
#include "Bullet3Dynamics/ConstraintSolver/b3FixedConstraint.h"
#include "Bullet3Dynamics/shared/b3IntegrateTransforms.h"
#include "Bullet3OpenCL/Raycast/b3GpuRaycast.h"
#include "Bullet3OpenCL/RigidBody/b3GpuNarrowPhaseInternalData.h"

void computeContactPlaneConvex(int pairIndex, int bodyIndexA, int bodyIndexB, int collidableIndexA,
                               int collidableIndexB, const b3RigidBodyData* rigidBodies,
                               const b3Collidable* collidables, const b3ConvexPolyhedronData* convexShapes,
                               const b3Vector3* convexVertices, const int* convexIndices, const b3GpuFace* faces,
                               b3Contact4* globalContactsOut, int& nGlobalContactsOut, int maxContactCapacity);
void computeContactSphereConvex(int pairIndex, int bodyIndexA, int bodyIndexB, int collidableIndexA,
                                int collidableIndexB, const b3RigidBodyData* rigidBodies,
                                const b3Collidable* collidables, const b3ConvexPolyhedronData* convexShapes,
                                const b3Vector3* convexVertices, const int* convexIndices, const b3GpuFace* faces,
                                b3Contact4* globalContactsOut, int& nGlobalContactsOut, int maxContactCapacity);

// host twins of the compound kernels (b3ConvexHullContact.cpp, external linkage there)
void processCompoundPairsKernel(const b3Int4* gpuCompoundPairs, const b3RigidBodyData* rigidBodies,
                                const b3Collidable* collidables, const b3ConvexPolyhedronData* convexShapes,
                                const b3AlignedObjectArray<b3Vector3>& vertices,
                                const b3AlignedObjectArray<b3Vector3>& uniqueEdges,
                                const b3AlignedObjectArray<b3GpuFace>& faces, const b3AlignedObjectArray<int>& indices,
                                b3Aabb* aabbs, const b3GpuChildShape* gpuChildShapes,
                                b3AlignedObjectArray<b3Vector3>& gpuCompoundSepNormalsOut,
                                b3AlignedObjectArray<int>& gpuHasCompoundSepNormalsOut, int numCompoundPairs, int i);
void clipCompoundsHullHullKernel(const b3Int4* gpuCompoundPairs, const b3RigidBodyData* rigidBodies,
                                 const b3Collidable* collidables, const b3ConvexPolyhedronData* convexShapes,
                                 const b3AlignedObjectArray<b3Vector3>& vertices,
                                 const b3AlignedObjectArray<b3Vector3>& uniqueEdges,
                                 const b3AlignedObjectArray<b3GpuFace>& faces, const b3AlignedObjectArray<int>& indices,
                                 const b3GpuChildShape* gpuChildShapes,
                                 const b3AlignedObjectArray<b3Vector3>& gpuCompoundSepNormalsOut,
                                 const b3AlignedObjectArray<int>& gpuHasCompoundSepNormalsOut,
                                 b3Contact4Data* globalContactsOut, int* nGlobalContactsOut, int numCompoundPairs,
                                 int maxContactCapacity, int i);
void computeContactPlaneCompound(int pairIndex, int bodyIndexA, int bodyIndexB, int collidableIndexA,
                                 int collidableIndexB, const b3RigidBodyData* rigidBodies,
                                 const b3Collidable* collidables, const b3ConvexPolyhedronData* convexShapes,
                                 const b3GpuChildShape* cpuChildShapes, const b3Vector3* convexVertices,
                                 const int* convexIndices, const b3GpuFace* faces, b3Contact4* globalContactsOut,
                                 int& nGlobalContactsOut, int maxContactCapacity);

// host twins of the concave kernels (shared headers, compiled into b3ConvexHullContact.cpp)
void b3BvhTraversal(const b3Int4* pairs, const b3RigidBodyData* rigidBodies, const b3Collidable* collidables,
                    b3Aabb* aabbs, b3Int4* concavePairsOut, volatile int* numConcavePairsOut,
                    const b3BvhSubtreeInfo* subtreeHeadersRoot, const b3QuantizedBvhNode* quantizedNodesRoot,
                    const b3BvhInfo* bvhInfos, int numPairs, int maxNumConcavePairsCapacity, int id);
void b3FindConcaveSeparatingAxisKernel(b3Int4* concavePairs, const b3RigidBodyData* rigidBodies,
                                       const b3Collidable* collidables, const b3ConvexPolyhedronData* convexShapes,
                                       const b3Vector3* vertices, const b3Vector3* uniqueEdges, const b3GpuFace* faces,
                                       const int* indices, const b3GpuChildShape* gpuChildShapes, b3Aabb* aabbs,
                                       b3Vector3* concaveSeparatingNormalsOut, b3Int4* clippingFacesOut,
                                       b3Vector3* worldVertsA1Out, b3Vector3* worldNormalsA1Out,
                                       b3Vector3* worldVertsB1Out, int* hasSeparatingNormals, int vertexFaceCapacity,
                                       int numConcavePairs, int pairIdx);
void clipFacesAndFindContactsKernel(const b3Vector3* separatingNormals, const int* hasSeparatingAxis,
                                    b3Int4* clippingFacesOut, b3Vector3* worldVertsA1, b3Vector3* worldNormalsA1,
                                    b3Vector3* worldVertsB1, b3Vector3* worldVertsB2, int vertexFaceCapacity,
                                    int pairIndex);
void b3NewContactReductionKernel(b3Int4* pairs, const b3RigidBodyData* rigidBodies,
                                 const b3Vector3* separatingNormals, const int* hasSeparatingAxis,
                                 b3Contact4Data* globalContactsOut, b3Int4* clippingFaces, b3Vector3* worldVertsB2,
                                 volatile int* nGlobalContactsOut, int vertexFaceCapacity, int contactCapacity,
                                 int numPairs, int pairIndex);

extern "C" {

// registerConcaveMesh's BVH for one mesh (b3GpuNarrowPhase.cpp:556-610: b3OptimizedBvh::build over
// the unscaled vertices with quantized AABB compression and the mesh's local AABB), then
// b3BvhTraversal for every pair.  The collidable of the mesh must carry BVH index 0.  Writes the
// triangle-convex pairs (int4: bodyA, bodyB, triangle, child or 0) in the traversal's order;
// returns their count (only cap written).
int ref_concave_pairs(const float* mesh_verts, int nverts, const int* mesh_indices, int ntris, const float* aabb_min,
                      const float* aabb_max, const b3RigidBodyData* bodies, const b3Collidable* cols,
                      const b3Aabb* aabbs, int nbodies, const int* pairs, int npairs, int* out, int cap) {
    b3AlignedObjectArray<b3Vector3> V;
    V.resize(nverts);
    for (int i = 0; i < nverts; i++) V[i] = b3MakeVector3(mesh_verts[3 * i], mesh_verts[3 * i + 1], mesh_verts[3 * i + 2]);
    b3AlignedObjectArray<int> I;
    I.resize(3 * ntris);
    for (int i = 0; i < 3 * ntris; i++) I[i] = mesh_indices[i];
    b3TriangleIndexVertexArray meshInterface;
    b3IndexedMesh mesh;
    mesh.m_numTriangles = ntris;
    mesh.m_numVertices = nverts;
    mesh.m_vertexBase = (const unsigned char*)&V.at(0).x;
    mesh.m_vertexStride = sizeof(b3Vector3);
    mesh.m_triangleIndexStride = 3 * sizeof(int);
    mesh.m_triangleIndexBase = (const unsigned char*)&I.at(0);
    meshInterface.addIndexedMesh(mesh);
    b3OptimizedBvh bvh;
    const b3Vector3 mn = b3MakeVector3(aabb_min[0], aabb_min[1], aabb_min[2]);
    const b3Vector3 mx = b3MakeVector3(aabb_max[0], aabb_max[1], aabb_max[2]);
    bvh.build(&meshInterface, true, mn, mx);
    b3BvhInfo info;
    info.m_aabbMin = bvh.m_bvhAabbMin;
    info.m_aabbMax = bvh.m_bvhAabbMax;
    info.m_quantization = bvh.m_bvhQuantization;
    info.m_numNodes = bvh.getQuantizedNodeArray().size();
    info.m_numSubTrees = bvh.getSubtreeInfoArray().size();
    info.m_nodeOffset = 0;
    info.m_subTreeOffset = 0;
    std::vector<b3Aabb> A(aabbs, aabbs + nbodies);
    std::vector<b3Int4> outv(cap > 0 ? cap : 1);
    volatile int n = 0;
    const b3Int4* P = reinterpret_cast<const b3Int4*>(pairs);
    for (int i = 0; i < npairs; i++)
        b3BvhTraversal(P, bodies, cols, A.data(), outv.data(), &n, &bvh.getSubtreeInfoArray()[0],
                       &bvh.getQuantizedNodeArray()[0], &info, npairs, cap, i);
    for (int i = 0; i < n && i < cap; i++) memcpy(&out[4 * i], &outv[i], sizeof(b3Int4));
    return n;
}

// b3FindConcaveSeparatingAxisKernel, clipFacesAndFindContactsKernel and b3NewContactReductionKernel
// for every triangle-convex pair in order (vertexFaceCapacity 64, as the pipeline allocates);
// out_index[m] = the pair's index.  Returns the manifold count.
int ref_concave_contacts(const b3RigidBodyData* bodies, const b3Collidable* cols, const b3ConvexPolyhedronData* hulls,
                         const b3GpuFace* faces, const int* indices, const b3Vector3* verts, const b3Vector3* edges,
                         const b3GpuChildShape* children, const b3Aabb* aabbs, int nbodies, const int* tri_pairs, int n,
                         b3Contact4Data* out, int* out_index, int cap) {
    const int capv = 64;
    const int m = n > 0 ? n : 1;
    std::vector<b3Int4> tp(m);
    memcpy(tp.data(), tri_pairs, sizeof(b3Int4) * n);
    std::vector<b3Aabb> A(aabbs, aabbs + nbodies);
    std::vector<b3Vector3> sep(m), wA1((size_t)m * capv), nA1(m), wB1((size_t)m * capv), wB2((size_t)m * capv);
    std::vector<b3Int4> clip(m);
    std::vector<int> has(m, 0);
    std::vector<b3Contact4Data> tmp(m);
    memset(tmp.data(), 0, sizeof(b3Contact4Data) * m);
    volatile int nc = 0;
    int k = 0;
    for (int i = 0; i < n; i++) {
        b3FindConcaveSeparatingAxisKernel(tp.data(), bodies, cols, hulls, verts, edges, faces, indices, children,
                                          A.data(), sep.data(), clip.data(), wA1.data(), nA1.data(), wB1.data(),
                                          has.data(), capv, n, i);
        clipFacesAndFindContactsKernel(sep.data(), has.data(), clip.data(), wA1.data(), nA1.data(), wB1.data(),
                                       wB2.data(), capv, i);
        const int before = nc;
        b3NewContactReductionKernel(tp.data(), bodies, sep.data(), has.data(), tmp.data(), clip.data(), wB2.data(),
                                    &nc, capv, m, n, i);
        if (nc > before && k < cap) {
            out[k] = tmp[before];
            out_index[k] = i;
            k++;
        }
    }
    return k;
}

// The reference's compound kernels (host twins), one child pair at a time, on the given child pairs
// (int4: bodyA, bodyB, child shape of A or -1, child shape of B or -1; both sides convex hulls):
// processCompoundPairsKernel then clipCompoundsHullHullKernel.  Writes the manifolds in child-pair
// order, out_index[m] = child pair index; returns the count.
int ref_compound_hull_contacts(const b3RigidBodyData* bodies, const b3Collidable* cols,
                               const b3ConvexPolyhedronData* hulls, const b3GpuFace* faces, int nfaces,
                               const int* indices, int nindices, const b3Vector3* verts, int nverts,
                               const b3Vector3* edges, int nedges, const b3GpuChildShape* children,
                               const int* child_pairs, int n, b3Contact4Data* out, int* out_index, int cap) {
    b3AlignedObjectArray<b3Vector3> V, E, sep;
    b3AlignedObjectArray<b3GpuFace> F;
    b3AlignedObjectArray<int> I, has;
    V.resize(nverts);
    for (int i = 0; i < nverts; i++) V[i] = verts[i];
    E.resize(nedges > 0 ? nedges : 1);
    for (int i = 0; i < nedges; i++) E[i] = edges[i];
    F.resize(nfaces);
    for (int i = 0; i < nfaces; i++) F[i] = faces[i];
    I.resize(nindices);
    for (int i = 0; i < nindices; i++) I[i] = indices[i];
    sep.resize(n > 0 ? n : 1);
    has.resize(n > 0 ? n : 1);
    const b3Int4* cp = reinterpret_cast<const b3Int4*>(child_pairs);
    int m = 0;
    std::vector<b3Contact4Data> tmp(1);
    for (int i = 0; i < n; i++) {
        processCompoundPairsKernel(cp, bodies, cols, hulls, V, E, F, I, nullptr, children, sep, has, n, i);
        if (!has[i]) continue;
        int nc = 0;
        memset(&tmp[0], 0, sizeof(b3Contact4Data));
        clipCompoundsHullHullKernel(cp, bodies, cols, hulls, V, E, F, I, children, sep, has, &tmp[0], &nc, n, 64, i);
        if (nc > 0 && m < cap) {
            out[m] = tmp[0];
            out_index[m] = i;
            m++;
        }
    }
    return m;
}

// computeContactPlaneCompound for one (plane body, compound body) pair: one manifold per child
// that touches the plane, in child order.  Returns the count.
int ref_plane_compound_contacts(const b3RigidBodyData* bodies, const b3Collidable* cols,
                                const b3ConvexPolyhedronData* hulls, const b3GpuFace* faces, const int* indices,
                                const b3Vector3* verts, const b3GpuChildShape* children, int plane_body,
                                int compound_body, b3Contact4Data* out, int cap) {
    std::vector<b3Contact4> tmp(cap > 0 ? cap : 1);
    memset(tmp.data(), 0, sizeof(b3Contact4) * tmp.size());
    int nc = 0;
    computeContactPlaneCompound(0, plane_body, compound_body, bodies[plane_body].m_collidableIdx,
                                bodies[compound_body].m_collidableIdx, bodies, cols, hulls, children, verts, indices,
                                faces, tmp.data(), nc, cap);
    for (int i = 0; i < nc && i < cap; i++) memcpy(&out[i], &tmp[i], sizeof(b3Contact4Data));
    return nc;
}

// Hull tables from b3ConvexUtility (+ vertex-mean local centre as registerConvexHullShape sets it).
// counts4 in: capacities (verts, faces, indices, edges); out: sizes.  Returns 0 on success.
int ref_hull(const float* xyz, int n, float* verts_out, float* planes_out, int* face_counts_out, int* indices_out,
             float* edges_out, int* counts4) {
    b3AlignedObjectArray<b3Vector3> pts;
    for (int i = 0; i < n; i++) pts.push_back(b3MakeVector3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
    b3ConvexUtility util;
    util.initializePolyhedralFeatures(&pts[0], pts.size(), true);
    int nv = util.m_vertices.size(), nf = util.m_faces.size(), ne = util.m_uniqueEdges.size(), ni = 0;
    for (int f = 0; f < nf; f++) ni += util.m_faces[f].m_indices.size();
    bool fits = counts4[0] >= nv && counts4[1] >= nf && counts4[2] >= ni && counts4[3] >= ne;
    counts4[0] = nv; counts4[1] = nf; counts4[2] = ni; counts4[3] = ne;
    if (!fits) return 1;
    for (int i = 0; i < nv; i++)
        for (int k = 0; k < 3; k++) verts_out[3 * i + k] = util.m_vertices[i][k];
    int off = 0;
    for (int f = 0; f < nf; f++) {
        for (int k = 0; k < 4; k++) planes_out[4 * f + k] = util.m_faces[f].m_plane[k];
        face_counts_out[f] = util.m_faces[f].m_indices.size();
        for (int k = 0; k < face_counts_out[f]; k++) indices_out[off++] = util.m_faces[f].m_indices[k];
    }
    for (int i = 0; i < ne; i++)
        for (int k = 0; k < 3; k++) edges_out[3 * i + k] = util.m_uniqueEdges[i][k];
    return 0;
}

// World AABBs with b3TransformAabb2, margin 0 (as initializeGpuAabbsFull does per step).
void ref_aabbs(const b3RigidBodyData* bodies, int n, const b3Collidable* cols, const b3Aabb* local_aabbs,
               b3Aabb* out) {
    (void)cols;
    for (int i = 0; i < n; i++) {
        const b3Aabb& la = local_aabbs[bodies[i].m_collidableIdx];
        b3Float4 mn, mx;
        b3TransformAabb2(la.m_minVec, la.m_maxVec, 0.f, bodies[i].m_pos, bodies[i].m_quat, &mn, &mx);
        out[i].m_minVec = mn;
        out[i].m_minIndices[3] = i;
        out[i].m_maxVec = mx;
        out[i].m_signedMaxIndices[3] = bodies[i].m_invMass == 0.f ? 0 : 1;
    }
}

// Pair set from the reference's dynamic-BVH broadphase, filtered by the tight inclusive test
// (b3TestAabbAgainstAabb) and with static-static pairs removed; output (a<b) sorted.
int ref_pairs_dbvt(const b3Aabb* aabbs, int n, int* out_xy, int cap) {
    b3DynamicBvhBroadphase bp(n);
    for (int i = 0; i < n; i++) {
        b3Vector3 mn = b3MakeVector3(aabbs[i].m_min[0], aabbs[i].m_min[1], aabbs[i].m_min[2]);
        b3Vector3 mx = b3MakeVector3(aabbs[i].m_max[0], aabbs[i].m_max[1], aabbs[i].m_max[2]);
        bp.createProxy(mn, mx, i, 0, 1, 1);
    }
    bp.calculateOverlappingPairs();
    b3OverlappingPairCache* cache = bp.getOverlappingPairCache();
    std::vector<std::pair<int, int>> ps;
    for (int k = 0; k < cache->getNumOverlappingPairs(); k++) {
        const b3BroadphasePair& p = cache->getOverlappingPairArray()[k];
        int a = std::min(p.x, p.y), b = std::max(p.x, p.y);
        if (aabbs[a].m_signedMaxIndices[3] == 0 && aabbs[b].m_signedMaxIndices[3] == 0) continue;
        if (!b3TestAabbAgainstAabb(aabbs[a].m_minVec, aabbs[a].m_maxVec, aabbs[b].m_minVec, aabbs[b].m_maxVec))
            continue;
        ps.push_back({a, b});
    }
    std::sort(ps.begin(), ps.end());
    ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
    int np = (int)ps.size();
    for (int k = 0; k < np && k < cap; k++) {
        out_xy[2 * k] = ps[k].first;
        out_xy[2 * k + 1] = ps[k].second;
    }
    return np;
}

// Contacts for each pair with the reference's CPU functions; writes one manifold per pair that
// produced contact (in pair order) and out_pair_index[m] = pair index.  Sphere-sphere and
// plane-sphere have no CPU code in the reference; such pairs are skipped here (return count only).
int ref_contacts(const b3RigidBodyData* bodies, int nbodies, const b3Collidable* cols, int ncols,
                 const b3ConvexPolyhedronData* hulls, int nhulls, const b3GpuFace* faces, int nfaces,
                 const int* indices, int nindices, const b3Vector3* verts, int nverts, const b3Vector3* edges,
                 int nedges, const int* pairs_xy, int npairs, b3Contact4Data* out, int* out_pair_index, int cap) {
    b3AlignedObjectArray<b3RigidBodyData> B;
    B.resize(nbodies);
    for (int i = 0; i < nbodies; i++) B[i] = bodies[i];
    b3AlignedObjectArray<b3Collidable> C;
    C.resize(ncols);
    for (int i = 0; i < ncols; i++) C[i] = cols[i];
    b3AlignedObjectArray<b3ConvexPolyhedronData> H;
    H.resize(nhulls);
    for (int i = 0; i < nhulls; i++) H[i] = hulls[i];
    b3AlignedObjectArray<b3GpuFace> F;
    F.resize(nfaces);
    for (int i = 0; i < nfaces; i++) F[i] = faces[i];
    b3AlignedObjectArray<int> I;
    I.resize(nindices);
    for (int i = 0; i < nindices; i++) I[i] = indices[i];
    b3AlignedObjectArray<b3Float4> V;
    V.resize(nverts);
    for (int i = 0; i < nverts; i++) V[i] = verts[i];
    b3AlignedObjectArray<b3Float4> E;
    E.resize(nedges > 0 ? nedges : 1);
    for (int i = 0; i < nedges; i++) E[i] = edges[i];
    int n = 0;
    for (int p = 0; p < npairs; p++) {
        int a = pairs_xy[2 * p], b = pairs_xy[2 * p + 1];
        int ca = bodies[a].m_collidableIdx, cb = bodies[b].m_collidableIdx;
        int ta = cols[ca].m_shapeType, tb = cols[cb].m_shapeType;
        int before = n;
        if (ta == SHAPE_CONVEX_HULL && tb == SHAPE_CONVEX_HULL) {
            b3AlignedObjectArray<b3Contact4Data> tmp;
            int nc = 0;
            b3ContactConvexConvexSAT(p, a, b, ca, cb, B, C, H, V, E, I, F, tmp, nc, 1);
            if (nc > 0 && n < cap) out[n++] = tmp[0];
        } else {
            b3Contact4 c4;
            memset(&c4, 0, sizeof(c4));
            int nc = 0;
            if (ta == SHAPE_PLANE && tb == SHAPE_CONVEX_HULL)
                computeContactPlaneConvex(p, a, b, ca, cb, bodies, cols, hulls, verts, indices, faces, &c4, nc, 1);
            else if (tb == SHAPE_PLANE && ta == SHAPE_CONVEX_HULL)
                computeContactPlaneConvex(p, b, a, cb, ca, bodies, cols, hulls, verts, indices, faces, &c4, nc, 1);
            else if (ta == SHAPE_SPHERE && tb == SHAPE_CONVEX_HULL)
                computeContactSphereConvex(p, a, b, ca, cb, bodies, cols, hulls, verts, indices, faces, &c4, nc, 1);
            else if (tb == SHAPE_SPHERE && ta == SHAPE_CONVEX_HULL)
                computeContactSphereConvex(p, b, a, cb, ca, bodies, cols, hulls, verts, indices, faces, &c4, nc, 1);
            if (nc > 0 && n < cap) out[n++] = c4;
        }
        if (n > before) out_pair_index[n - 1] = p;
    }
    return n;
}

// b3PgsJacobiSolver(usePgs).solveGroup with 2 friction directions, no warm start (avoids the
// dangling m_originalContactPoint write, b3PgsJacobiSolver.cpp:868,1595-1613), no split impulse.
// use_pgs: 0 Jacobi, 1 PGS, 2 PGS with B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS.
void ref_solve(b3RigidBodyData* bodies, b3InertiaData* inertias, int nbodies, const b3Contact4Data* contacts, int nc,
               int use_pgs, int iterations, float dt) {
    b3AlignedObjectArray<b3Contact4> C;
    C.resize(nc);
    for (int i = 0; i < nc; i++) memcpy(&C[i], &contacts[i], sizeof(b3Contact4Data));
    b3PgsJacobiSolver solver(use_pgs != 0);
    b3ContactSolverInfo info;
    info.m_solverMode = B3_SOLVER_USE_2_FRICTION_DIRECTIONS | B3_SOLVER_SIMD;
    if (use_pgs == 2) info.m_solverMode |= B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS;
    info.m_splitImpulse = false;
    info.m_numIterations = iterations;
    info.m_timeStep = dt;
    solver.solveGroup(bodies, inertias, nbodies, nc ? &C[0] : 0, nc, 0, 0, info);
}

void ref_integrate(b3RigidBodyData* bodies, int n, float dt, float damping, const float* g) {
    b3Float4 grav = b3MakeFloat4(g[0], g[1], g[2], 0.f);
    for (int i = 0; i < n; i++) integrateSingleTransform(bodies, i, dt, damping, grav);
}

// registerPhysicsInstance (b3GpuRigidBodyPipeline.cpp:603-625: the world AABB through the
// reference's own b3TransformAabb with margin 0.01) followed by the record-filling lines of
// b3GpuNarrowPhase::registerRigidBody (b3GpuNarrowPhase.cpp:830-901), in the reference's types:
// b3RigidBodyData and b3InertiaData of one body.  (registerRigidBody itself needs an OpenCL
// context; its arithmetic is these lines.)
void ref_register_body(float mass, const float* position, const float* orientation, int collidableIndex,
                       const float* localMin, const float* localMax, b3RigidBodyData* body, b3InertiaData* inertia) {
    b3Vector3 localAabbMin = b3MakeVector3(localMin[0], localMin[1], localMin[2]);
    b3Vector3 localAabbMax = b3MakeVector3(localMax[0], localMax[1], localMax[2]);
    b3Vector3 aabbMin, aabbMax;
    b3Scalar margin = 0.01f;
    b3Transform t;
    t.setIdentity();
    t.setOrigin(b3MakeVector3(position[0], position[1], position[2]));
    t.setRotation(b3Quaternion(orientation[0], orientation[1], orientation[2], orientation[3]));
    b3TransformAabb(localAabbMin, localAabbMax, margin, t, aabbMin, aabbMax);

    memset(body, 0, sizeof(*body));
    body->m_frictionCoeff = 1.f;
    body->m_restituitionCoeff = 0.f;
    body->m_angVel = b3MakeVector3(0, 0, 0);
    body->m_linVel = b3MakeVector3(0, 0, 0);
    body->m_pos = b3MakeVector3(position[0], position[1], position[2]);
    body->m_quat.setValue(orientation[0], orientation[1], orientation[2], orientation[3]);
    body->m_collidableIdx = collidableIndex;
    body->m_invMass = mass ? 1.f / mass : 0.f;
    memset(inertia, 0, sizeof(*inertia));
    if (mass == 0.f) {
        inertia->m_initInvInertia.setValue(0, 0, 0, 0, 0, 0, 0, 0, 0);
        inertia->m_invInertiaWorld.setValue(0, 0, 0, 0, 0, 0, 0, 0, 0);
    } else {
        b3Vector3 halfExtents = (aabbMax - aabbMin);
        b3Vector3 localInertia;
        float lx = 2.f * halfExtents[0];
        float ly = 2.f * halfExtents[1];
        float lz = 2.f * halfExtents[2];
        localInertia.setValue((mass / 12.0f) * (ly * ly + lz * lz), (mass / 12.0f) * (lx * lx + lz * lz),
                              (mass / 12.0f) * (lx * lx + ly * ly));
        b3Vector3 invLocalInertia;
        invLocalInertia[0] = 1.f / localInertia[0];
        invLocalInertia[1] = 1.f / localInertia[1];
        invLocalInertia[2] = 1.f / localInertia[2];
        invLocalInertia[3] = 0.f;
        inertia->m_initInvInertia.setValue(invLocalInertia[0], 0, 0, 0, invLocalInertia[1], 0, 0, 0,
                                           invLocalInertia[2]);
        b3Matrix3x3 m(body->m_quat);
        inertia->m_invInertiaWorld = m.scaled(invLocalInertia) * m.transpose();
    }
}

// b3GpuRaycast::castRaysHost (b3GpuRaycast.cpp:175-247), the reference's CPU twin of its ray
// kernels: every body in index order, spheres by sphere_intersect, hulls by rayConvex in the
// body's frame.  It reads no member of the b3GpuRaycast object (whose constructor compiles
// OpenCL programs), so it is called on uninitialised storage of the class; of the narrowphase
// data it reads the hull records and faces only.  hits: in/out (hitFraction is the bound).
void ref_cast_rays(const b3RayInfo* rays, int nrays, b3RayHit* hits, const b3RigidBodyData* bodies, int nbodies,
                   const b3Collidable* cols, int ncols, const b3ConvexPolyhedronData* hulls, int nhulls,
                   const b3GpuFace* faces, int nfaces) {
    b3AlignedObjectArray<b3RayInfo> r;
    b3AlignedObjectArray<b3RayHit> h;
    for (int i = 0; i < nrays; i++) {
        r.push_back(rays[i]);
        h.push_back(hits[i]);
    }
    b3GpuNarrowPhaseInternalData* npd = new b3GpuNarrowPhaseInternalData();
    for (int i = 0; i < nhulls; i++) npd->m_convexPolyhedra.push_back(hulls[i]);
    for (int i = 0; i < nfaces; i++) npd->m_convexFaces.push_back(faces[i]);
    alignas(16) static unsigned char storage[sizeof(b3GpuRaycast)];
    reinterpret_cast<b3GpuRaycast*>(storage)->castRaysHost(r, h, nbodies, bodies, ncols, cols, npd);
    for (int i = 0; i < nrays; i++) hits[i] = h[i];
    delete npd;
}

// Joints through the reference's CPU constraint classes and b3PgsJacobiSolver (PGS, no
// contacts): type 3 = b3Point2PointConstraint(a, b, pivotInA, pivotInB), type 4 =
// b3FixedConstraint(a, b, frameInA = (identity, pivotInA), frameInB = (inverse(relTargetAB),
// pivotInB)) so that its m_relTargetAB equals the given one.  spec per joint: type, a, b, then
// pivotInA xyz, pivotInB xyz, relTargetAB xyzw (10 floats after the 3 ints, as floats).
void ref_solve_joints(b3RigidBodyData* bodies, b3InertiaData* inertias, int nbodies, const int* types, const int* ab,
                      const float* params, int njoints, int iterations, float dt) {
    b3AlignedObjectArray<b3TypedConstraint*> cons;
    for (int j = 0; j < njoints; j++) {
        const float* p = params + 10 * j;
        b3Vector3 pa = b3MakeVector3(p[0], p[1], p[2]), pb = b3MakeVector3(p[3], p[4], p[5]);
        if (types[j] == 3) {
            cons.push_back(new b3Point2PointConstraint(ab[2 * j], ab[2 * j + 1], pa, pb));
        } else {
            b3Transform fa, fb;
            fa.setIdentity();
            fa.setOrigin(pa);
            fb.setIdentity();
            fb.setOrigin(pb);
            fb.setRotation(b3Quaternion(p[6], p[7], p[8], p[9]).inverse());
            cons.push_back(new b3FixedConstraint(ab[2 * j], ab[2 * j + 1], fa, fb));
        }
    }
    b3PgsJacobiSolver solver(true);
    b3ContactSolverInfo info;
    info.m_solverMode = B3_SOLVER_USE_2_FRICTION_DIRECTIONS | B3_SOLVER_SIMD;
    info.m_splitImpulse = false;
    info.m_numIterations = iterations;
    info.m_timeStep = dt;
    solver.solveGroup(bodies, inertias, nbodies, 0, 0, njoints ? &cons[0] : 0, njoints, info);
    for (int j = 0; j < cons.size(); j++) delete cons[j];
}

int ref_sizeof(int which) {
    switch (which) {
        case 0: return (int)sizeof(b3RigidBodyData);
        case 1: return (int)sizeof(b3InertiaData);
        case 2: return (int)sizeof(b3Collidable);
        case 3: return (int)sizeof(b3ConvexPolyhedronData);
        case 4: return (int)sizeof(b3GpuFace);
        case 5: return (int)sizeof(b3Aabb);
        case 6: return (int)sizeof(b3Contact4Data);
    }
    return -1;
}

}  // extern "C"
