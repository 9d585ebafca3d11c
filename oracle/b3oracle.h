/*
 * b3oracle.h -- CPU oracle for the GPU rigid-body step.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU algorithms for this path (each function
 * cites the reference file:line it follows).  Only the test-suite, the smoke check and
 * the bench's CPU-baseline leg load it; the product library never links or calls it.
 *
 * Parity pin: the restatement is checked against outputs of the reference's own code,
 * compiled in place from its sources (oracle/build_ref.sh -> oracle/_ref), and the
 * resulting golden vectors are committed under tests/golden/.
 *
 * Arithmetic: compiled with -ffp-contract=off; every formula uses the same evaluation
 * order as the CUDA kernels, so all stages except the integrator's sinf/cosf agree bit-for-bit.
 * Layouts are byte-identical to the reference structs (b3RigidBodyData 80 B, b3InertiaData 96 B,
 * b3Collidable 16 B, b3ConvexPolyhedronData 96 B, b3GpuFace 32 B, b3Aabb 32 B, b3Contact4Data 112 B).
 */
#ifndef B3ORACLE_H
#define B3ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x, y, z, w; } of4;
typedef struct { of4 pos, quat, linVel, angVel; int collidableIdx; float invMass, restitution, friction; } obody;
typedef struct { of4 row[3]; } omat3;
typedef struct { omat3 invInertiaWorld, initInvInertia; } oinertia;
typedef struct { int numChildShapes; float radius; int shapeType; int shapeIndex; } ocollidable;
typedef struct {
    of4 localCenter, extents, mC, mE;
    float radius;
    int faceOffset, numFaces, numVertices, vertexOffset, uniqueEdgesOffset, numUniqueEdges, unused;
} ohull;
typedef struct { of4 plane; int indexOffset, numIndices, pad0, pad1; } oface;
typedef struct { float minv[3]; int minw; float maxv[3]; int maxw; } oaabb;
typedef struct {
    of4 worldPosB[4];
    of4 worldNormalOnB;
    unsigned short restitutionCmp, frictionCmp;
    int batchIdx, bodyA, bodyB, childIndexA, childIndexB, unused1, unused2;
} ocontact;
typedef struct { int x, y, z, w; } opair;
/* b3GpuChildShape (Bullet3Collision/NarrowPhaseCollision/shared/b3Collidable.h:41-62): child pose
 * and its convex hull collidable */
typedef struct { of4 pos, orn; int shapeIndex, numChildShapes, collidableShapeIndex, shapeType; } ochild;

typedef struct {
    const ocollidable* cols;
    const oaabb* local_aabbs;
    const ohull* hulls;
    const oface* faces;
    const int* indices;
    const of4* verts;
    const of4* edges;
    int num_collidables;
    const ochild* children; /* child shapes of the compounds (collidable.shapeIndex = first child) */
} oshapes;

/* 1 = OpenMP threads available in this build */
int oracle_num_threads(void);
void oracle_set_threads(int n);

/* b3TransformAabb2 (Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h:24-43), margin 0,
 * min.w = body index, max.w = invMass != 0 */
void oracle_aabbs(const obody* bodies, int n, const oshapes* sh, oaabb* out);

/* Exact overlapping pairs (a < b, sorted) of the given AABBs, static-static excluded.
 * brute force restates b3GpuGridBroadphase::calculateOverlappingPairsHost
 * (src/Bullet3OpenCL/BroadphaseCollision/b3GpuGridBroadphase.cpp:260-294) with the inclusive
 * test of gridBroadphase.cl:89-94; returns the pair count (may exceed cap; only cap written). */
int oracle_pairs_bruteforce(const oaabb* aabbs, int n, opair* out, int cap);
/* Same set through a sort-based uniform grid (cell >= every dynamic AABB extent) for large n. */
int oracle_pairs_grid(const oaabb* aabbs, int n, float cell, opair* out, int cap);

/* Contact manifolds for each pair in order (one manifold or none per pair); returns count,
 * writes pair.z = manifold index or -1.  See b3oracle.c for the per-shape reference functions. */
int oracle_contacts(const obody* bodies, const oshapes* sh, opair* pairs, int npairs, ocontact* out, int cap,
                    unsigned short friction_cmp);

/* Local AABB of a compound of n children (child_local[i] = the local AABB of child i's hull). */
void oracle_compound_local_aabb(const oaabb* child_local, const ochild* children, int n, oaabb* out);
/* Compound pairs: the child pairs (bodyA, bodyB, child shape of A or -1, child shape of B or -1) of
 * every pair with a compound, in (pair, child of A, child of B) order; returns the count (only cap
 * written). */
int oracle_compound_pairs(const obody* bodies, const oshapes* sh, const opair* pairs, int npairs, opair* out,
                          int cap);
/* One manifold or none per child pair (hull children: processCompoundPairsKernel +
 * clipCompoundsHullHullKernel; plane against a child: computeContactPlaneCompound), in child-pair
 * order; out_index[m] = child pair index.  Returns the count. */
int oracle_compound_contacts(const obody* bodies, const oshapes* sh, const opair* child_pairs, int n, ocontact* out,
                             int* out_index, int cap);

/* Concave meshes (collidable shapeType 5: a shape record whose faces are the triangles, the
 * collidable's numChildShapes = its BVH index).  Triangle-convex pairs (mesh body, other body,
 * triangle, child shape of a compound or 0) of the pairs whose first body is a mesh and whose second
 * a hull or a compound, in (pair, triangle, child) order: the triangles whose quantized leaf box
 * overlaps the second body's quantized world AABB (b3BvhTraversal, shared/b3BvhTraversal.h:11-111).
 * aabbs: the world AABBs by body.  Returns the count (only cap written). */
int oracle_concave_pairs(const obody* bodies, const oshapes* sh, const oaabb* aabbs, const opair* pairs, int npairs,
                         opair* out, int cap);
/* One manifold or none per triangle-convex pair (b3FindConcaveSeparatingAxisKernel,
 * b3FindClippingFaces, clipFacesAndFindContactsKernel, b3NewContactReductionKernel), in pair order;
 * out_index[m] = the pair's index.  Returns the count. */
int oracle_concave_contacts(const obody* bodies, const oshapes* sh, const oaabb* aabbs, const opair* tri_pairs, int n,
                            ocontact* out, int* out_index, int cap);

/* b3PgsJacobiSolver::solveGroup (Bullet3Dynamics/ConstraintSolver/b3PgsJacobiSolver.cpp:170)
 * with USE_2_FRICTION_DIRECTIONS, no warm start, no split impulse, erp, contact threshold.
 * mode 0 = PGS (usePgs=true, sequential row order), 1 = Jacobi (mass splitting), 2 = PGS with
 * B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS (per point: contact row, then its friction rows).
 * impulses_out (optional): 12 floats per manifold: per point (normal, lateral1, lateral2).
 * Returns the number of iterations run. residual_out (optional): last relative residual. */
int oracle_solve(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts, int ncontacts,
                 int mode, int iterations, float dt, float erp, float threshold, float residual_tol,
                 float* impulses_out, float* residual_out);
/* Solve in a given manifold order (PGS only): order[k] = manifold index solved k-th; interleave as
 * mode 2 of oracle_solve. */
int oracle_solve_ordered(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts,
                         int ncontacts, const int* order, int interleave, int iterations, float dt, float erp,
                         float threshold, float* impulses_out);

/* oracle_solve_ordered with a warm start (warm: 12 floats per manifold, per point normal,
 * first lateral (dir1), second lateral (dir2) -- the layout of impulses_out; NULL = cold), a
 * residual tolerance (0 = run all iterations) and the warm-start fallback: a warm start whose
 * first-sweep residual exceeds 1 (a cold start's) is dropped and the solve restarts cold
 * (*discarded_out = 1; the dropped sweep counts in the returned iteration count). */
int oracle_solve_ordered_ex(obody* bodies, const oinertia* inertias, int nbodies, const ocontact* contacts,
                            int ncontacts, const int* order, int interleave, const float* warm, int iterations,
                            float dt, float erp, float threshold, float residual_tol, float* impulses_out,
                            float* residual_out, int* discarded_out);

/* integrateSingleTransform (Bullet3Dynamics/shared/b3IntegrateTransforms.h:5-55) for every body */
void oracle_integrate(obody* bodies, int n, float dt, float damping, const float gravity[3]);

/* Batch legality: no dynamic body appears twice within one colour.  Returns the number of
 * violations (0 = legal); statics (invMass 0) never conflict. */
int oracle_check_batches(const ocontact* contacts, int n, const int* color, const obody* bodies, int nbodies);

/* One full step (AABB, pairs, contacts, solve, integrate); returns the manifold count. */
typedef struct {
    float dt, damping, gravity[3], erp, threshold, cell, residual_tol;
    int mode, iterations, use_grid;
    unsigned short friction_cmp;
} ostep_params;
int oracle_step(obody* bodies, const oinertia* inertias, int n, const oshapes* sh, const ostep_params* p,
                int* npairs_out, int* npoints_out);

/* Ray casts (b3GpuRaycast::castRays, Bullet3OpenCL/Raycast/b3GpuRaycast.cpp:248-373, whose per-ray
 * work is rayCastPairsKernel / rayCastKernel, kernels/rayCastKernels.cl:261-439): for every ray,
 * the bodies in index order; hulls by rayConvex (:157-217) in the body's frame (qtRotate
 * quaternion form), spheres by sphere_intersect (:224-248); planes and other shapes are skipped;
 * a body equal to the hit's m_hitResult2 on input is skipped.  Output per ray: hitFraction 1 when
 * nothing is hit, else the closest fraction, hit body, interpolated point and normalised normal
 * (a hull's face normal in the body's frame, as the kernel returns it).  With body_scene, ray r
 * only sees the bodies of scene (int)from.w. */
typedef struct { of4 from, to; } oray;
typedef struct { float hitFraction; int hitBody, hitResult1, hitResult2; of4 hitPoint, hitNormal; } oray_hit;
void oracle_cast_rays(const obody* bodies, int nbodies, const oshapes* sh, const oray* rays, oray_hit* hits,
                      int nrays, const int* body_scene);

/* Joints (b3GpuGenericConstraint, Bullet3OpenCL/RigidBody/b3GpuGenericConstraint.h:77-93):
 * type 3 point to point, 4 fixed; flags bit 0 = enabled. */
typedef struct {
    int type, rbA, rbB;
    float breakingImpulseThreshold;
    of4 pivotInA, pivotInB, relTargetAB;
    int flags, uid, pad[2];
} ojoint;
/* The joint solver's batching (initBatchConstraintsKernel, kernels/jointSolver.cl:400-419, then
 * b3GpuPgsConstraintSolver::sortConstraintByBatch3, b3GpuPgsConstraintSolver.cpp:781-907, with
 * simdWidth = n + 1 and staticIdx = -1).  Writes the joint indices batch by batch into order[n]
 * and the batch offsets into batch_off[nbatches + 1]; returns nbatches. */
int oracle_joint_batches(const ojoint* joints, int n, const obody* bodies, int nbodies, int* order, int* batch_off);
/* b3GpuPgsConstraintSolver::solveJoints (b3GpuPgsConstraintSolver.cpp:927-944): rows of every
 * joint (getInfo2Kernel, jointSolver.cl:651-870), 4 PGS iterations over the batches in order
 * (solveJointConstraintRows, :303-329), the break check (:352-371) and the velocity write-back
 * (:631-648).  Updates the bodies' velocities and the joints' flags in place. */
void oracle_solve_joints(obody* bodies, const oinertia* inertias, int nbodies, ojoint* joints, int n,
                         const int* order, const int* batch_off, int nbatches);
/* The acos the joint rows use (asin Maclaurin series with half-angle reduction). */
float oracle_joint_acos(float x);

/* Shape and body registration (oracle/b3hull.c).  oracle_hull: the hull tables
 * registerConvexHullShape builds from a point cloud (b3ConvexHullComputer + b3ConvexUtility +
 * vertex-mean local centre): vertices xyz, face planes xyzw, face index counts and indices, unique
 * edge directions xyz.  counts4 in: capacities (vertices, faces, indices, edges); out: sizes.
 * Returns 0, 1 when a buffer is too small, -1 on allocation failure. */
int oracle_hull(const float* xyz, int n, float* verts_out, float* planes_out, int* face_counts_out,
                int* indices_out, float* edges_out, float* center_out, int* counts4);
/* registerPhysicsInstance + registerRigidBody: the body record (b3RigidBodyData, 20 floats) and
 * the inertia record (b3InertiaData, 24 floats) for a body of the given shape's local AABB. */
int oracle_register_body(float mass, const float pos[3], const float orn[4], int collidable, const float local_min[3],
                         const float local_max[3], float* body_out, float* inertia_out);

#ifdef __cplusplus
}
#endif

#endif
