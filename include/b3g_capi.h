/*
 * b3g_capi.h -- C ABI of the GB300-native GPU rigid-body step.
 *
 * This is the thin boundary that the drop-in C++ classes (b3GpuRigidBodyPipeline,
 * b3GpuNarrowPhase, b3GpuGridBroadphase; see include/b3g_compat.h) and foreign
 * bindings (ctypes, cgo, JNI) call.  Plain pointers and sizes only; every entry
 * point returns a b3gStatus (0 = ok) and never aborts.  Each function names the
 * reference interface it replaces (paths relative to the reference project root,
 * src/Bullet3OpenCL/...).
 *
 * Threading: one world per host thread, one CUDA stream per world, exactly like
 * the reference's single in-order cl_command_queue (b3GpuRigidBodyPipeline.h:33).
 * Device pointers returned by getters are borrowed and stay valid until the next
 * b3g_write_all_to_gpu / b3g_destroy.
 */
#ifndef B3G_CAPI_H
#define B3G_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct b3gWorld* b3g_handle;

typedef enum b3gStatus {
    B3G_OK = 0,
    B3G_ERR_INVALID_ARG = 1,      /* null handle / pointer, bad size */
    B3G_ERR_INVALID_INDEX = 2,    /* reference returns -1 + b3Error (b3GpuRigidBodyPipeline.cpp:620-624) */
    B3G_ERR_CAPACITY = 3,         /* a b3Config capacity was exceeded (b3GpuNarrowPhase.cpp:821-825) */
    B3G_ERR_CUDA = 4,             /* a CUDA runtime call failed; see b3g_last_error() */
    B3G_ERR_NOT_UPLOADED = 5,     /* step/stage called before b3g_write_all_to_gpu */
    B3G_ERR_UNSUPPORTED = 6,      /* compound / concave shapes */
    B3G_ERR_BARRIER_TIMEOUT = 7,  /* a persistent kernel's bounded grid barrier gave up */
    B3G_ERR_DEGENERATE = 8        /* convex hull input is degenerate (fewer than 4 affinely independent points) */
} b3gStatus;

/* Device-side status word bits (b3g_status). Set by kernels, read once per step. */
#define B3G_FLAG_PAIR_OVERFLOW     0x1u   /* reference: b3GpuGridBroadphase.cpp:164-168,233-237 */
#define B3G_FLAG_CONTACT_OVERFLOW  0x2u   /* reference: b3ConvexHullContact.cpp:2851-2855,4358-4362 */
#define B3G_FLAG_BATCH_OVERFLOW    0x4u   /* reference: b3GpuPgsContactSolver.cpp:1499-1504 */
#define B3G_FLAG_BARRIER_TIMEOUT   0x8u
#define B3G_FLAG_NAN               0x10u
#define B3G_FLAG_CLIP_OVERFLOW     0x20u
#define B3G_FLAG_MLP_TIMEOUT       0x40u  /* a tensor-core wait of the warm-start network gave up */
#define B3G_FLAG_WARM_DISCARDED    0x80u  /* a warm start was worse than a cold start and was dropped */

#define B3G_SOLVER_PGS 0      /* b3PgsJacobiSolver(true)  -- graph-coloured Gauss-Seidel on the GPU */
#define B3G_SOLVER_JACOBI 1   /* b3PgsJacobiSolver(false) -- mass-splitting Jacobi */

/* PGS work split.  NONE: every manifold is solved grid-wide, one grid barrier per colour.
 * SHARED: each block owns a contiguous range of the dynamic bodies in broadphase cell order and
 * solves the manifolds inside its range alone, the range's body deltas and inverse inertias staged
 * in shared memory (the rest run grid-wide); STREAMED: the same with the block's manifold records
 * streamed through shared memory in bulk-copied tiles; GLOBAL_DELTAS: the same ranges with the
 * deltas left in global memory.  AUTO uses the split b3g_autotune measured fastest on the world's
 * own state when it has run, else NONE (the fastest measured on GB300 for piles of 256k boxes).
 * All are legal Gauss-Seidel orders. */
#define B3G_PGS_PARTITIONS_AUTO 0
#define B3G_PGS_PARTITIONS_GLOBAL_DELTAS 1
#define B3G_PGS_PARTITIONS_NONE 2
#define B3G_PGS_PARTITIONS_SHARED 3
#define B3G_PGS_PARTITIONS_STREAMED 4

/* Warm start of the PGS solve (b3gConfig.warm_start).  A contact point "persists" when the
 * previous step had a manifold for the same body pair with a point within 0.05 of it (points on
 * body B, world space); persisting points then start from that point's converged impulses, as
 * B3_SOLVER_USE_WARMSTARTING does with cached contact points.  LEARNED predicts the initial
 * impulses of every point with the network attached by b3g_set_warm_start_model;
 * PERSISTENT_LEARNED predicts only the new points.  RECORD starts cold and records the
 * network's features and the points' persistence for training (b3g_read_warm_samples).
 * Whatever the source, a warm start whose first sweep has a residual above a cold start's (1) is
 * dropped and the solve restarts cold (B3G_FLAG_WARM_DISCARDED).  Without a network attached,
 * LEARNED is cold and PERSISTENT_LEARNED is PERSISTENT. */
#define B3G_WARM_COLD 0
#define B3G_WARM_LEARNED 1
#define B3G_WARM_RECORD 2
#define B3G_WARM_PERSISTENT 3
#define B3G_WARM_PERSISTENT_LEARNED 4

/* One configuration struct replaces b3Config (b3Config.h:4-37) plus the constants the
 * reference hard-codes (dt 1/60 b3GpuPgsContactSolver.cpp:672, damping 0.99
 * b3GpuRigidBodyPipeline.cpp:468, gravity :92, friction 0.7 b3ConvexHullContact.cpp:1384). */
typedef struct b3gConfig {
    int max_bodies;            /* m_maxConvexBodies */
    int max_shapes;            /* m_maxConvexShapes (collidables) */
    int max_pairs;             /* m_maxBroadphasePairs; 0 = 8 * max_bodies */
    int max_contacts;          /* m_maxContactCapacity; 0 = 4 * max_bodies */
    float grid_cell_size;      /* 0 = automatic: the largest world-AABB extent any dynamic body can reach */
    int grid_dim;              /* cells per axis, power of two (reference: 128, b3GpuGridBroadphase.cpp:38-49) */
    float gravity[3];
    float angular_damping;     /* 0.99 */
    int solver_mode;           /* B3G_SOLVER_PGS or B3G_SOLVER_JACOBI */
    int solver_iterations;     /* b3ContactSolverInfo::m_numIterations */
    float erp;                 /* Baumgarte factor, b3ContactSolverInfo::m_erp = 0.2 */
    float contact_threshold;   /* contact processing threshold 0.02 (b3PgsJacobiSolver.h:44) */
    float contact_friction;    /* friction stored in every contact: 0.7 as in the reference */
    float residual_tol;        /* >0: stop PGS/Jacobi when the impulse residual drops below it */
    int update_world_inertia;  /* 0 = reference behaviour (world inverse inertia frozen at registration) */
    int use_cuda_graph;        /* capture the whole step as one CUDA graph */
    int warm_start;            /* B3G_WARM_*: initial impulses of the PGS solve (0 = cold, the reference) */
    int barrier_spin_limit;    /* polls before a grid barrier gives up (0 = default, about a second) */
    int solver_blocks_per_sm;  /* persistent solver blocks per SM (0 = default; clamped to co-residency) */
    int pgs_partitions;        /* B3G_PGS_PARTITIONS_*: how the PGS solver splits work across blocks */
    int pgs_interleave;        /* 1: PGS rows in the order of B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS
                                  (per point: contact row, then its two friction rows), one pass per iteration;
                                  0: all contact rows, then all friction rows (the reference default).
                                  PGS only; the Jacobi solver ignores it */
    int warm_start_max_points; /* point slots (4 per manifold, in manifold order) that get features and
                                  predictions when warm_start != 0; 0 = 8 x bodies (at least 8192) */
    int autotune;              /* 1: the first b3g_step after an upload runs b3g_autotune (3 repeats) */
    int broadphase;            /* B3G_BROADPHASE_GRID (0), _LBVH (1) or _AUTO (2), see b3g_set_broadphase */
    int pgs_tail_manifolds;    /* PGS with grid-wide colours: the trailing colours of at most this many
                                  manifolds each are solved by one block, one grid barrier for all of
                                  them (0 = 32: a colour that fits one warp; measured on GB300, larger
                                  tails serialise their colours on one SM and cost more than the
                                  barriers they save; 1 effectively turns it off) */
    int pgs_flow;              /* PGS with grid-wide colours and a fixed sweep count (no residual_tol, no
                                  warm start): 1 = dataflow sweeps (per-body update counters instead of
                                  a grid barrier per colour; same order, same results); 0 (default) and
                                  2 = a grid barrier per colour, measured faster on GB300 from 16k to
                                  300k manifolds */
    int max_compound_child_pairs;  /* child pairs of the compound pairs per step (0 = max_pairs); only
                                      allocated when a compound is registered */
    int max_concave_pairs;     /* triangle-convex pairs of the concave-mesh pairs per step
                                  (m_maxTriConvexPairCapacity; 0 = max_pairs); only allocated when a
                                  concave mesh is registered */
    float warm_start_factor;   /* B3G_WARM_PERSISTENT*: the persisting points' carried impulses are
                                  scaled by this (b3ContactSolverInfo::m_warmstartingFactor, 0.85 in
                                  the reference's B3_SOLVER_USE_WARMSTARTING); 0 counts as 1 */
} b3gConfig;

/* Per-step counters, copied once per step from the device. */
typedef struct b3gStepStats {
    int num_pairs;
    int num_contacts;       /* manifolds */
    int num_points;         /* contact points (rows) */
    int num_colors;         /* PGS batches */
    int iterations;         /* solver sweeps actually run */
    float residual;         /* last relative impulse residual (0 if not tracked) */
    unsigned int status;    /* B3G_FLAG_* bits */
    int num_large;          /* bodies handled by the large-AABB path */
    int num_child_pairs;    /* compound child pairs of the last contact stage (after the capacity clamp) */
    int num_concave_pairs;  /* triangle-convex pairs of the last contact stage (after the capacity clamp) */
} b3gStepStats;

/* ------------------------------------------------------------------ lifetime */
/* Fills the defaults listed above. */
b3gStatus b3g_config_default(b3gConfig* cfg);
/* Replaces the b3GpuNarrowPhase + b3GpuGridBroadphase + b3GpuRigidBodyPipeline constructors
 * (b3GpuNarrowPhase.cpp:18, b3GpuGridBroadphase.cpp:24, b3GpuRigidBodyPipeline.cpp:65).
 * Host registries only; no device memory is touched until b3g_write_all_to_gpu. */
b3gStatus b3g_create(const b3gConfig* cfg, int cuda_device, b3g_handle* out);
b3gStatus b3g_destroy(b3g_handle h);
/* b3GpuNarrowPhase::reset (b3GpuNarrowPhase.cpp:946-962) with what = B3G_RESET_SHAPES_AND_BODIES:
 * every shape and body is dropped (and the device state freed; the next b3g_write_all_to_gpu
 * uploads afresh); b3GpuRigidBodyPipeline::reset (b3GpuRigidBodyPipeline.cpp:141-147) with
 * B3G_RESET_CONSTRAINTS: every joint is dropped.  Flags may be combined; the configuration,
 * device, stream and attached network stay. */
#define B3G_RESET_SHAPES_AND_BODIES 1
#define B3G_RESET_CONSTRAINTS 2
b3gStatus b3g_reset(b3g_handle h, int what);
/* Text of the last error on this thread. */
const char* b3g_last_error(void);
/* Library version string. */
const char* b3g_version(void);

/* ------------------------------------------------------------------ shapes (b3GpuNarrowPhase) */
/* b3GpuNarrowPhase::registerSphereShape (b3GpuNarrowPhase.cpp:159) */
b3gStatus b3g_register_sphere(b3g_handle h, float radius, int* out_collidable);
/* b3GpuNarrowPhase::registerPlaneShape (b3GpuNarrowPhase.cpp:202) */
b3gStatus b3g_register_plane(b3g_handle h, const float normal[3], float constant, int* out_collidable);
/* b3GpuNarrowPhase::registerConvexHullShape(const float*, int stride, int n, const float* scaling)
 * (b3GpuNarrowPhase.cpp:298-314): builds the hull, merges coplanar faces, finds unique edges. */
b3gStatus b3g_register_hull(b3g_handle h, const float* verts, int stride_bytes, int num_verts,
                            const float scaling[3], int* out_collidable);
/* b3GpuNarrowPhase::registerConvexHullShape(b3ConvexUtility*) (b3GpuNarrowPhase.cpp:316-368):
 * registers precomputed hull tables (vertices xyz, faces as plane + index lists, unique edges).
 * face_planes: 4 floats per face; face_index_counts: indices per face; face_indices: flat.
 * The local centre is the vertex mean, as in the reference (:324-329). */
b3gStatus b3g_register_hull_tables(b3g_handle h, const float* verts_xyz, int num_verts,
                                   const float* face_planes, const int* face_index_counts, int num_faces,
                                   const int* face_indices, const float* unique_edges_xyz, int num_edges,
                                   int* out_collidable);
/* b3GpuNarrowPhase::registerCompoundShape (b3GpuNarrowPhase.cpp:370-433): a compound of convex
 * hulls (each child's shapeIndex an earlier hull collidable).  Its local AABB is the union of the
 * children's, moved into the compound's frame (b3TransformAabb, margin 0).  A pair with a compound
 * expands into child pairs (compound-compound: children whose world AABBs overlap; compound against
 * a hull or a plane: every child), one manifold per child pair at most, as the reference's
 * findCompoundPairsKernel / processCompoundPairsKernel / clipCompoundsHullHullKernel
 * (b3ConvexHullContact.cpp:1419-2022) and computeContactPlaneCompound (:2182) compute them.  Compounds
 * against spheres give no contacts. */
struct b3gChildShape;
struct b3gBvhInfo;
struct b3gBvhNode;
b3gStatus b3g_register_compound(b3g_handle h, const struct b3gChildShape* children, int num_children,
                                int* out_collidable);
/* Host copy of the registered compound children (b3gChildShape, b3g_types.h; capacity 0: count only). */
b3gStatus b3g_read_child_shapes(b3g_handle h, struct b3gChildShape* host_children, int capacity, int* num);
/* b3GpuNarrowPhase::registerConcaveMesh (b3GpuNarrowPhase.cpp:521-613) + registerConcaveMeshShape
 * (:615-667): a static triangle mesh.  vertices: num_vertices points stride_bytes apart (>= 12),
 * indices: 3 per triangle; scaling multiplies the vertices.  The collidable's shape record lists
 * the triangles as faces (plane = normalised (v1 - v0) x (v2 - v0), w = -n.v0) and a quantized BVH
 * over them (b3g_read_mesh_bvh).  A mesh collides with hulls and compounds (one manifold per
 * touching triangle, or triangle and child, as b3BvhTraversal / b3FindConcaveSeparatingAxisKernel /
 * clipFacesAndFindContactsKernel / b3NewContactReductionKernel compute them), and with spheres (one
 * point per touching triangle, computeContactSphereTriangle) when its body is the pair's first
 * (lower index), as in the reference; not with planes or other meshes.  The
 * reference traverses with the other body's world AABB in the mesh's own frame, so meshes are
 * meant to stay at the identity pose.  -> -1 + b3Error in the Python / C++ layers on invalid input. */
b3gStatus b3g_register_concave_mesh(b3g_handle h, const float* vertices, int stride_bytes, int num_vertices,
                                    const int* indices, int num_triangles, const float scaling[3],
                                    int* out_collidable);
/* Host copy of the meshes' BVHs (b3gBvhInfo / b3gBvhNode, b3g_types.h; capacities 0: counts only). */
b3gStatus b3g_read_mesh_bvh(b3g_handle h, struct b3gBvhInfo* infos, int capacity_infos, struct b3gBvhNode* nodes,
                            int capacity_nodes, int* num_infos, int* num_nodes);

/* ------------------------------------------------------------------ bodies (b3GpuRigidBodyPipeline) */
/* b3GpuRigidBodyPipeline::registerPhysicsInstance (b3GpuRigidBodyPipeline.cpp:603-669) together with
 * b3GpuNarrowPhase::registerRigidBody (b3GpuNarrowPhase.cpp:816-908): world AABB with margin 0.01,
 * AABB-box inertia, mass 0 => static large proxy. */
b3gStatus b3g_register_body(b3g_handle h, float mass, const float pos[3], const float orn[4],
                            int collidable, int user_index, int* out_body);
/* writeAllInstancesToGpu (b3GpuRigidBodyPipeline.cpp:597) + writeAllBodiesToGpu
 * (b3GpuNarrowPhase.cpp:915-944) + writeAabbsToGpu (b3GpuGridBroadphase.cpp:297-302):
 * allocates every device buffer at its capacity and uploads the registries. */
b3gStatus b3g_write_all_to_gpu(b3g_handle h);
/* b3GpuRigidBodyPipeline::setGravity (b3GpuRigidBodyPipeline.cpp:587-590) */
b3gStatus b3g_set_gravity(b3g_handle h, const float g[3]);
/* Changes the solver mode / iteration count / residual target between steps. */
b3gStatus b3g_set_solver(b3g_handle h, int mode, int iterations, float residual_tol);

/* Batched independent scenes.  The reference steps one world per pipeline; a batch of N scenes
 * there is N pipelines stepped one after another (b3GpuRigidBodyPipeline::stepSimulation,
 * b3GpuRigidBodyPipeline.cpp:221-463, once per scene).  Here one world holds every scene and one
 * step advances them all: scene s owns the bodies [first_body[s], first_body[s+1]) (the last scene
 * runs to the last registered body), including its own static bodies (planes), and no pair is
 * formed across scenes, even where scenes occupy the same region of space.  Each scene's cells are
 * shifted by a per-scene offset in the hashed grid, so overlapping scenes do not crowd the same
 * cells; each body tests only its own scene's static bodies.  Call between registration and
 * b3g_write_all_to_gpu; num_scenes <= 1 restores the single-scene world.  Offsets must start at 0
 * and be non-decreasing (empty scenes are allowed). */
#define B3G_MAX_SCENES (1 << 20)
b3gStatus b3g_set_scene_offsets(b3g_handle h, const int* first_body, int num_scenes);

/* Broadphase algorithm for the dynamic bodies (b3GpuBroadphaseInterface implementations,
 * Bullet3OpenCL/BroadphaseCollision/).  GRID: the uniform hashed grid of b3GpuGridBroadphase
 * (complete while every dynamic AABB fits one grid cell).  LBVH: the linear BVH of
 * b3GpuParallelLinearBvhBroadphase (b3GpuParallelLinearBvh.cpp:108-359): Morton codes of the AABB
 * centres, a binary radix tree, one traversal per body; complete for any AABB sizes.  Both emit the
 * same canonical pair list (static bodies go through the same sweep and prune / unbounded list
 * either way).  Valid before or after the upload; takes effect at the next pair search. */
#define B3G_BROADPHASE_GRID 0
#define B3G_BROADPHASE_LBVH 1
#define B3G_BROADPHASE_AUTO 2 /* the grid until b3g_autotune times both and keeps the faster */
b3gStatus b3g_set_broadphase(b3g_handle h, int mode);

/* Autotuner (no reference counterpart: the reference's OpenCL kernels use fixed work-group
 * sizes).  Times candidate launch shapes on the world's current state and keeps the fastest of
 * each: the radix sort's block count and the pair kernel's grid (pair stage), the thread-per-pair
 * narrowphase kernel's grid (contact stage) and, for PGS with pgs_partitions = AUTO, the solver's
 * work split (NONE / SHARED / GLOBAL_DELTAS / STREAMED; solve stage).  Each candidate runs the
 * stages `repeats` + 1 times from the same saved body state (the first run is not kept; the
 * median is); the bodies are put back afterwards, so the simulation state is unchanged.  Launch
 * shapes never change results except the PGS split, whose orders are all legal Gauss-Seidel
 * orders.  Allocates and frees one body-sized scratch buffer; synchronises the stream. */
typedef struct b3gTuning {
    int pgs_partitions;        /* chosen B3G_PGS_PARTITIONS_* (-1: not tuned, the AUTO rule applies) */
    int pairs_blocks_per_sm;   /* pair kernel blocks per SM (256 threads each) */
    int narrow_blocks_per_sm;  /* thread-per-pair narrowphase blocks per SM */
    int sort_blocks_per_sm;    /* radix sort blocks per SM */
    float pairs_ms;            /* median stage times with the chosen shapes */
    float contacts_ms;
    float solve_ms;
    int candidates_timed;
    int broadphase;            /* the pair search in use: B3G_BROADPHASE_GRID or _LBVH (AUTO: the faster) */
} b3gTuning;
b3gStatus b3g_autotune(b3g_handle h, float dt, int repeats, b3gTuning* out);
b3gStatus b3g_get_tuning(b3g_handle h, b3gTuning* out);
/* Marks the start (on = 1) and end (0) of the region an external profiler started with profiling
 * off should capture (cudaProfilerStart / cudaProfilerStop; no reference counterpart). */
b3gStatus b3g_profiler_range(int on);

/* ------------------------------------------------------------------ joints */
/* b3GpuRigidBodyPipeline::createPoint2PointConstraint / createFixedConstraint / removeConstraintByUid
 * (b3GpuRigidBodyPipeline.cpp:159-219).  Joints are solved every step right before the contacts,
 * as b3GpuPgsConstraintSolver::solveJoints does (b3GpuPgsConstraintSolver.cpp:927-944: PGS, 4
 * iterations, dt 1/60, erp 0.2, damping 1, batches from a greedy colouring of the joints): rows
 * from getInfo2Point2Point / getInfo2FixedOrientation (kernels/jointSolver.cl:488-630), a joint
 * whose row impulse reaches its breaking threshold is disabled for good.  Joints may be created
 * and removed before or after the upload; *out_uid is the joint's id. */
#define B3G_JOINT_POINT2POINT 3
#define B3G_JOINT_FIXED 4
b3gStatus b3g_create_point2point_constraint(b3g_handle h, int body_a, int body_b, const float pivot_in_a[3],
                                            const float pivot_in_b[3], float breaking_threshold, int* out_uid);
b3gStatus b3g_create_fixed_constraint(b3g_handle h, int body_a, int body_b, const float pivot_in_a[3],
                                      const float pivot_in_b[3], const float rel_target_ab[4],
                                      float breaking_threshold, int* out_uid);
b3gStatus b3g_remove_constraint(b3g_handle h, int uid);
b3gStatus b3g_get_num_constraints(b3g_handle h, int* n);
/* the joints (b3gJoint == b3GpuGenericConstraint, flags as the device last left them) and the
 * order the solver sweeps them in: joint indices batch by batch, batch_offsets[num_batches + 1]
 * (the order of the last joint solve: B3G_ERR_INVALID_ARG while a change to the joint list has
 * not been solved yet; order or batch_offsets may be NULL to query sizes) */
b3gStatus b3g_read_constraints(b3g_handle h, void* host_joints, int capacity, int* n);
b3gStatus b3g_read_joint_order(b3g_handle h, int* order, int capacity, int* batch_offsets, int offsets_capacity,
                               int* num_batches);

/* ------------------------------------------------------------------ ray casts */
/* b3GpuRigidBodyPipeline::castRays (b3GpuRigidBodyPipeline.cpp) -> b3GpuRaycast::castRays
 * (Bullet3OpenCL/Raycast/b3GpuRaycast.cpp:248-373): n rays (b3gRayInfo == b3RayInfo) from host
 * memory against the bodies' current poses; hits (b3gRayHit == b3RayHit) in/out: on input
 * hitResult2 names a body the ray ignores (-1: none); on output hitFraction is 1 when nothing is
 * hit, else the closest hit's fraction along from->to, hitBody, hitPoint and the normalised
 * hitNormal (a hull's face normal in the body's own frame, as the reference's kernel returns it;
 * a sphere's from its centre).  Hulls and spheres are hit, planes are not (as in the reference);
 * equal fractions go to the lower body index.  In a world of several scenes a ray sees only the
 * scene (int)from.w.  Rebuilds the broadphase grid from the current poses; synchronises. */
b3gStatus b3g_cast_rays(b3g_handle h, const void* host_rays, void* host_hits, int n);
/* The same cast on device buffers (b3gRayInfo / b3gRayHit arrays already on the world's device;
 * the work b3GpuRaycast::castRays does after its uploads, b3GpuRaycast.cpp:282-366): enqueued on
 * the world's stream, returns without synchronising. */
b3gStatus b3g_cast_rays_device(b3g_handle h, const void* device_rays, void* device_hits, int n);

/* ------------------------------------------------------------------ parallel primitives */
/* The reference's ParallelPrimitives classes (src/Bullet3OpenCL/ParallelPrimitives/), on caller
 * device buffers.  Each call allocates its own scratch, runs on the device's default stream and
 * synchronises before returning. */
/* b3RadixSort32CL::execute(keyValuesInOut, sortBits) (b3RadixSort32CL.cpp:174): stable LSD sort of
 * n (key, value) pairs of uint32 (b3SortData), in place, by key bits [0, sort_bits) exactly (the
 * reference rounds sort_bits up to its pass width; the two agree for multiples of 8). */
b3gStatus b3g_radix_sort32(int cuda_device, void* d_key_values, int n, int sort_bits);
/* b3RadixSort32CL::execute(keysInOut, sortBits): the same for keys alone. */
b3gStatus b3g_radix_sort32_keys(int cuda_device, void* d_keys, int n, int sort_bits);
/* b3PrefixScanCL::execute(src, dst, n, &sum): EXCLUSIVE scan of n uint32 (src may equal dst);
 * *host_sum = the total. */
b3gStatus b3g_prefix_scan32(int cuda_device, const void* d_src, void* d_dst, int n, unsigned int* host_sum);
/* b3BoundSearchCL::execute(src, nSrc, dst, nDst, option) (b3BoundSearchCL.cpp:69): src is n
 * (key, value) int pairs sorted by key; for every key k in [0, n_dst) present in src, LOWER writes
 * dst[k] = its first index, UPPER one past its last; buckets without elements are left as they
 * are; COUNT writes upper - lower for every bucket (0 where absent). */
#define B3G_BOUND_LOWER 0
#define B3G_BOUND_UPPER 1
#define B3G_BOUND_COUNT 2
b3gStatus b3g_bound_search(int cuda_device, const void* d_sorted_pairs, int n, void* d_dst, int n_dst, int option);
/* b3FillCL::execute(src, value, n, offset): d_dst[offset + i] = value for i in [0, n). */
b3gStatus b3g_fill32(int cuda_device, void* d_dst, int value, int n, int offset);

/* ------------------------------------------------------------------ the step */
/* b3GpuRigidBodyPipeline::stepSimulation (b3GpuRigidBodyPipeline.cpp:221-463): AABBs, pairs,
 * contacts, batching, solve, integrate -- enqueued on the world's stream (one CUDA graph
 * launch when use_cuda_graph is set); returns without synchronising. */
b3gStatus b3g_step(b3g_handle h, float dt);
/* Individual stages, same order as stepSimulation. */
b3gStatus b3g_setup_aabbs(b3g_handle h);                     /* setupGpuAabbsFull :500-575 */
b3gStatus b3g_calculate_overlapping_pairs(b3g_handle h);     /* b3GpuGridBroadphase::calculateOverlappingPairs :117-259 */
b3gStatus b3g_compute_contacts(b3g_handle h);                /* b3GpuNarrowPhase::computeContacts :751-809 */
/* b3GpuNarrowPhase::computeContacts(pairs, numPairs, aabbs, numObjects) (b3GpuNarrowPhase.cpp:751)
 * on the caller's pairs: d_pairs holds n b3gPair (b3Int4: x, y = body indices) in device memory on
 * the world's device.  The pairs replace the world's pair list (kept in the canonical (min, max)
 * order, so the manifolds come out in that order); pairs naming a body outside [0, bodies) or a
 * body twice are dropped and flag B3G_FLAG_PAIR_OVERFLOW.  Asynchronous on the world's stream. */
b3gStatus b3g_compute_contacts_for_pairs(b3g_handle h, const void* d_pairs, int n);
b3gStatus b3g_solve_joints(b3g_handle h);                    /* b3GpuPgsConstraintSolver::solveJoints :927-944 */
b3gStatus b3g_solve_contacts(b3g_handle h, float dt);        /* b3GpuPgsContactSolver::solveContacts :568-1103 */
b3gStatus b3g_integrate(b3g_handle h, float dt);             /* b3GpuRigidBodyPipeline::integrate :465-498 */
/* Waits for the world's stream. */
b3gStatus b3g_synchronize(b3g_handle h);
/* Reads the per-step counters (synchronises). */
b3gStatus b3g_get_stats(b3g_handle h, b3gStepStats* out);
/* Device status word (B3G_FLAG_*), synchronises; clear=1 resets it. */
b3gStatus b3g_status(b3g_handle h, unsigned int* flags, int clear);

/* ------------------------------------------------------------------ getters (borrowed device pointers) */
b3gStatus b3g_get_num_bodies(b3g_handle h, int* n);                       /* getNumBodies */
b3gStatus b3g_get_body_buffer(b3g_handle h, void** dptr);                 /* getBodyBuffer :65 -> b3RigidBodyData* */
b3gStatus b3g_get_inertia_buffer(b3g_handle h, void** dptr);              /* b3GpuNarrowPhase::getBodyInertiasGpu */
b3gStatus b3g_get_aabb_buffer(b3g_handle h, void** dptr);                 /* b3GpuBroadphaseInterface::getAabbBufferWS */
b3gStatus b3g_get_pair_buffer(b3g_handle h, void** dptr, int* num_pairs); /* getOverlappingPairBuffer + getNumOverlap (syncs) */
b3gStatus b3g_get_contact_buffer(b3g_handle h, void** dptr, int* num);    /* b3GpuNarrowPhase::getContactsGpu + getNumContactsGpu (syncs) */
b3gStatus b3g_get_stream(b3g_handle h, void** cuda_stream);

/* ------------------------------------------------------------------ host copies */
b3gStatus b3g_read_bodies(b3g_handle h, void* host_bodies, int n);        /* readbackAllBodiesToCpu */
b3gStatus b3g_write_bodies(b3g_handle h, const void* host_bodies, int n); /* setObjectTransform/VelocityCpu + write */
b3gStatus b3g_read_inertias(b3g_handle h, void* host_inertias, int n);
b3gStatus b3g_read_aabbs(b3g_handle h, void* host_aabbs, int n);
b3gStatus b3g_write_aabbs(b3g_handle h, const void* host_aabbs, int n);   /* feeds the broadphase identical AABBs */
b3gStatus b3g_read_pairs(b3g_handle h, void* host_pairs, int capacity, int* num_pairs);
b3gStatus b3g_read_contacts(b3g_handle h, void* host_contacts, int capacity, int* num_contacts);
/* Writes contacts for the solver stage (used to solve identical manifolds in parity tests). */
b3gStatus b3g_write_contacts(b3g_handle h, const void* host_contacts, int num_contacts);
/* Reads the colour (batch) of every manifold after the solver stage (PGS). */
b3gStatus b3g_read_batches(b3g_handle h, int* host_batch, int capacity, int* num);
/* Reads the PGS solve order of the last solver stage: manifold indices in an order whose
 * sequential Gauss-Seidel sweep gives the GPU's results bit for bit (manifolds the GPU solves
 * concurrently share no dynamic body).  Colour-overflow leftovers come last, in manifold order.
 * No counterpart in the reference (its order is the manifold order). */
b3gStatus b3g_read_solve_order(b3g_handle h, int* host_order, int capacity, int* num);
/* Reads per-point solver impulses (normal, lateral1, lateral2) after the solve: 3 floats per
 * point, 4 point slots per manifold. */
b3gStatus b3g_read_impulses(b3g_handle h, float* host, int capacity_manifolds, int* num);

/* Host-side reads of the shape tables (for checks). */
b3gStatus b3g_get_num_collidables(b3g_handle h, int* n);
/* Host registry copies of the registered bodies and inertias (as registered, before upload;
 * b3GpuNarrowPhase::m_bodyBufferCPU / m_inertiaBufferCPU).  No GPU needed. */
b3gStatus b3g_read_registered_bodies(b3g_handle h, void* bodies, void* inertias, int n);
b3gStatus b3g_read_shape_tables(b3g_handle h, void* collidables, void* hulls, void* faces, int* indices,
                                void* vertices, void* edges, void* local_aabbs, int* counts6);

/* ------------------------------------------------------------------ stage profiling */
/* Records CUDA events around each stage on the world's stream when on=1. */
b3gStatus b3g_set_profiling(b3g_handle h, int on);
/* Milliseconds per stage of the last profiled step (7 floats): aabb, pairs, contacts, joints
 * (the reference's batching slot: contact batching is fused into the solver), the contact solver
 * (row setup, colouring and sweeps), 0 (the solver is one stage), integrate. */
b3gStatus b3g_get_stage_times(b3g_handle h, float* ms7);
/* Number of kernels this library launched since creation (counted on the host at launch). */
b3gStatus b3g_get_launch_count(b3g_handle h, long long* n);
/* Records timing event `slot` (0..15) on the world's stream; b3g_event_elapsed returns the
 * milliseconds between two recorded slots (synchronising on the later one). */
b3gStatus b3g_record_event(b3g_handle h, int slot);
b3gStatus b3g_event_elapsed(b3g_handle h, int slot_start, int slot_end, float* ms);

/* ------------------------------------------------------------------ convex hull (host only, no GPU) */
/* b3ConvexUtility::initializePolyhedralFeatures (Bullet3Collision/NarrowPhaseCollision/b3ConvexUtility.cpp:26-246)
 * as called from registerConvexHullShape.  Output capacities are given in counts6 on entry
 * (vertices, faces, indices, edges, -, -) and replaced by the sizes written on return.
 * verts_out: xyz per vertex; planes_out: 4 floats per face; face_counts_out: indices per face;
 * indices_out: flat; edges_out: xyz per unique edge; center_out: vertex mean. */
b3gStatus b3g_hull_compute(const float* verts, int stride_bytes, int num_verts, const float scaling[3],
                           float* verts_out, float* planes_out, int* face_counts_out, int* indices_out,
                           float* edges_out, float* center_out, int* counts6);

/* ---- learned warm start (no counterpart in the reference) --------------------------------------
 * A 12 -> 128 -> 128 -> 128 -> 3 GELU network predicting, per contact point, the converged
 * impulses of its contact row and its two friction rows (second direction first) from 12 local
 * features: relative velocity of A w.r.t. B at the point (3), normal (3), separation (1),
 * inverse masses of A and B (2), points in the manifold (1), |tangential relative velocity| (1),
 * dt * (gravity . normal) (1).  BF16 tensor-core forward and backward passes with FP32
 * accumulation, Adam on FP32 master weights, all on the GPU.
 * Parameter layout (B3G_MLP_PARAMS floats): W1[12][128] b1[128] W2[128][128] b2[128] W3[128][128]
 * b3[128] W4[128][3] b4[3], W[in][out] row-major.  Normalisation (B3G_MLP_NORM floats): feature
 * mean[12], feature 1/std[12], target mean[3], target 1/std[3]; the network works in normalised
 * units and predictions are returned in impulse units.  Errors: b3g_last_error. */
#define B3G_MLP_PARAMS 35075
#define B3G_MLP_NORM 30
typedef struct b3gMlpImpl* b3g_mlp;
b3gStatus b3g_mlp_create(int cuda_device, unsigned long long seed, b3g_mlp* out);
b3gStatus b3g_mlp_destroy(b3g_mlp m);
b3gStatus b3g_mlp_set_params(b3g_mlp m, const float* params, int n);
b3gStatus b3g_mlp_get_params(b3g_mlp m, float* params, int n);
b3gStatus b3g_mlp_set_normalization(b3g_mlp m, const float* norm, int n);
b3gStatus b3g_mlp_get_normalization(b3g_mlp m, float* norm, int n);
/* n rows of 12 features (host) -> n rows of 3 predicted impulses (host) */
b3gStatus b3g_mlp_predict(b3g_mlp m, const float* features, int n, float* impulses);
/* uploads a training set (n x 12 features, n x 3 target impulses, host) */
b3gStatus b3g_mlp_set_training_data(b3g_mlp m, const float* features, const float* targets, int n);
/* `steps` Adam steps on consecutive batches of the training set starting at batch `first_batch`
 * (wrapping); mean_loss = mean over the steps of the batch mean-squared error (normalised units) */
b3gStatus b3g_mlp_train(b3g_mlp m, int steps, int batch, float lr, int first_batch, double* mean_loss);
/* gradients of the mean-squared error of one batch w.r.t. every parameter (B3G_MLP_PARAMS floats,
 * public layout), without an update: the gradient check of the backward kernels */
b3gStatus b3g_mlp_gradients(b3g_mlp m, const float* features, const float* targets, int n, float* grads,
                            double* loss);

/* Attaches a warm-start network to a world (same device; not owned; NULL detaches), used by
 * B3G_WARM_LEARNED and B3G_WARM_PERSISTENT_LEARNED. */
b3gStatus b3g_set_warm_start_model(b3g_handle h, b3g_mlp m);
/* Training samples of the last solve (warm_start LEARNED, RECORD or PERSISTENT_LEARNED): for every
 * active contact point with features, its 12 features, its 3 converged impulses (contact, second
 * friction direction, first friction direction) and (is_new, optional) whether it had no
 * persisting predecessor.  *num = samples available; at most `capacity` are written. */
b3gStatus b3g_read_warm_samples(b3g_handle h, float* features, float* targets, int* is_new, int capacity,
                                int* num);
/* The initial impulses of the last solve, 12 floats per manifold in the b3g_read_impulses layout
 * (per point: normal, lateral 1, lateral 2); zero for a cold start. */
b3gStatus b3g_read_warm_start(b3g_handle h, float* host, int capacity_manifolds, int* num);

/* ---- device buffers of the C++ layer's b3OpenCLArray ----------------------------------------------
 * The reference's b3OpenCLArray (Bullet3OpenCL/ParallelPrimitives/b3OpenCLArray.h:39-300) wraps
 * clCreateBuffer / clEnqueueWriteBuffer / clEnqueueReadBuffer / clEnqueueCopyBuffer; these three
 * calls are what its CUDA look-alike in include/b3g_compat.h uses, so that header needs no CUDA
 * headers.  Copies are synchronous; kind: B3G_COPY_H2D, B3G_COPY_D2H or B3G_COPY_D2D. */
#define B3G_COPY_H2D 0
#define B3G_COPY_D2H 1
#define B3G_COPY_D2D 2
b3gStatus b3g_buffer_alloc(int cuda_device, size_t bytes, void** out);
b3gStatus b3g_buffer_free(int cuda_device, void* p);
b3gStatus b3g_buffer_copy(int cuda_device, void* dst, const void* src, size_t bytes, int kind);

/* ---- allocation-free grid broadphase (no counterpart in the reference) -------------------------
 * The uniform-grid pair search of b3g_calculate_overlapping_pairs, run on the current CUDA device
 * over caller-owned device buffers, with all scratch in one fixed, statically sized device array
 * (about 7.4 MB) instead of memory from cudaMalloc.  For callers that must not allocate: code
 * running inside a frame or real-time loop with a fixed memory budget, or a host that owns every
 * device allocation itself.
 *   d_aabbs      n world AABBs (b3gAabb, 32 B each, 16-byte aligned device memory); only the
 *                min/max xyz are read.  Every AABB is a small proxy: no static-body list.
 *   n            0 .. B3G_NOALLOC_MAX_AABBS
 *   cell_size    > 0 and >= the largest AABB extent on any axis (the 27-cell search is then exact)
 *   grid_dim     power of two, 4 .. B3G_NOALLOC_MAX_GRID_DIM cells per axis (coordinates wrap)
 *   d_pairs      max_pairs b3gPair slots (device): (a, b, -1, -1), a < b, sorted by (a, b)
 *   max_pairs    1 .. B3G_NOALLOC_MAX_PAIRS
 *   d_num_pairs  one device int: the number of overlapping pairs found; when it exceeds
 *                max_pairs, max_pairs of them (an unspecified subset) are written, sorted
 *   cuda_stream  cudaStream_t the work is enqueued on (0 = legacy default stream); the call
 *                returns without waiting for it.
 * Larger sizes are rejected with B3G_ERR_CAPACITY before anything is enqueued.  The first call
 * on a device looks up the scratch array's address (cudaGetSymbolAddress) and the SM count: make
 * it before any stream capture.  Both are cached per device index for the life of the process; a
 * cudaDeviceReset (or any other teardown of the device's primary context) leaves the cached
 * address stale, so do not call this entry point on a device after resetting it.  No scratch content has to start at zero: each call resets the
 * counters it uses in its first kernel and validates the never-cleared cell table on use.  All
 * calls on one device share the one scratch array, so calls whose work overlaps in time (two
 * streams, or two host threads) race: serialise them on one stream or with events. */
#define B3G_NOALLOC_MAX_AABBS 65536
#define B3G_NOALLOC_MAX_PAIRS 262144
#define B3G_NOALLOC_MAX_GRID_DIM 64
b3gStatus b3g_grid_pairs_noalloc(const void* d_aabbs, int n, float cell_size, int grid_dim, void* d_pairs,
                                 int max_pairs, int* d_num_pairs, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif
