// Internal state shared by the host orchestration (world.cu) and the stage launchers.
#ifndef B3G_WORLD_INTERNAL_H
#define B3G_WORLD_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "b3g_capi.h"
#include "b3g_types.h"
#include "primitives.h"

namespace b3g {

namespace mlp {
struct Model;
}

// hull-hull pairs whose faces all have at most this many vertices take the thread-per-pair path
#define B3G_SMALL_FACE_VERTS 8
// ... and whose pair has at most this many SAT axes (faces of both + edge pairs); pairs with more
// take the warp-per-pair path, whose lanes split the axes
#define B3G_SMALL_PAIR_AXES 64

enum PairType { PT_HULL_HULL = 0, PT_PLANE_HULL = 1, PT_SPHERE_HULL = 2, PT_SPHERE_SPHERE = 3, PT_PLANE_SPHERE = 4,
                PT_HULL_HULL_SMALL = 5, PT_COUNT = 6 };

// Per-step device counters (one 256-byte block, copied to the host once per step).
struct DevCounters {
    int num_pairs;        // pairs emitted (may exceed capacity -> overflow flag)
    int num_contacts;     // manifolds
    int num_points;
    int num_colors;
    int iterations;
    float residual;
    unsigned int status;
    int type_count[PT_COUNT];
    int new_manifolds;    // PGS: manifolds without a colour carried over from the last solve
    int pad[64 - 8 - PT_COUNT];
};

// Compact solver records.  A b3SolverConstraint row (Bullet3Dynamics/ConstraintSolver/
// b3SolverConstraint.h) is rebuilt on the fly from these: relpos x axis and the inverse-inertia
// products are recomputed with the same operations the setup used, so the iterations see the
// same values as precomputed rows while reading 88 B per contact point instead of 240 B.
struct SolverPoints {
    float4* nf = nullptr;    // [m]      contact normal xyz, w = friction coefficient
    float4* rel1 = nullptr;  // [4m+j]   rel_pos1 xyz, w = jacDiagABInv of the contact row
    float4* rel2 = nullptr;  // [4m+j]   rel_pos2 xyz, w = rhs of the contact row
    float4* dir2 = nullptr;  // [4m+j]   second friction direction xyz, w = its jacDiagABInv
    float4* dir1 = nullptr;  // [4m+j]   first friction direction xyz, w = its jacDiagABInv
    float2* rhsf = nullptr;  // [4m+j]   rhs of the dir2 row, rhs of the dir1 row
    float4* imp = nullptr;   // [4m+j]   applied impulses: contact, dir2, dir1, (unused)
    // colour-ordered records only: the rows' angular components (inverse inertia x relpos x axis),
    // precomputed by the setup with the sweep's own operations: contact row A / B, dir2 row A / B,
    // dir1 row A / B packed as (cA.xyz, 2A.x) (cB.xyz, 2A.y) (2A.z, 2B.xyz) (1A.xyz, 1B.x) (1B.yz)
    float4* angP = nullptr;  // [4m+j]
    float4* angQ = nullptr;
    float4* angR = nullptr;
    float4* angS = nullptr;
    float2* angT = nullptr;
};

// Joint solver records.  A row of b3SolverConstraint (jointSolver.cl:129-160) is rebuilt from
// them with the same values: a ball joint's rows have the unit axes as linear Jacobian and the
// skew rows of -a1 and a2 (the rotated pivots) as angular Jacobians; a fixed joint's angular rows
// have +-unit axes.  So the joint keeps -a1 and a2 once and a row keeps only what differs.
struct JointHdr {      // 64 B per joint
    float4 m1_lo;      // -a1 xyz, w = lower limit of every row
    float4 a2_hi;      // a2 xyz, w = upper limit
    int A, B;          // bodies
    int active_rows;   // rows to sweep: 3 / 6, 0 when the joint is disabled
    float imA, imB;    // inverse masses at setup
    int pad[3];
};
struct JointRow {      // 32 B per row (+ 4 B applied impulse in its own array)
    float4 angA_rhs;   // angular component A xyz, w = rhs
    float4 angB_jinv;  // angular component B xyz, w = jacDiagABInv
};

// Launch shapes chosen by the autotuner (b3g_autotune); the defaults are the untuned shapes.
struct LaunchTuning {
    int pgs_partitions = -1;        // B3G_PGS_PARTITIONS_* used when the config says AUTO (-1: rule)
    int pairs_blocks_per_sm = 8;    // k_find_pairs grid = SMs x this (bodies per thread)
    int narrow_blocks_per_sm = 8;   // k_hull_hull_small grid = SMs x this (pairs per thread)
    int sort_blocks_per_sm = 4;     // radix sort: blocks (one contiguous chunk each) = SMs x this
};
static constexpr int B3G_MAX_SORT_BLOCKS_PER_SM = 8;
// finite static proxies sorted per scene in shared memory; a scene with more is scanned whole
static constexpr int B3G_SAP_MAX_PER_SCENE = 4096;

struct DeviceState {
    LaunchTuning tune;
    float4* ray_buf = nullptr;    // b3g_cast_rays: rays (2 float4 each) and hits, grown on demand
    b3gRayHit* hit_buf = nullptr;
    int ray_cap = 0;              // capacity of ray_order (rays per call)
    int ray_host_cap = 0;         // capacity of ray_buf / hit_buf (host-buffer calls only)
    uint32_t* ray_order = nullptr;  // 4 * ray_cap: Morton keys and ray indices, ping-pong for the sort
    int* ray_n = nullptr;           // device copy of the ray count (sort length)
    // LBVH broadphase (b3gConfig.broadphase = B3G_BROADPHASE_LBVH; own allocations): the dynamic
    // bodies sorted by (scene, Morton code of the AABB centre), a binary radix tree over them
    int broadphase = 0;
    int scene_bits = 0;                    // bits of the scene index above the 30 Morton bits
    uint64_t* lbvh_keys[2] = {nullptr, nullptr};
    uint32_t* lbvh_vals[2] = {nullptr, nullptr};
    const uint64_t* lbvh_sorted_keys = nullptr;
    const uint32_t* lbvh_sorted_vals = nullptr;
    int2* lbvh_child = nullptr;            // internal node -> children (leaf l stored as ~l)
    int2* lbvh_range = nullptr;            // internal node -> first and last leaf below it
    int* lbvh_parent = nullptr;            // parents of the leaves [0, n), of the internal nodes [n, 2n)
    float4* lbvh_box = nullptr;            // internal node -> AABB min, max
    int* lbvh_flag = nullptr;              // bottom-up refit: children finished per internal node
    unsigned int* lbvh_bounds = nullptr;   // centre bounds, order-preserving encodings: min xyz, ~max xyz
    int lbvh_cap = 0;
    // joints (own allocations, grown on demand; the host registry is authoritative except for
    // the enabled flags, which the device's break check clears)
    b3gJoint* joints = nullptr;
    JointHdr* joint_hdr = nullptr;   // 1 per joint
    JointRow* joint_rows = nullptr;  // 6 per joint
    float* joint_imp = nullptr;      // 6 per joint: applied impulses
    int* joint_order = nullptr;      // joint indices batch by batch
    int* joint_batch_off = nullptr;  // num_joint_batches + 1
    int* joint_uniq = nullptr;       // the bodies joints name, once each
    float2* joint_mass = nullptr;    // batching scratch: both bodies' inverse masses per joint
    float4* joint_dv = nullptr;      // 2 per body
    int joint_cap = 0, joint_dv_bodies = 0;
    int num_joints = 0, num_joint_batches = 0, num_joint_uniq = 0, max_joint_batch = 0;
    // sizes fixed at upload
    int num_bodies = 0, num_dynamic = 0, num_large = 0, num_collidables = 0;
    int max_pairs = 0, max_contacts = 0;
    int num_sms = 0;
    // registries
    b3gBody* bodies = nullptr;
    b3gInertia* inertias = nullptr;
    b3gCollidable* collidables = nullptr;
    b3gAabb* local_aabbs = nullptr;
    b3gHull* hulls = nullptr;
    b3gFace* faces = nullptr;
    int* indices = nullptr;
    b3gFloat4* vertices = nullptr;
    b3gFloat4* edges = nullptr;
    int* dyn_slot = nullptr;      // body -> dynamic slot or -1
    uint32_t* hull_face_dup = nullptr;  // per hull: bit f set when face f's normal is exactly the negation of
                                        // an earlier face's (f < 32): its SAT axis repeats that face's
    int* col_small = nullptr;     // per collidable: 0, or for a hull whose faces all have <= B3G_SMALL_FACE_VERTS
                                  // vertices: 1 | faces << 1 | unique edges << 16
    int* large_list = nullptr;    // static bodies (large proxies), grouped by scene
    // independent scenes (b3g_set_scene_offsets); nullptr / 1 when the world is one scene
    int num_scenes = 1;
    int* body_scene = nullptr;    // per body: its scene
    int* large_off = nullptr;     // per scene: first entry in large_list (num_scenes + 1)
    // static bodies with finite AABBs: 1-axis sweep and prune instead of the brute-force list
    int num_sap = 0;
    int sap_axis = 0;             // axis of the sweep (largest spread of the proxies' centres)
    int* sap_list = nullptr;      // finite static bodies, grouped by scene
    int* sap_off = nullptr;       // per scene: first entry in sap_list (num_scenes + 1)
    int* sap_sorted = nullptr;    // per scene: the same bodies sorted by AABB min along the axis
    float* sap_min = nullptr;     // their AABB mins along the axis (sorted)
    float* sap_ext = nullptr;     // per scene: largest AABB extent along the axis (rounded up; inf: unsorted)
    // broadphase
    b3gAabb* aabbs = nullptr;
    uint32_t* cell_keys[2] = {nullptr, nullptr};
    uint32_t* cell_vals[2] = {nullptr, nullptr};
    uint32_t* cell_start = nullptr;   // dense per hash cell, validated on use (no per-step clear)
    int grid_dim = 128, grid_bits = 7;
    float inv_cell = 1.f;
    int body_bits = 1;                // bits needed for a body index
    uint64_t* pair_keys[2] = {nullptr, nullptr};
    b3gPair* pairs = nullptr;
    int* type_lists = nullptr;        // PT_COUNT * max_pairs
    // narrowphase
    b3gContact4* contact_slots = nullptr;  // one per pair slot, then one per compound child pair, then
                                           // one per concave triangle-convex pair
    int* contact_flag = nullptr;           // per slot: 1 if a manifold was produced
    int* contact_index = nullptr;          // per slot: exclusive scan of contact_flag
    int* manifold_pair = nullptr;          // manifold -> slot index (< pair count: a pair)
    // compounds (allocated when one is registered): child shapes, the per-pair child-pair counts
    // and their scan, the child pairs (bodyA, bodyB, child of A or -1, child of B or -1)
    b3gChildShape* children = nullptr;
    int num_children = 0;
    int max_child_pairs = 0;
    int* child_count = nullptr;
    int* child_offset = nullptr;
    int4* child_pairs = nullptr;
    // concave meshes (allocated when one is registered): their BVHs, the per-pair triangle-convex
    // pair counts and their scan, the triangle-convex pairs (mesh body, other body, triangle,
    // child of the other body or 0)
    b3gBvhInfo* bvh_infos = nullptr;
    b3gBvhNode* bvh_nodes = nullptr;
    int num_meshes = 0;
    int max_concave_pairs = 0;
    int* concave_count = nullptr;
    int* concave_offset = nullptr;
    int4* concave_pairs = nullptr;
    b3gContact4* contacts_compact = nullptr;  // filled on demand for the drop-in getter
    // solver
    SolverPoints sp;                       // compact contact-point records
    SolverPoints sp_ord;                   // PGS: the same records in colour order
    int4* manifold_hdr_ord = nullptr;
    float4* manifold_inv_mass_ord = nullptr;  // (invMass A, invMass B, 0, 0)
    float4* inertia_ord = nullptr;         // PGS: per ordered manifold, A's then B's inverse world inertia rows (6)
    const uint32_t* cell_sorted_bodies = nullptr;  // set by the broadphase: dynamic bodies in cell order
    const uint32_t* cell_sorted_keys = nullptr;    // ... and their cell hashes
    int* body_slot = nullptr;              // body -> position in cell order (PGS partitions)
    int* manifold_group = nullptr;         // PGS processing group of each manifold
    int* group_counts = nullptr;           // 3 x (num_sms * B3G_PGS_MAX_BLOCKS_PER_SM * 64 + 64 + 2)
    int* manifold_color = nullptr;
    int* color_order = nullptr;            // manifolds sorted by colour
    int* manifold_pos = nullptr;           // PGS: position of each manifold in colour order
    unsigned long long* prev_mkey = nullptr;  // PGS: last solve's manifold body-pair keys (ascending)
    int* prev_mcolor = nullptr;            // PGS: ... and their colours
    int* prev_mn = nullptr;                // PGS: [0] their number, [1] colours of the last fresh
                                           // colouring, [2] 1: colour the next solve from scratch,
                                           // [3] solves since the last fresh colouring
    int* color_offsets = nullptr;          // B3G_MAX_COLORS + 1
    unsigned long long* color_claim = nullptr;  // per body
    float4* dv = nullptr;                  // per body: lin xyz | ang xyz (2 float4)
    float4* dv_sum = nullptr;              // Jacobi: per body sum of split deltas (2 float4)
    int4* manifold_hdr = nullptr;          // bodyA, bodyB, active point mask, points
    float2* manifold_inv_mass = nullptr;
    int* body_manifold_count = nullptr;    // Jacobi split counts
    int* body_list_offsets = nullptr;
    int* body_list = nullptr;              // Jacobi: manifold*2+side grouped by body
    uint32_t* jac_keys[2] = {nullptr, nullptr};
    uint32_t* jac_vals[2] = {nullptr, nullptr};
    float4* split_dv = nullptr;            // Jacobi: 2 sides * 2 float4 per manifold
    double* residual_acc = nullptr;        // per iteration: sum d^2, sum l^2
    // learned warm start
    mlp::Model* ws_model = nullptr;        // attached network (not owned)
    float* ws_features = nullptr;          // 12 features per point slot 4m+j
    int ws_rows_cap = 0;                   // point slots with features
    int* ws_rows = nullptr;                // device: slots of the current step
    float4* ws_init = nullptr;             // initial impulses of the last solve (per slot)
    unsigned char* ws_new = nullptr;       // per slot: 1 = no persisting predecessor
    // the previous solve's manifolds (first ws_rows_cap / 4), for persisting contact points
    unsigned long long* prev_keys = nullptr;  // body-pair key (min << body_bits | max), ascending
    float4* prev_pts = nullptr;            // per slot: point on B (world), w = 1 if active
    float4* prev_imp = nullptr;            // per slot: converged impulses (contact, dir2, dir1)
    int* prev_n = nullptr;                 // device: manifolds stored
    // control
    DevCounters* counters = nullptr;
    unsigned int* barrier = nullptr;       // count, gen, abort
    void* sort_scratch = nullptr;
    void* scan_scratch = nullptr;
    int* d_num_dynamic = nullptr;          // device copy of num_dynamic (sort length)
    int* d_num_bodies = nullptr;           // device copy of num_bodies
    PrimConfig prim;
    cudaError_t launch_error = cudaSuccess;  // first failed launch not reported through cudaGetLastError
};

#define B3G_MAX_COLORS 256
// PGS partitioned solver: at most this many persistent blocks per SM (sizes group_counts), and
// this much dynamic shared memory per block (owned body deltas and inertias, streamed tiles)
#define B3G_PGS_MAX_BLOCKS_PER_SM 4
#define B3G_PGS_MAX_SMEM (220 * 1024)
// streamed PGS tiles: bytes per manifold of one tile buffer (header, inverse masses, normal,
// 4 points x (rel1, rel2, imp, dir2, dir1, rhsf)), and the per-block tile list capacity
#define B3G_PGS_TILE_BYTES 400
#define B3G_PGS_MAX_TILES 512

// stage launchers (each returns the number of kernels it launched)
int launch_aabbs(DeviceState& d, cudaStream_t s);
int launch_pairs(DeviceState& d, cudaStream_t s);
int launch_cells(DeviceState& d, cudaStream_t s);
int launch_cast_rays(DeviceState& d, const float4* rays, b3gRayHit* hits, int n, cudaStream_t s);
void launch_set_int(int* p, int v, cudaStream_t s);
long long launch_joints(DeviceState& d, const b3gConfig& cfg, cudaStream_t s);
long long launch_joint_masses(const DeviceState& d, int n, float2* out, cudaStream_t s);
int launch_contacts(DeviceState& d, float friction, cudaStream_t s);
int launch_compact_contacts(DeviceState& d, cudaStream_t s);
int launch_solver(DeviceState& d, const b3gConfig& cfg, float dt, cudaStream_t s);
int launch_pairs_external(DeviceState& d, const b3gPair* pairs, int n, cudaStream_t s);
cudaError_t solver_prepare();  // kernel attributes, once per device before the first solve

// sets the message b3g_last_error returns (this thread) and passes the status through
b3gStatus report_error(b3gStatus st, const char* msg);

// allocation-free grid broadphase (noalloc.cu): the radix sorts run with sms * 4 blocks, so the
// static scratch covers devices with up to B3G_NOALLOC_MAX_SORT_BLOCKS / 4 SMs
#define B3G_NOALLOC_MAX_SORT_BLOCKS 1024
size_t noalloc_scratch_bytes();
cudaError_t noalloc_scratch_address(void** out);
int launch_grid_pairs_noalloc(void* scratch, int num_sms, const b3gAabb* aabbs, int n, float inv_cell, int bits,
                              int body_bits, b3gPair* pairs, int max_pairs, int* num_out, cudaStream_t s);
int launch_integrate(DeviceState& d, const b3gConfig& cfg, float dt, cudaStream_t s);

}  // namespace b3g

#endif
