// Host orchestration and the C ABI (include/b3g_capi.h).
//
// Mirrors the reference's host classes on the hot path:
//   b3GpuNarrowPhase  shape/body registry + device tables (src/Bullet3OpenCL/RigidBody/b3GpuNarrowPhase.cpp)
//   b3GpuGridBroadphase                        (src/Bullet3OpenCL/BroadphaseCollision/b3GpuGridBroadphase.cpp)
//   b3GpuRigidBodyPipeline stepSimulation      (src/Bullet3OpenCL/RigidBody/b3GpuRigidBodyPipeline.cpp:221-463)
// The step enqueues every stage on one stream with no host synchronisation; device-side
// counts drive all kernels (fixed launch shapes), so the whole step can be captured once
// as a CUDA graph and replayed.
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "b3g_capi.h"
#include "common.cuh"
#include "hull.h"
#include "warmstart.h"
#include "world_internal.h"

using namespace b3g;

static thread_local std::string g_last_error;

static b3gStatus fail(b3gStatus st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

b3gStatus b3g::report_error(b3gStatus st, const char* msg) {
    g_last_error = msg ? msg : "";
    return st;
}

#define CUDA_TRY(expr)                                                                              \
    do {                                                                                            \
        cudaError_t _e = (expr);                                                                    \
        if (_e != cudaSuccess)                                                                      \
            return fail(B3G_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, \
                        __LINE__);                                                                  \
    } while (0)

struct StageEvents {
    cudaEvent_t ev[8];
    bool created = false;
};

struct b3gWorld {
    b3gConfig cfg;
    int device = 0;
    cudaStream_t stream = nullptr;
    // host registries
    std::vector<b3gCollidable> collidables;
    std::vector<b3gAabb> local_aabbs;
    std::vector<b3gHull> hulls;
    std::vector<b3gFace> faces;
    std::vector<int> indices;
    std::vector<b3gFloat4> vertices;
    std::vector<b3gFloat4> edges;
    std::vector<b3gChildShape> children;  // the compounds' children (collidable.shapeIndex = first)
    std::vector<b3gBvhInfo> bvh_infos;    // per concave mesh (collidable.numChildShapes = its index)
    std::vector<b3gBvhNode> bvh_nodes;
    std::vector<b3gBody> bodies;
    std::vector<b3gInertia> inertias;
    std::vector<int> user_index;
    std::vector<int> scene_first;  // first body of each independent scene (empty: one scene)
    bool uploaded = false;
    DeviceState d;
    std::vector<void*> allocations;
    // captured steps: [0] the plain step, [1] the same step with an event-record node between
    // stages (profiling), each rebuilt when the step's parameters change
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        float dt = -1.f;
        int mode = -1, iters = -1;
        float tol = -1.f;
        long long kernels = 0;
    } graphs[2];
    // profiling
    bool profiling = false;
    StageEvents events;
    float stage_ms[7] = {0, 0, 0, 0, 0, 0, 0};
    long long launches = 0;
    b3gStepStats last_stats{};
    cudaEvent_t user_events[16] = {};
    b3g_mlp ws_mlp = nullptr;  // attached warm-start network (not owned)
    bool tuned = false;        // b3g_autotune ran on the current upload
    b3gTuning tuning{};        // its last result
    // joints: the host registry; the device copy matches it (but for the enabled flags, which
    // the device's break check clears) while joints_dirty is false
    std::vector<b3gJoint> joints;
    int next_joint_uid = 0;
    bool joints_dirty = false;
    std::vector<int> joint_order, joint_batch_off;
};

static b3gStatus sync_joint_flags(b3gWorld* h);

static void free_lbvh_buffers(b3g::DeviceState& d) {
    for (auto* p : d.lbvh_keys) cudaFree(p);
    for (auto* p : d.lbvh_vals) cudaFree(p);
    cudaFree(d.lbvh_child);
    cudaFree(d.lbvh_range);
    cudaFree(d.lbvh_parent);
    cudaFree(d.lbvh_box);
    cudaFree(d.lbvh_flag);
    cudaFree(d.lbvh_bounds);
}

// LBVH buffers for the world's dynamic bodies (84 B per body), allocated on first use
static b3gStatus alloc_lbvh(b3g::DeviceState& d) {
    const int n = std::max(2, d.num_dynamic);
    if (d.lbvh_cap >= n) return B3G_OK;
    free_lbvh_buffers(d);
    d.lbvh_keys[0] = d.lbvh_keys[1] = nullptr;
    d.lbvh_vals[0] = d.lbvh_vals[1] = nullptr;
    d.lbvh_cap = 0;
    const size_t m = (size_t)n;
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_keys[0]), m * sizeof(uint64_t)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_keys[1]), m * sizeof(uint64_t)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_vals[0]), m * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_vals[1]), m * sizeof(uint32_t)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_child), m * sizeof(int2)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_range), m * sizeof(int2)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_parent), 2 * m * sizeof(int)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_box), 2 * m * sizeof(float4)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_flag), m * sizeof(int)));
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d.lbvh_bounds), 8 * sizeof(unsigned int)));
    d.lbvh_cap = n;
    return B3G_OK;
}

static void free_joint_buffers(b3g::DeviceState& d) {
    cudaFree(d.joints);
    cudaFree(d.joint_hdr);
    cudaFree(d.joint_rows);
    cudaFree(d.joint_imp);
    cudaFree(d.joint_order);
    cudaFree(d.joint_batch_off);
    cudaFree(d.joint_uniq);
    cudaFree(d.joint_mass);
    cudaFree(d.joint_dv);
}

// Drops the captured step graphs (the next step captures again).
static void drop_graphs(b3gWorld* w) {
    for (auto& g : w->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = b3gWorld::StepGraph();
    }
}

static void free_device(b3gWorld* w) {
    drop_graphs(w);
    for (void* p : w->allocations) cudaFree(p);
    w->allocations.clear();
    free_joint_buffers(w->d);
    free_lbvh_buffers(w->d);
    w->d = DeviceState();
    w->uploaded = false;
}

template <typename T>
static b3gStatus dalloc(b3gWorld* w, T** p, size_t count) {
    if (count == 0) count = 1;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e != cudaSuccess)
        return fail(B3G_ERR_CUDA, "cudaMalloc(%zu bytes) failed: %s", count * sizeof(T), cudaGetErrorString(e));
    w->allocations.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return B3G_OK;
}

#define TRY(expr)                         \
    do {                                  \
        b3gStatus _s = (expr);            \
        if (_s != B3G_OK) return _s;      \
    } while (0)

// ---------------------------------------------------------------------------------- config
extern "C" b3gStatus b3g_config_default(b3gConfig* c) {
    if (!c) return fail(B3G_ERR_INVALID_ARG, "null config");
    std::memset(c, 0, sizeof(*c));
    c->max_bodies = 128 * 1024;  // b3Config::m_maxConvexBodies
    c->max_shapes = 8 * 1024;
    c->max_pairs = 0;
    c->max_contacts = 0;
    c->grid_cell_size = 0.f;
    c->grid_dim = 128;
    c->gravity[0] = 0.f;
    c->gravity[1] = -9.8f;
    c->gravity[2] = 0.f;
    c->angular_damping = 0.99f;
    c->solver_mode = B3G_SOLVER_PGS;
    c->solver_iterations = 10;
    c->erp = 0.2f;
    c->contact_threshold = 0.02f;
    c->contact_friction = 0.7f;
    c->residual_tol = 0.f;
    c->update_world_inertia = 0;
    c->use_cuda_graph = 1;
    c->warm_start = 0;
    return B3G_OK;
}

extern "C" const char* b3g_last_error(void) { return g_last_error.c_str(); }
extern "C" const char* b3g_version(void) { return "b3g-gb300 0.1 (sm_103a)"; }

extern "C" b3gStatus b3g_create(const b3gConfig* cfg, int cuda_device, b3g_handle* out) {
    if (!out) return fail(B3G_ERR_INVALID_ARG, "null output handle");
    b3gWorld* w = new b3gWorld();
    if (cfg)
        w->cfg = *cfg;
    else
        b3g_config_default(&w->cfg);
    if (w->cfg.grid_dim < 4 || (w->cfg.grid_dim & (w->cfg.grid_dim - 1))) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "grid_dim must be a power of two >= 4");
    }
    if (w->cfg.grid_dim > 1024) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "grid_dim must be <= 1024 (hash fits in 30 bits)");
    }
    if (w->cfg.pgs_partitions < B3G_PGS_PARTITIONS_AUTO || w->cfg.pgs_partitions > B3G_PGS_PARTITIONS_STREAMED) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "pgs_partitions must be one of B3G_PGS_PARTITIONS_*");
    }
    if (w->cfg.warm_start < B3G_WARM_COLD || w->cfg.warm_start > B3G_WARM_PERSISTENT_LEARNED ||
        w->cfg.warm_start_max_points < 0) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "warm_start must be one of B3G_WARM_* and warm_start_max_points >= 0");
    }
    if (w->cfg.pgs_interleave != 0 && w->cfg.pgs_interleave != 1) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "pgs_interleave must be 0 or 1");
    }
    if (w->cfg.solver_blocks_per_sm < 0) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "solver_blocks_per_sm must be >= 0");
    }
    if (w->cfg.broadphase < B3G_BROADPHASE_GRID || w->cfg.broadphase > B3G_BROADPHASE_AUTO) {
        delete w;
        return fail(B3G_ERR_INVALID_ARG, "broadphase must be B3G_BROADPHASE_GRID, _LBVH or _AUTO");
    }
    w->device = cuda_device;
    *out = w;
    return B3G_OK;
}

extern "C" b3gStatus b3g_reset(b3g_handle h, int what) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (what & ~(B3G_RESET_SHAPES_AND_BODIES | B3G_RESET_CONSTRAINTS)) return fail(B3G_ERR_INVALID_ARG, "unknown reset flags");
    if (h->uploaded) {
        CUDA_TRY(cudaSetDevice(h->device));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    if (what & B3G_RESET_CONSTRAINTS) {
        h->joints.clear();
        h->joint_order.clear();
        h->joint_batch_off.clear();
        h->joints_dirty = true;
    }
    if (what & B3G_RESET_SHAPES_AND_BODIES) {
        free_device(h);  // the next upload allocates afresh
        h->collidables.clear();
        h->local_aabbs.clear();
        h->hulls.clear();
        h->faces.clear();
        h->indices.clear();
        h->vertices.clear();
        h->edges.clear();
        h->children.clear();
        h->bvh_infos.clear();
        h->bvh_nodes.clear();
        h->bodies.clear();
        h->inertias.clear();
        h->user_index.clear();
        h->scene_first.clear();
        h->tuned = false;
        h->tuning = b3gTuning{};
        h->last_stats = b3gStepStats{};
        h->joints_dirty = true;
    }
    return B3G_OK;
}

extern "C" b3gStatus b3g_destroy(b3g_handle h) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (h->uploaded) {
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream);
    }
    free_device(h);
    if (h->events.created)
        for (auto& e : h->events.ev) cudaEventDestroy(e);
    for (auto& e : h->user_events)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- shapes
static b3gStatus add_collidable(b3gWorld* w, const b3gCollidable& c, const b3gAabb& aabb, int* out) {
    if ((int)w->collidables.size() >= w->cfg.max_shapes)
        return fail(B3G_ERR_CAPACITY, "allocateCollidable out-of-range %d", w->cfg.max_shapes);
    w->collidables.push_back(c);
    w->local_aabbs.push_back(aabb);
    if (out) *out = (int)w->collidables.size() - 1;
    return B3G_OK;
}

static b3gAabb make_aabb(float x0, float y0, float z0, float x1, float y1, float z1) {
    b3gAabb a;
    a.minv[0] = x0; a.minv[1] = y0; a.minv[2] = z0; a.minw = 0;
    a.maxv[0] = x1; a.maxv[1] = y1; a.maxv[2] = z1; a.maxw = 0;
    return a;
}

extern "C" b3gStatus b3g_register_sphere(b3g_handle h, float radius, int* out) {
    if (!h || !out) return fail(B3G_ERR_INVALID_ARG, "null argument");
    if (!(radius > 0.f)) return fail(B3G_ERR_INVALID_ARG, "sphere radius must be positive");
    b3gCollidable c{0, radius, B3G_SHAPE_SPHERE, 0};
    return add_collidable(h, c, make_aabb(-radius, -radius, -radius, radius, radius, radius), out);
}

extern "C" b3gStatus b3g_register_plane(b3g_handle h, const float n[3], float constant, int* out) {
    if (!h || !n || !out) return fail(B3G_ERR_INVALID_ARG, "null argument");
    b3gFace f{};
    f.plane = b3gFloat4{n[0], n[1], n[2], constant};
    f.indexOffset = 0;
    f.numIndices = 0;
    int faceIndex = (int)h->faces.size();
    h->faces.push_back(f);
    b3gCollidable c{0, constant, B3G_SHAPE_PLANE, faceIndex};
    return add_collidable(h, c, make_aabb(-1e30f, -1e30f, -1e30f, 1e30f, 1e30f, 1e30f), out);
}

static b3gStatus add_hull(b3gWorld* w, const std::vector<float>& vxyz, const std::vector<float>& planes,
                          const std::vector<int>& counts, const std::vector<int>& idx, const std::vector<float>& exyz,
                          int* out) {
    const int nv = (int)vxyz.size() / 3;
    if (nv < 1) return fail(B3G_ERR_INVALID_ARG, "hull has no vertices");
    b3gHull hull{};
    // local centre = vertex mean (b3GpuNarrowPhase.cpp:324-329)
    float cx = 0, cy = 0, cz = 0;
    for (int i = 0; i < nv; i++) {
        cx = cx + vxyz[3 * i];
        cy = cy + vxyz[3 * i + 1];
        cz = cz + vxyz[3 * i + 2];
    }
    float inv = 1.f / (float)nv;
    hull.localCenter = b3gFloat4{cx * inv, cy * inv, cz * inv, 0.f};
    hull.numUniqueEdges = (int)exyz.size() / 3;
    hull.uniqueEdgesOffset = (int)w->edges.size();
    for (int i = 0; i < hull.numUniqueEdges; i++)
        w->edges.push_back(b3gFloat4{exyz[3 * i], exyz[3 * i + 1], exyz[3 * i + 2], 0.f});
    hull.faceOffset = (int)w->faces.size();
    hull.numFaces = (int)counts.size();
    int off = 0;
    for (int f = 0; f < hull.numFaces; f++) {
        b3gFace face{};
        face.plane = b3gFloat4{planes[4 * f], planes[4 * f + 1], planes[4 * f + 2], planes[4 * f + 3]};
        face.indexOffset = (int)w->indices.size();
        face.numIndices = counts[f];
        for (int k = 0; k < counts[f]; k++) {
            int vi = idx[off + k];
            if (vi < 0 || vi >= nv) return fail(B3G_ERR_INVALID_INDEX, "face index %d out of range", vi);
            w->indices.push_back(vi);
        }
        off += counts[f];
        w->faces.push_back(face);
    }
    hull.numVertices = nv;
    hull.vertexOffset = (int)w->vertices.size();
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < nv; i++) {
        w->vertices.push_back(b3gFloat4{vxyz[3 * i], vxyz[3 * i + 1], vxyz[3 * i + 2], 0.f});
        for (int k = 0; k < 3; k++) {
            mn[k] = std::min(mn[k], vxyz[3 * i + k]);
            mx[k] = std::max(mx[k], vxyz[3 * i + k]);
        }
    }
    int hullIndex = (int)w->hulls.size();
    w->hulls.push_back(hull);
    b3gCollidable c{0, 0.f, B3G_SHAPE_CONVEX_HULL, hullIndex};
    return add_collidable(w, c, make_aabb(mn[0], mn[1], mn[2], mx[0], mx[1], mx[2]), out);
}

extern "C" b3gStatus b3g_register_compound(b3g_handle h, const b3gChildShape* children, int num_children,
                                           int* out) {
    if (!h || !out) return fail(B3G_ERR_INVALID_ARG, "null argument");
    if (h->uploaded) return fail(B3G_ERR_INVALID_ARG, "register shapes before the upload");
    // the collidable slot is taken first, as allocateCollidable runs first (b3GpuNarrowPhase.cpp:372-374)
    if ((int)h->collidables.size() >= h->cfg.max_shapes)
        return fail(B3G_ERR_CAPACITY, "allocateCollidable out-of-range %d", h->cfg.max_shapes);
    if (!children || num_children < 1) return fail(B3G_ERR_INVALID_ARG, "a compound needs at least one child");
    // the union of the children's local AABBs moved into the compound's frame (b3GpuNarrowPhase.cpp:391-431)
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < num_children; i++) {
        const int c = children[i].shapeIndex;
        if (c < 0 || c >= (int)h->collidables.size() || h->collidables[c].shapeType != B3G_SHAPE_CONVEX_HULL)
            return fail(B3G_ERR_INVALID_INDEX, "compound child %d is not a convex hull collidable", i);
        v3 a, b;
        transform_aabb(h->local_aabbs[c], f4v3(children[i].childPosition), f4q(children[i].childOrientation), 0.f, a,
                       b);
        if (a.x < mn[0]) mn[0] = a.x;
        if (a.y < mn[1]) mn[1] = a.y;
        if (a.z < mn[2]) mn[2] = a.z;
        if (mx[0] < b.x) mx[0] = b.x;
        if (mx[1] < b.y) mx[1] = b.y;
        if (mx[2] < b.z) mx[2] = b.z;
    }
    b3gCollidable col{num_children, 0.f, B3G_SHAPE_COMPOUND, (int)h->children.size()};
    const b3gStatus st = add_collidable(h, col, make_aabb(mn[0], mn[1], mn[2], mx[0], mx[1], mx[2]), out);
    if (st != B3G_OK) return st;
    for (int i = 0; i < num_children; i++) {
        b3gChildShape c = children[i];
        c.childPosition.w = 0.f;
        c.numChildShapes = 0;
        c.collidableShapeIndex = 0;
        c.shapeType = B3G_SHAPE_CONVEX_HULL;
        h->children.push_back(c);
    }
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_child_shapes(b3g_handle h, b3gChildShape* host, int capacity, int* num) {
    if (!h || !num) return fail(B3G_ERR_INVALID_ARG, "null argument");
    *num = (int)h->children.size();
    if (host && capacity > 0)
        std::copy(h->children.begin(), h->children.begin() + std::min(capacity, *num), host);
    return B3G_OK;
}

// b3QuantizedBvh::quantize (b3QuantizedBvh.h:314-341) with the bounds of a mesh's BVH: min corners
// rounded down to even, max corners up to odd, so that dequantized boxes contain the originals
static void mesh_quantize(unsigned short out[3], const float p[3], bool isMax, const b3gBvhInfo& bi) {
    const float mn[3] = {bi.aabbMin.x, bi.aabbMin.y, bi.aabbMin.z};
    const float q[3] = {bi.quantization.x, bi.quantization.y, bi.quantization.z};
    for (int k = 0; k < 3; k++) {
        const float v = (p[k] - mn[k]) * q[k];
        out[k] = isMax ? (unsigned short)(((unsigned short)(v + 1.f)) | 1) : (unsigned short)(((unsigned short)v) & 0xfffe);
    }
}

// The triangle BVH of a concave mesh, built over the triangles in index order (each internal node
// halves its triangle range), so that a depth-first walk meets the overlapping triangles in index
// order; nodes in depth-first order, an internal node's box the union of its children's quantized
// boxes.  Returns the subtree's node count.
static int build_mesh_bvh(std::vector<b3gBvhNode>& nodes, const std::vector<b3gBvhNode>& leaves, int lo, int hi) {
    const size_t me = nodes.size();
    if (hi - lo == 1) {
        nodes.push_back(leaves[lo]);
        return 1;
    }
    nodes.push_back(b3gBvhNode{});
    const int mid = lo + (hi - lo) / 2;
    const int nl = build_mesh_bvh(nodes, leaves, lo, mid);
    const int nr = build_mesh_bvh(nodes, leaves, mid, hi);
    const b3gBvhNode L = nodes[me + 1], R = nodes[me + 1 + nl];
    b3gBvhNode& n = nodes[me];
    for (int k = 0; k < 3; k++) {
        n.quantizedAabbMin[k] = std::min(L.quantizedAabbMin[k], R.quantizedAabbMin[k]);
        n.quantizedAabbMax[k] = std::max(L.quantizedAabbMax[k], R.quantizedAabbMax[k]);
    }
    n.escapeIndexOrTriangleIndex = -(1 + nl + nr);
    return 1 + nl + nr;
}

extern "C" b3gStatus b3g_register_concave_mesh(b3g_handle h, const float* verts, int stride_bytes, int num_vertices,
                                               const int* tri, int num_triangles, const float scaling[3], int* out) {
    if (!h || !verts || !tri || !out) return fail(B3G_ERR_INVALID_ARG, "null argument");
    if (h->uploaded) return fail(B3G_ERR_INVALID_ARG, "register shapes before the upload");
    if ((int)h->collidables.size() >= h->cfg.max_shapes)
        return fail(B3G_ERR_CAPACITY, "allocateCollidable out-of-range %d", h->cfg.max_shapes);
    if (stride_bytes < 12) return fail(B3G_ERR_INVALID_ARG, "stride must be >= 12 bytes");
    if (num_vertices < 3 || num_triangles < 1) return fail(B3G_ERR_INVALID_ARG, "a mesh needs a triangle");
    for (int i = 0; i < 3 * num_triangles; i++)
        if (tri[i] < 0 || tri[i] >= num_vertices)
            return fail(B3G_ERR_INVALID_INDEX, "triangle index %d out of range", tri[i]);
    const float sx = scaling ? scaling[0] : 1.f, sy = scaling ? scaling[1] : 1.f, sz = scaling ? scaling[2] : 1.f;
    std::vector<v3> v(num_vertices);
    for (int i = 0; i < num_vertices; i++) {
        const float* p = reinterpret_cast<const float*>(reinterpret_cast<const char*>(verts) + (size_t)i * stride_bytes);
        v[i] = mk3(p[0] * sx, p[1] * sy, p[2] * sz);
    }
    // the shape record: the triangles as faces, the scaled vertices (b3GpuNarrowPhase.cpp:615-667)
    b3gHull hull{};
    hull.uniqueEdgesOffset = (int)h->edges.size();
    hull.faceOffset = (int)h->faces.size();
    hull.numFaces = num_triangles;
    for (int t = 0; t < num_triangles; t++) {
        const v3 v0 = v[tri[3 * t]], v1 = v[tri[3 * t + 1]], v2 = v[tri[3 * t + 2]];
        const v3 c = cross3(v1 - v0, v2 - v0);
        const float inv = 1.f / sqrtf(dot3(c, c));
        const v3 n = mk3(c.x * inv, c.y * inv, c.z * inv);
        b3gFace f{};
        f.plane = b3gFloat4{n.x, n.y, n.z, -dot3(n, v0)};
        f.indexOffset = (int)h->indices.size();
        f.numIndices = 3;
        for (int k = 0; k < 3; k++) h->indices.push_back(tri[3 * t + k]);
        h->faces.push_back(f);
    }
    hull.numVertices = num_vertices;
    hull.vertexOffset = (int)h->vertices.size();
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = 0; i < num_vertices; i++) {
        h->vertices.push_back(b3gFloat4{v[i].x, v[i].y, v[i].z, 0.f});
        const float p[3] = {v[i].x, v[i].y, v[i].z};
        for (int k = 0; k < 3; k++) {
            if (p[k] < mn[k]) mn[k] = p[k];
            if (mx[k] < p[k]) mx[k] = p[k];
        }
    }
    const int hullIndex = (int)h->hulls.size();
    h->hulls.push_back(hull);
    // the quantization (b3QuantizedBvh::setQuantizationValues, margin 1) and the leaves: each
    // triangle's AABB widened to at least 0.002 per axis (b3OptimizedBvh::build's quantized leaf
    // callback), from the scaled vertices
    b3gBvhInfo bi{};
    bi.aabbMin = b3gFloat4{mn[0] - 1.f, mn[1] - 1.f, mn[2] - 1.f, 0.f};
    bi.aabbMax = b3gFloat4{mx[0] + 1.f, mx[1] + 1.f, mx[2] + 1.f, 0.f};
    bi.quantization = b3gFloat4{65533.f / (bi.aabbMax.x - bi.aabbMin.x), 65533.f / (bi.aabbMax.y - bi.aabbMin.y),
                                65533.f / (bi.aabbMax.z - bi.aabbMin.z), 0.f};
    bi.nodeOffset = (int)h->bvh_nodes.size();
    bi.numTriangles = num_triangles;
    std::vector<b3gBvhNode> leaves(num_triangles);
    for (int t = 0; t < num_triangles; t++) {
        float lo[3] = {1e18f, 1e18f, 1e18f}, hi[3] = {-1e18f, -1e18f, -1e18f};
        for (int k = 0; k < 3; k++) {
            const v3 p = v[tri[3 * t + k]];
            const float c[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; a++) {
                if (c[a] < lo[a]) lo[a] = c[a];
                if (hi[a] < c[a]) hi[a] = c[a];
            }
        }
        for (int a = 0; a < 3; a++)
            if (hi[a] - lo[a] < 0.002f) {
                hi[a] = hi[a] + 0.001f;
                lo[a] = lo[a] - 0.001f;
            }
        mesh_quantize(leaves[t].quantizedAabbMin, lo, false, bi);
        mesh_quantize(leaves[t].quantizedAabbMax, hi, true, bi);
        leaves[t].escapeIndexOrTriangleIndex = t;
    }
    bi.numNodes = build_mesh_bvh(h->bvh_nodes, leaves, 0, num_triangles);
    const int bvhIndex = (int)h->bvh_infos.size();
    h->bvh_infos.push_back(bi);
    b3gCollidable col{bvhIndex, 0.f, B3G_SHAPE_CONCAVE_TRIMESH, hullIndex};
    return add_collidable(h, col, make_aabb(mn[0], mn[1], mn[2], mx[0], mx[1], mx[2]), out);
}

extern "C" b3gStatus b3g_read_mesh_bvh(b3g_handle h, b3gBvhInfo* infos, int capacity_infos, b3gBvhNode* nodes,
                                       int capacity_nodes, int* num_infos, int* num_nodes) {
    if (!h || !num_infos || !num_nodes) return fail(B3G_ERR_INVALID_ARG, "null argument");
    *num_infos = (int)h->bvh_infos.size();
    *num_nodes = (int)h->bvh_nodes.size();
    if (infos && capacity_infos > 0)
        std::copy(h->bvh_infos.begin(), h->bvh_infos.begin() + std::min(capacity_infos, *num_infos), infos);
    if (nodes && capacity_nodes > 0)
        std::copy(h->bvh_nodes.begin(), h->bvh_nodes.begin() + std::min(capacity_nodes, *num_nodes), nodes);
    return B3G_OK;
}

extern "C" b3gStatus b3g_register_hull(b3g_handle h, const float* verts, int stride_bytes, int num_verts,
                                       const float scaling[3], int* out) {
    if (!h || !verts || !out) return fail(B3G_ERR_INVALID_ARG, "null argument");
    if (stride_bytes < 12) return fail(B3G_ERR_INVALID_ARG, "stride must be >= 12 bytes");
    HullTables t;
    if (build_hull(verts, stride_bytes, num_verts, scaling, t) != 0)
        return fail(B3G_ERR_DEGENERATE, "degenerate convex hull input (%d points)", num_verts);
    return add_hull(h, t.vertices, t.planes, t.face_counts, t.indices, t.edges, out);
}

extern "C" b3gStatus b3g_register_hull_tables(b3g_handle h, const float* verts_xyz, int num_verts,
                                              const float* face_planes, const int* face_index_counts, int num_faces,
                                              const int* face_indices, const float* unique_edges_xyz, int num_edges,
                                              int* out) {
    if (!h || !verts_xyz || !face_planes || !face_index_counts || !out || num_verts < 1 || num_faces < 1)
        return fail(B3G_ERR_INVALID_ARG, "invalid hull tables");
    std::vector<float> v(verts_xyz, verts_xyz + 3 * num_verts);
    std::vector<float> p(face_planes, face_planes + 4 * num_faces);
    std::vector<int> c(face_index_counts, face_index_counts + num_faces);
    int total = 0;
    for (int x : c) total += x;
    std::vector<int> idx(face_indices, face_indices + total);
    std::vector<float> e;
    if (num_edges > 0) e.assign(unique_edges_xyz, unique_edges_xyz + 3 * num_edges);
    return add_hull(h, v, p, c, idx, e, out);
}

// ---------------------------------------------------------------------------------- bodies
static m33 host_qmat(const float q[4]) { return qmat(quat{q[0], q[1], q[2], q[3]}); }

extern "C" b3gStatus b3g_register_body(b3g_handle h, float mass, const float pos[3], const float orn[4],
                                       int collidable, int user_index, int* out) {
    if (!h || !pos || !orn || !out) return fail(B3G_ERR_INVALID_ARG, "null argument");
    if (collidable < 0 || collidable >= (int)h->collidables.size())
        return fail(B3G_ERR_INVALID_INDEX, "registerPhysicsInstance using invalid collidableIndex");
    if ((int)h->bodies.size() >= h->cfg.max_bodies)
        return fail(B3G_ERR_CAPACITY, "registerRigidBody: exceeding the number of rigid bodies, %d > %d",
                    (int)h->bodies.size(), h->cfg.max_bodies);
    if (h->uploaded) return fail(B3G_ERR_INVALID_ARG, "register bodies before b3g_write_all_to_gpu");
    // world AABB with margin 0.01 (b3TransformAabb, b3GpuRigidBodyPipeline.cpp:613-618)
    const b3gAabb& la = h->local_aabbs[collidable];
    const float margin = 0.01f;
    m33 R = host_qmat(orn);
    float he[3], c[3];
    for (int k = 0; k < 3; k++) {
        he[k] = 0.5f * (la.maxv[k] - la.minv[k]) + margin;
        c[k] = 0.5f * (la.maxv[k] + la.minv[k]);
    }
    v3 cw = mmul(R, mk3(c[0], c[1], c[2])) + mk3(pos[0], pos[1], pos[2]);
    v3 hv = mk3(he[0], he[1], he[2]);
    v3 ext = mk3(dot3(hv, mk3(fabsf(R.r0.x), fabsf(R.r0.y), fabsf(R.r0.z))),
                 dot3(hv, mk3(fabsf(R.r1.x), fabsf(R.r1.y), fabsf(R.r1.z))),
                 dot3(hv, mk3(fabsf(R.r2.x), fabsf(R.r2.y), fabsf(R.r2.z))));
    v3 amin = cw - ext, amax = cw + ext;

    b3gBody b{};
    b.pos = b3gFloat4{pos[0], pos[1], pos[2], 0.f};
    b.quat = b3gFloat4{orn[0], orn[1], orn[2], orn[3]};
    b.linVel = b3gFloat4{0, 0, 0, 0};
    b.angVel = b3gFloat4{0, 0, 0, 0};
    b.collidableIdx = collidable;
    b.invMass = mass != 0.f ? 1.f / mass : 0.f;
    b.restitution = 0.f;
    b.friction = 1.f;  // b3GpuNarrowPhase.cpp:835-839
    b3gInertia I{};
    if (mass != 0.f) {
        // AABB-box inertia with the full extent as "half extent" (b3GpuNarrowPhase.cpp:876-901)
        float halfExtents[3] = {amax.x - amin.x, amax.y - amin.y, amax.z - amin.z};
        float lx = 2.f * halfExtents[0], ly = 2.f * halfExtents[1], lz = 2.f * halfExtents[2];
        float li[3] = {(mass / 12.0f) * (ly * ly + lz * lz), (mass / 12.0f) * (lx * lx + lz * lz),
                       (mass / 12.0f) * (lx * lx + ly * ly)};
        float inv[3] = {1.f / li[0], 1.f / li[1], 1.f / li[2]};
        I.initInvInertia.row[0] = b3gFloat4{inv[0], 0, 0, 0};
        I.initInvInertia.row[1] = b3gFloat4{0, inv[1], 0, 0};
        I.initInvInertia.row[2] = b3gFloat4{0, 0, inv[2], 0};
        v3 rows[3] = {mk3(R.r0.x * inv[0], R.r0.y * inv[1], R.r0.z * inv[2]),
                      mk3(R.r1.x * inv[0], R.r1.y * inv[1], R.r1.z * inv[2]),
                      mk3(R.r2.x * inv[0], R.r2.y * inv[1], R.r2.z * inv[2])};
        for (int r = 0; r < 3; r++) {
            I.invInertiaWorld.row[r].x = dot3(rows[r], R.r0);
            I.invInertiaWorld.row[r].y = dot3(rows[r], R.r1);
            I.invInertiaWorld.row[r].z = dot3(rows[r], R.r2);
            I.invInertiaWorld.row[r].w = 0.f;
        }
    }
    h->bodies.push_back(b);
    h->inertias.push_back(I);
    h->user_index.push_back(user_index);
    *out = (int)h->bodies.size() - 1;
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- batched scenes
extern "C" b3gStatus b3g_set_scene_offsets(b3g_handle h, const int* first_body, int num_scenes) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (h->uploaded) return fail(B3G_ERR_INVALID_ARG, "set scene offsets before b3g_write_all_to_gpu");
    if (num_scenes <= 1) {
        h->scene_first.clear();
        return B3G_OK;
    }
    if (!first_body) return fail(B3G_ERR_INVALID_ARG, "null scene offset table");
    if (num_scenes > B3G_MAX_SCENES) return fail(B3G_ERR_CAPACITY, "%d scenes > %d", num_scenes, B3G_MAX_SCENES);
    if (first_body[0] != 0) return fail(B3G_ERR_INVALID_ARG, "the first scene must start at body 0");
    for (int s = 1; s < num_scenes; s++)
        if (first_body[s] < first_body[s - 1])
            return fail(B3G_ERR_INVALID_ARG, "scene offsets must be non-decreasing (scene %d)", s);
    h->scene_first.assign(first_body, first_body + num_scenes);
    return B3G_OK;
}

extern "C" b3gStatus b3g_set_gravity(b3g_handle h, const float g[3]) {
    if (!h || !g) return fail(B3G_ERR_INVALID_ARG, "null argument");
    h->cfg.gravity[0] = g[0];
    h->cfg.gravity[1] = g[1];
    h->cfg.gravity[2] = g[2];
    drop_graphs(h);  // force re-capture
    return B3G_OK;
}

extern "C" b3gStatus b3g_set_solver(b3g_handle h, int mode, int iterations, float residual_tol) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (mode != B3G_SOLVER_PGS && mode != B3G_SOLVER_JACOBI) return fail(B3G_ERR_INVALID_ARG, "bad solver mode");
    if (iterations < 1 || iterations > 4096) return fail(B3G_ERR_INVALID_ARG, "iterations out of range");
    h->cfg.solver_mode = mode;
    h->cfg.solver_iterations = iterations;
    h->cfg.residual_tol = residual_tol;
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- upload
static int bits_for(int n) {
    int b = 1;
    while ((1 << b) < n) b++;
    return b;
}

extern "C" b3gStatus b3g_write_all_to_gpu(b3g_handle h) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    CUDA_TRY(cudaSetDevice(h->device));
    if (!h->stream) CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    cudaStreamSynchronize(h->stream);
    if (sync_joint_flags(h) != B3G_OK) return B3G_ERR_CUDA;
    free_device(h);
    h->joints_dirty = true;  // a new upload: batch and upload the joints again at the next solve
    h->tuned = false;
    h->tuning = b3gTuning{};
    DeviceState& d = h->d;
    const int N = (int)h->bodies.size();
    if (N < 1) return fail(B3G_ERR_INVALID_ARG, "no bodies registered");
    int sms = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    d.num_sms = sms;
    d.num_bodies = N;
    d.num_collidables = (int)h->collidables.size();
    // dynamic (small) and static (large) proxies, as registerPhysicsInstance does (:650-657)
    // static bodies: unbounded AABBs (planes) are tested by every body of their scene; finite
    // ones go through the 1-axis sweep and prune
    std::vector<int> dyn_slot(N, -1), large, sap;
    int nd = 0;
    float max_extent = 0.f;
    for (int i = 0; i < N; i++) {
        if (h->bodies[i].invMass != 0.f) {
            dyn_slot[i] = nd++;
            const b3gAabb& la = h->local_aabbs[h->bodies[i].collidableIdx];
            float hx = 0.5f * (la.maxv[0] - la.minv[0]), hy = 0.5f * (la.maxv[1] - la.minv[1]),
                  hz = 0.5f * (la.maxv[2] - la.minv[2]);
            // largest world-AABB extent the body can reach under any rotation: 2 |half extents|
            float e = 2.f * std::sqrt(hx * hx + hy * hy + hz * hz);
            max_extent = std::max(max_extent, e);
        } else {
            const b3gAabb& la = h->local_aabbs[h->bodies[i].collidableIdx];
            bool finite = true;
            for (int k = 0; k < 3; k++)
                if (!(std::fabs(la.minv[k]) < 1e10f && std::fabs(la.maxv[k]) < 1e10f)) finite = false;
            (finite ? sap : large).push_back(i);
        }
    }
    d.num_dynamic = nd;
    d.num_large = (int)large.size();
    d.num_sap = (int)sap.size();
    {
        // sweep axis: largest spread of the finite static bodies' positions
        double m[3] = {0, 0, 0}, q[3] = {0, 0, 0};
        for (int i : sap)
            for (int k = 0; k < 3; k++) {
                const double x = (&h->bodies[i].pos.x)[k];
                m[k] += x;
                q[k] += x * x;
            }
        d.sap_axis = 0;
        double best = -1.0;
        for (int k = 0; k < 3 && !sap.empty(); k++) {
            const double var = q[k] / sap.size() - (m[k] / sap.size()) * (m[k] / sap.size());
            if (var > best) { best = var; d.sap_axis = k; }
        }
    }
    // independent scenes: per-body scene index and, per scene, its range of the large list (bodies
    // are registered scene by scene, so the large list is already grouped by scene)
    std::vector<int> body_scene, large_off;
    d.num_scenes = 1;
    if (!h->scene_first.empty()) {
        const int S = (int)h->scene_first.size();
        if (h->scene_first.back() > N) return fail(B3G_ERR_INVALID_ARG, "scene offsets beyond the registered bodies");
        d.num_scenes = S;
        body_scene.assign(N, 0);
        for (int sc = 0; sc < S; sc++) {
            int e = sc + 1 < S ? h->scene_first[sc + 1] : N;
            for (int i = h->scene_first[sc]; i < e; i++) body_scene[i] = sc;
        }
        large_off.assign(S + 1, 0);
        for (int i : large) large_off[body_scene[i] + 1]++;
        for (int sc = 0; sc < S; sc++) large_off[sc + 1] += large_off[sc];
    }
    std::vector<int> sap_off(d.num_scenes + 1, 0);
    for (int i : sap) sap_off[(d.num_scenes > 1 ? body_scene[i] : 0) + 1]++;
    for (int sc = 0; sc < d.num_scenes; sc++) sap_off[sc + 1] += sap_off[sc];
    float cell = h->cfg.grid_cell_size > 0.f ? h->cfg.grid_cell_size : max_extent;
    // exactness of the 27-cell search needs cell >= every dynamic AABB extent
    if (cell < max_extent) cell = max_extent;
    if (!(cell > 0.f)) cell = 1.f;
    d.inv_cell = 1.f / cell;
    d.grid_dim = h->cfg.grid_dim;
    d.grid_bits = bits_for(d.grid_dim);
    d.body_bits = bits_for(N + 1);
    if (2 * d.body_bits > 64) return fail(B3G_ERR_CAPACITY, "too many bodies");
    d.max_pairs = h->cfg.max_pairs > 0 ? h->cfg.max_pairs : std::max(4096, 24 * N);
    // at most one manifold per pair, and one per compound child pair: contact storage is sized with
    // the pair capacity (plus the child pairs') so that no manifold index can exceed it
    d.num_children = (int)h->children.size();
    d.max_child_pairs = d.num_children > 0 ? (h->cfg.max_compound_child_pairs > 0 ? h->cfg.max_compound_child_pairs
                                                                                  : d.max_pairs)
                                           : 0;
    d.num_meshes = (int)h->bvh_infos.size();
    d.max_concave_pairs =
        d.num_meshes > 0 ? (h->cfg.max_concave_pairs > 0 ? h->cfg.max_concave_pairs : d.max_pairs) : 0;
    d.max_contacts = d.max_pairs + d.max_child_pairs + d.max_concave_pairs;
    d.prim.sort_blocks = sms * d.tune.sort_blocks_per_sm;
    d.prim.scan_blocks = sms * 2;

    const size_t nh = std::max<size_t>(1, h->hulls.size()), nf = std::max<size_t>(1, h->faces.size()),
                 ni = std::max<size_t>(1, h->indices.size()), nvx = std::max<size_t>(1, h->vertices.size()),
                 ne = std::max<size_t>(1, h->edges.size());
    TRY(dalloc(h, &d.bodies, N));
    TRY(dalloc(h, &d.inertias, N));
    TRY(dalloc(h, &d.collidables, d.num_collidables));
    TRY(dalloc(h, &d.local_aabbs, d.num_collidables));
    TRY(dalloc(h, &d.hulls, nh));
    TRY(dalloc(h, &d.faces, nf));
    TRY(dalloc(h, &d.indices, ni));
    TRY(dalloc(h, &d.vertices, nvx));
    TRY(dalloc(h, &d.edges, ne));
    TRY(dalloc(h, &d.dyn_slot, N));
    TRY(dalloc(h, &d.col_small, d.num_collidables));
    TRY(dalloc(h, &d.hull_face_dup, nh));
    TRY(dalloc(h, &d.large_list, std::max(1, d.num_large)));
    TRY(dalloc(h, &d.sap_list, std::max(1, d.num_sap)));
    TRY(dalloc(h, &d.sap_sorted, std::max(1, d.num_sap)));
    TRY(dalloc(h, &d.sap_min, std::max(1, d.num_sap)));
    TRY(dalloc(h, &d.sap_off, d.num_scenes + 1));
    TRY(dalloc(h, &d.sap_ext, d.num_scenes));
    if (d.num_scenes > 1) {
        TRY(dalloc(h, &d.body_scene, N));
        TRY(dalloc(h, &d.large_off, d.num_scenes + 1));
    }
    TRY(dalloc(h, &d.aabbs, N));
    for (int k = 0; k < 2; k++) {
        TRY(dalloc(h, &d.cell_keys[k], std::max(1, nd)));
        TRY(dalloc(h, &d.cell_vals[k], std::max(1, nd)));
        TRY(dalloc(h, &d.pair_keys[k], d.max_pairs));
        TRY(dalloc(h, &d.jac_keys[k], 2 * (size_t)d.max_contacts));
        TRY(dalloc(h, &d.jac_vals[k], 2 * (size_t)d.max_contacts));
    }
    const size_t ncells = (size_t)1 << (3 * d.grid_bits);
    TRY(dalloc(h, &d.cell_start, ncells));
    TRY(dalloc(h, &d.pairs, d.max_pairs));
    TRY(dalloc(h, &d.type_lists, (size_t)PT_COUNT * d.max_pairs));
    TRY(dalloc(h, &d.contact_slots, d.max_contacts));
    TRY(dalloc(h, &d.contact_flag, d.max_contacts));
    TRY(dalloc(h, &d.contact_index, d.max_contacts));
    TRY(dalloc(h, &d.manifold_pair, d.max_contacts));
    if (d.num_children > 0) {
        TRY(dalloc(h, &d.children, d.num_children));
        TRY(dalloc(h, &d.child_count, d.max_pairs));
        TRY(dalloc(h, &d.child_offset, d.max_pairs));
        TRY(dalloc(h, &d.child_pairs, d.max_child_pairs));
    }
    if (d.num_meshes > 0) {
        TRY(dalloc(h, &d.bvh_infos, d.num_meshes));
        TRY(dalloc(h, &d.bvh_nodes, h->bvh_nodes.size()));
        TRY(dalloc(h, &d.concave_count, d.max_pairs));
        TRY(dalloc(h, &d.concave_offset, d.max_pairs));
        TRY(dalloc(h, &d.concave_pairs, d.max_concave_pairs));
    }
    TRY(dalloc(h, &d.contacts_compact, d.max_contacts));
    TRY(dalloc(h, &d.sp.nf, d.max_contacts));
    TRY(dalloc(h, &d.sp.rel1, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp.rel2, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp.dir2, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp.dir1, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp.rhsf, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp.imp, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.nf, d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.rel1, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.rel2, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.dir2, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.dir1, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.rhsf, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.imp, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.angP, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.angQ, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.angR, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.angS, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.sp_ord.angT, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.manifold_hdr_ord, d.max_contacts));
    TRY(dalloc(h, &d.body_slot, N));
    TRY(dalloc(h, &d.manifold_group, d.max_contacts));
    TRY(dalloc(h, &d.group_counts, 3 * ((size_t)sms * B3G_PGS_MAX_BLOCKS_PER_SM * 64 + 64 + 2)));
    TRY(dalloc(h, &d.manifold_inv_mass_ord, d.max_contacts));
    TRY(dalloc(h, &d.inertia_ord, 6 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.manifold_color, d.max_contacts));
    TRY(dalloc(h, &d.color_order, d.max_contacts));
    TRY(dalloc(h, &d.manifold_pos, d.max_contacts));
    TRY(dalloc(h, &d.prev_mkey, d.max_contacts));
    TRY(dalloc(h, &d.prev_mcolor, d.max_contacts));
    TRY(dalloc(h, &d.prev_mn, 4));  // manifolds of the last solve, colours of the last fresh colouring, recolour flag
    CUDA_TRY(cudaMemsetAsync(d.prev_mn, 0, 4 * sizeof(int), h->stream));
    TRY(dalloc(h, &d.color_offsets, 4 * (B3G_MAX_COLORS + 2)));  // offsets, fill, remaining, cursors
    TRY(dalloc(h, &d.color_claim, 4 * (size_t)N));  // claims, colour masks; again for cross-partition
    CUDA_TRY(solver_prepare());
    if (h->cfg.warm_start != 0) {
        // warm-start features (and predictions) for the first `cap` point slots
        long long cap = h->cfg.warm_start_max_points > 0 ? h->cfg.warm_start_max_points
                                                         : std::max(8192LL, 8LL * (long long)N);
        cap = std::min(cap, 4LL * (long long)d.max_contacts);
        cap = cap / 4 * 4;
        d.ws_rows_cap = (int)cap;
        const int wm = h->cfg.warm_start;
        if (wm == B3G_WARM_LEARNED || wm == B3G_WARM_RECORD || wm == B3G_WARM_PERSISTENT_LEARNED)
            TRY(dalloc(h, &d.ws_features, (size_t)cap * 12));
        TRY(dalloc(h, &d.ws_rows, 1));
        TRY(dalloc(h, &d.ws_init, (size_t)cap));
        TRY(dalloc(h, &d.ws_new, (size_t)cap));
        TRY(dalloc(h, &d.prev_keys, (size_t)cap / 4));
        TRY(dalloc(h, &d.prev_pts, (size_t)cap));
        TRY(dalloc(h, &d.prev_imp, (size_t)cap));
        TRY(dalloc(h, &d.prev_n, 1));
        CUDA_TRY(cudaMemsetAsync(d.prev_n, 0, sizeof(int), h->stream));
        if (h->ws_mlp) {
            d.ws_model = b3g_mlp_model(h->ws_mlp);
            CUDA_TRY(mlp::ensure_infer(*d.ws_model, d.ws_rows_cap));
            CUDA_TRY(cudaSetDevice(h->device));
        }
    }
    TRY(dalloc(h, &d.dv, 2 * (size_t)N));
    TRY(dalloc(h, &d.dv_sum, 2 * (size_t)N));
    TRY(dalloc(h, &d.manifold_hdr, d.max_contacts));
    TRY(dalloc(h, &d.manifold_inv_mass, d.max_contacts));
    TRY(dalloc(h, &d.body_manifold_count, N + 1));
    TRY(dalloc(h, &d.body_list_offsets, N + 1));
    TRY(dalloc(h, &d.split_dv, 4 * (size_t)d.max_contacts));
    TRY(dalloc(h, &d.residual_acc, 2 * 4096));
    TRY(dalloc(h, &d.counters, 1));
    TRY(dalloc(h, &d.barrier, 64));
    {
        unsigned char* p = nullptr;
        PrimConfig widest = d.prim;  // the autotuner may raise the sort's block count up to this
        widest.sort_blocks = sms * B3G_MAX_SORT_BLOCKS_PER_SM;
        TRY(dalloc(h, &p, radix_scratch_bytes(widest)));
        d.sort_scratch = p;
        TRY(dalloc(h, &p, scan_scratch_bytes(d.prim)));
        d.scan_scratch = p;
    }
    TRY(dalloc(h, &d.d_num_dynamic, 4));
    d.d_num_bodies = d.d_num_dynamic + 1;

    cudaStream_t s = h->stream;
    CUDA_TRY(cudaMemcpyAsync(d.bodies, h->bodies.data(), sizeof(b3gBody) * N, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.inertias, h->inertias.data(), sizeof(b3gInertia) * N, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.collidables, h->collidables.data(), sizeof(b3gCollidable) * d.num_collidables,
                             cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.local_aabbs, h->local_aabbs.data(), sizeof(b3gAabb) * d.num_collidables,
                             cudaMemcpyHostToDevice, s));
    if (!h->hulls.empty())
        CUDA_TRY(cudaMemcpyAsync(d.hulls, h->hulls.data(), sizeof(b3gHull) * h->hulls.size(), cudaMemcpyHostToDevice, s));
    if (!h->faces.empty())
        CUDA_TRY(cudaMemcpyAsync(d.faces, h->faces.data(), sizeof(b3gFace) * h->faces.size(), cudaMemcpyHostToDevice, s));
    if (!h->indices.empty())
        CUDA_TRY(cudaMemcpyAsync(d.indices, h->indices.data(), sizeof(int) * h->indices.size(), cudaMemcpyHostToDevice, s));
    if (!h->vertices.empty())
        CUDA_TRY(cudaMemcpyAsync(d.vertices, h->vertices.data(), sizeof(b3gFloat4) * h->vertices.size(),
                                 cudaMemcpyHostToDevice, s));
    if (!h->edges.empty())
        CUDA_TRY(cudaMemcpyAsync(d.edges, h->edges.data(), sizeof(b3gFloat4) * h->edges.size(), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.dyn_slot, dyn_slot.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s));
    if (d.num_children > 0)
        CUDA_TRY(cudaMemcpyAsync(d.children, h->children.data(), sizeof(b3gChildShape) * h->children.size(),
                                 cudaMemcpyHostToDevice, s));
    if (d.num_meshes > 0) {
        CUDA_TRY(cudaMemcpyAsync(d.bvh_infos, h->bvh_infos.data(), sizeof(b3gBvhInfo) * h->bvh_infos.size(),
                                 cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(d.bvh_nodes, h->bvh_nodes.data(), sizeof(b3gBvhNode) * h->bvh_nodes.size(),
                                 cudaMemcpyHostToDevice, s));
    }
    {
        // faces whose normal is the exact negation of an earlier face's (a box's opposite faces):
        // rotated and sign-flipped towards the other body they give the earlier face's SAT axis
        // and the same overlap, which never wins (the first minimum is kept), so the SAT skips them
        std::vector<uint32_t> dup(nh, 0u);
        for (size_t k = 0; k < h->hulls.size(); k++) {
            const b3gHull& hull = h->hulls[k];
            const int nf = std::min(hull.numFaces, 32);
            for (int f = 1; f < nf; f++) {
                const b3gFloat4& pf = h->faces[hull.faceOffset + f].plane;
                for (int g = 0; g < f; g++) {
                    const b3gFloat4& pg = h->faces[hull.faceOffset + g].plane;
                    // equal as numbers (the sign of a zero component only changes the sign of zeros in
                    // the rotated axis and its projections, never a comparison)
                    if (-pg.x == pf.x && -pg.y == pf.y && -pg.z == pf.z) {
                        dup[k] |= 1u << f;
                        break;
                    }
                }
            }
        }
        CUDA_TRY(cudaMemcpyAsync(d.hull_face_dup, dup.data(), sizeof(uint32_t) * nh, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaStreamSynchronize(s));  // `dup` is a local: finish the copy before it goes
    }
    std::vector<int> col_small(d.num_collidables, 0);
    for (int c = 0; c < d.num_collidables; c++) {
        const b3gCollidable& col = h->collidables[c];
        if (col.shapeType != B3G_SHAPE_CONVEX_HULL) continue;
        const b3gHull& hull = h->hulls[col.shapeIndex];
        int small = 1;
        for (int f = 0; f < hull.numFaces; f++)
            if (h->faces[hull.faceOffset + f].numIndices > B3G_SMALL_FACE_VERTS) small = 0;
        // small-faced hulls carry their SAT axis counts (faces, unique edges) for the per-pair choice
        col_small[c] = small ? (1 | (std::min(hull.numFaces, 0x7fff) << 1) | (std::min(hull.numUniqueEdges, 0x7fff) << 16))
                             : 0;
    }
    CUDA_TRY(cudaMemcpyAsync(d.col_small, col_small.data(), sizeof(int) * d.num_collidables, cudaMemcpyHostToDevice,
                             s));
    if (!large.empty())
        CUDA_TRY(cudaMemcpyAsync(d.large_list, large.data(), sizeof(int) * large.size(), cudaMemcpyHostToDevice, s));
    if (!sap.empty())
        CUDA_TRY(cudaMemcpyAsync(d.sap_list, sap.data(), sizeof(int) * sap.size(), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.sap_off, sap_off.data(), sizeof(int) * sap_off.size(), cudaMemcpyHostToDevice, s));
    if (d.num_scenes > 1) {
        CUDA_TRY(cudaMemcpyAsync(d.body_scene, body_scene.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(d.large_off, large_off.data(), sizeof(int) * (d.num_scenes + 1),
                                 cudaMemcpyHostToDevice, s));
    }
    int sizes[4] = {nd, N, 0, 0};
    CUDA_TRY(cudaMemcpyAsync(d.d_num_dynamic, sizes, sizeof(sizes), cudaMemcpyHostToDevice, s));
    // an all-ones cell table is never a valid run start (validated against sorted keys)
    CUDA_TRY(cudaMemsetAsync(d.cell_start, 0xff, sizeof(uint32_t) * ncells, s));
    CUDA_TRY(cudaMemsetAsync(d.counters, 0, sizeof(DevCounters), s));
    CUDA_TRY(cudaMemsetAsync(d.barrier, 0, 64 * sizeof(unsigned int), s));
    CUDA_TRY(cudaStreamSynchronize(s));
    d.scene_bits = d.num_scenes > 1 ? bits_for(d.num_scenes) : 0;
    d.broadphase = h->cfg.broadphase == B3G_BROADPHASE_LBVH ? B3G_BROADPHASE_LBVH : B3G_BROADPHASE_GRID;
    if (d.broadphase == B3G_BROADPHASE_LBVH) TRY(alloc_lbvh(d));
    h->uploaded = true;
    return B3G_OK;
}

extern "C" b3gStatus b3g_set_broadphase(b3g_handle h, int mode) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (mode < B3G_BROADPHASE_GRID || mode > B3G_BROADPHASE_AUTO)
        return fail(B3G_ERR_INVALID_ARG, "unknown broadphase %d", mode);
    h->cfg.broadphase = mode;
    if (!h->uploaded) return B3G_OK;
    CUDA_TRY(cudaSetDevice(h->device));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (mode == B3G_BROADPHASE_LBVH) TRY(alloc_lbvh(h->d));
    // AUTO: the grid until the autotuner (at its next run) picks
    h->d.broadphase = mode == B3G_BROADPHASE_LBVH ? B3G_BROADPHASE_LBVH : B3G_BROADPHASE_GRID;
    if (mode == B3G_BROADPHASE_AUTO) h->tuned = false;
    drop_graphs(h);  // the captured step has the other broadphase's launches
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- the step
#define REQUIRE_UPLOADED(h)                                                                        \
    do {                                                                                           \
        if (!(h)) return fail(B3G_ERR_INVALID_ARG, "null handle");                                 \
        if (!(h)->uploaded) return fail(B3G_ERR_NOT_UPLOADED, "call b3g_write_all_to_gpu first"); \
    } while (0)

static b3gStatus check_launch(b3gWorld* h) {
    cudaError_t e = h->d.launch_error;
    h->d.launch_error = cudaSuccess;
    cudaError_t e2 = cudaGetLastError();
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(B3G_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return B3G_OK;
}

// Stage boundary k of a profiled step: an event record on the stream, or, while the step is being
// captured, an event-record node of the graph (so a replay of the profiled graph times the stages
// of the captured step itself).
static void record(b3gWorld* h, int k) {
    if (!h->profiling) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(h->stream, &cs);
    if (cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(h->events.ev[k], h->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(h->events.ev[k], h->stream);
}

// ---------------------------------------------------------------------------------- joints
// b3GpuRigidBodyPipeline::createPoint2PointConstraint / createFixedConstraint /
// removeConstraintByUid (b3GpuRigidBodyPipeline.cpp:159-219) keep a host list of
// b3GpuGenericConstraint and clear the joint solver's batches; the batches are rebuilt before the
// next solve.  Same here: every change marks the registry dirty, and the next step (or
// b3g_solve_joints) batches and uploads it.

// Copies the device's enabled flags (cleared by the break check) into the host registry; valid
// while the device copy matches the registry.
static b3gStatus sync_joint_flags(b3gWorld* h) {
    DeviceState& d = h->d;
    if (h->joints_dirty || !h->uploaded || d.num_joints <= 0 || !d.joints) return B3G_OK;
    std::vector<b3gJoint> dev((size_t)d.num_joints);
    CUDA_TRY(cudaMemcpyAsync(dev.data(), d.joints, sizeof(b3gJoint) * dev.size(), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < dev.size() && i < h->joints.size(); ++i) h->joints[i].flags = dev[i].flags;
    return B3G_OK;
}

// sortConstraintByBatch3 (b3GpuPgsConstraintSolver.cpp:781-907) as the joint solver calls it
// (simdWidth = numConstraints + 1, staticIdx = -1, b3GpuPgsConstraintSolver.cpp:193,641-644): a
// body is "static" when its signed index is negative (inverse mass zero, index > 0; body 0 keeps
// index 0 and so counts as dynamic).  Each pass over the joints not yet batched takes, in list
// order, every joint whose non-static bodies no earlier joint of the pass took, and moves it to
// the front by swapping it with the first unbatched entry.
static void batch_joints(const std::vector<int>& sa, const std::vector<int>& sb, int num_bodies,
                         std::vector<int>& order, std::vector<int>& offsets) {
    const int n = (int)sa.size();
    std::vector<int> A(sa), B(sb);
    order.resize((size_t)n);
    for (int i = 0; i < n; ++i) order[(size_t)i] = i;
    offsets.assign(1, 0);
    std::vector<uint32_t> used((size_t)num_bodies / 32 + 1, 0u);
    std::vector<int> touched;
    int done = 0;
    while (done < n) {
        for (int b : touched) used[(size_t)b / 32] = 0;
        touched.clear();
        int count = 0;
        for (int i = done; i < n; ++i) {
            const int as = A[(size_t)i], bs = B[(size_t)i];
            const int a = as < 0 ? -as : as, b = bs < 0 ? -bs : bs;
            const bool a_static = as < 0, b_static = bs < 0;
            bool a_busy = false, b_busy = false;
            if (!a_static) a_busy = (used[(size_t)a / 32] >> (a & 31)) & 1u;
            if (!a_busy && !b_static) b_busy = (used[(size_t)b / 32] >> (b & 31)) & 1u;
            if (a_busy || b_busy) continue;
            if (!a_static) {
                used[(size_t)a / 32] |= 1u << (a & 31);
                touched.push_back(a);
            }
            if (!b_static) {
                used[(size_t)b / 32] |= 1u << (b & 31);
                touched.push_back(b);
            }
            if (i != done) {
                std::swap(A[(size_t)i], A[(size_t)done]);
                std::swap(B[(size_t)i], B[(size_t)done]);
                std::swap(order[(size_t)i], order[(size_t)done]);
            }
            ++done;
            ++count;
        }
        offsets.push_back(offsets.back() + count);
    }
}

template <typename T>
static b3gStatus joint_alloc(T** p, size_t count) {
    cudaFree(*p);
    *p = nullptr;
    CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(p), (count ? count : 1) * sizeof(T)));
    return B3G_OK;
}

// Batches and uploads a changed registry; the captured step graph is dropped when the joint
// stage's shape changed.
static b3gStatus prepare_joints(b3gWorld* h) {
    if (!h->joints_dirty) return B3G_OK;
    DeviceState& d = h->d;
    cudaStream_t s = h->stream;
    const int n = (int)h->joints.size();
    drop_graphs(h);
    d.num_joints = 0;
    d.num_joint_batches = 0;
    d.num_joint_uniq = 0;
    d.max_joint_batch = 0;
    h->joint_order.clear();
    h->joint_batch_off.assign(1, 0);
    if (n == 0) {
        h->joints_dirty = false;
        return B3G_OK;
    }
    if (n > d.joint_cap) {
        const int cap = std::max(n, std::max(64, 2 * d.joint_cap));
        TRY(joint_alloc(&d.joints, (size_t)cap));
        TRY(joint_alloc(&d.joint_hdr, (size_t)cap));
        TRY(joint_alloc(&d.joint_rows, 6 * (size_t)cap));
        TRY(joint_alloc(&d.joint_imp, 6 * (size_t)cap));
        TRY(joint_alloc(&d.joint_order, (size_t)cap));
        TRY(joint_alloc(&d.joint_batch_off, (size_t)cap + 1));
        TRY(joint_alloc(&d.joint_uniq, 2 * (size_t)cap));
        TRY(joint_alloc(&d.joint_mass, (size_t)cap));
        d.joint_cap = cap;
    }
    if (d.joint_dv_bodies != d.num_bodies) {
        TRY(joint_alloc(&d.joint_dv, 2 * (size_t)d.num_bodies));
        CUDA_TRY(cudaMemsetAsync(d.joint_dv, 0, 2 * sizeof(float4) * (size_t)d.num_bodies, s));
        d.joint_dv_bodies = d.num_bodies;
    }
    CUDA_TRY(cudaMemcpyAsync(d.joints, h->joints.data(), sizeof(b3gJoint) * (size_t)n, cudaMemcpyHostToDevice, s));
    // signed body indices from the bodies' current inverse masses (initBatchConstraintsKernel,
    // jointSolver.cl:400-419)
    launch_joint_masses(d, n, d.joint_mass, s);
    std::vector<float2> mass((size_t)n);
    CUDA_TRY(cudaMemcpyAsync(mass.data(), d.joint_mass, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<int> sa((size_t)n), sb((size_t)n);
    for (int i = 0; i < n; ++i) {
        const b3gJoint& c = h->joints[(size_t)i];
        sa[(size_t)i] = mass[(size_t)i].x != 0.f ? c.rbA : -c.rbA;
        sb[(size_t)i] = mass[(size_t)i].y != 0.f ? c.rbB : -c.rbB;
    }
    batch_joints(sa, sb, d.num_bodies, h->joint_order, h->joint_batch_off);
    std::vector<int> uniq;
    uniq.reserve(2 * (size_t)n);
    for (const b3gJoint& c : h->joints) {
        uniq.push_back(c.rbA);
        uniq.push_back(c.rbB);
    }
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    int widest = 0;
    for (size_t b = 0; b + 1 < h->joint_batch_off.size(); ++b)
        widest = std::max(widest, h->joint_batch_off[b + 1] - h->joint_batch_off[b]);
    CUDA_TRY(cudaMemcpyAsync(d.joint_order, h->joint_order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.joint_batch_off, h->joint_batch_off.data(), sizeof(int) * h->joint_batch_off.size(),
                             cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.joint_uniq, uniq.data(), sizeof(int) * uniq.size(), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors above are locals
    d.num_joints = n;
    d.num_joint_batches = (int)h->joint_batch_off.size() - 1;
    d.num_joint_uniq = (int)uniq.size();
    d.max_joint_batch = widest;
    h->joints_dirty = false;
    return B3G_OK;
}

static b3gStatus add_joint(b3gWorld* h, int type, int body_a, int body_b, const float* pa, const float* pb,
                           const float* rel, float threshold, int* out_uid) {
    if (!h || !pa || !pb) return fail(B3G_ERR_INVALID_ARG, "null argument");
    const int nb = (int)h->bodies.size();
    if (body_a < 0 || body_a >= nb || body_b < 0 || body_b >= nb)
        return fail(B3G_ERR_INVALID_INDEX, "joint body index out of range (%d, %d of %d bodies)", body_a, body_b, nb);
    if (body_a == body_b) return fail(B3G_ERR_INVALID_ARG, "a joint needs two different bodies");
    TRY(sync_joint_flags(h));
    b3gJoint c;
    std::memset(&c, 0, sizeof(c));
    c.type = type;
    c.rbA = body_a;
    c.rbB = body_b;
    c.breakingImpulseThreshold = threshold;
    c.pivotInA = b3gFloat4{pa[0], pa[1], pa[2], 0.f};
    c.pivotInB = b3gFloat4{pb[0], pb[1], pb[2], 0.f};
    if (rel) c.relTargetAB = b3gFloat4{rel[0], rel[1], rel[2], rel[3]};
    c.flags = 1;
    c.uid = h->next_joint_uid++;
    h->joints.push_back(c);
    h->joints_dirty = true;
    if (out_uid) *out_uid = c.uid;
    return B3G_OK;
}

extern "C" b3gStatus b3g_create_point2point_constraint(b3g_handle h, int body_a, int body_b, const float pivot_in_a[3],
                                                       const float pivot_in_b[3], float breaking_threshold,
                                                       int* out_uid) {
    return add_joint(h, B3G_JOINT_POINT2POINT, body_a, body_b, pivot_in_a, pivot_in_b, nullptr, breaking_threshold,
                     out_uid);
}

extern "C" b3gStatus b3g_create_fixed_constraint(b3g_handle h, int body_a, int body_b, const float pivot_in_a[3],
                                                 const float pivot_in_b[3], const float rel_target_ab[4],
                                                 float breaking_threshold, int* out_uid) {
    if (!rel_target_ab) return fail(B3G_ERR_INVALID_ARG, "null relative target");
    return add_joint(h, B3G_JOINT_FIXED, body_a, body_b, pivot_in_a, pivot_in_b, rel_target_ab, breaking_threshold,
                     out_uid);
}

extern "C" b3gStatus b3g_remove_constraint(b3g_handle h, int uid) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    TRY(sync_joint_flags(h));
    for (size_t i = 0; i < h->joints.size(); ++i) {
        if (h->joints[i].uid == uid) {  // swap with the last and pop, as the reference does
            std::swap(h->joints[i], h->joints.back());
            h->joints.pop_back();
            h->joints_dirty = true;
            return B3G_OK;
        }
    }
    return fail(B3G_ERR_INVALID_INDEX, "no joint with uid %d", uid);
}

extern "C" b3gStatus b3g_get_num_constraints(b3g_handle h, int* n) {
    if (!h || !n) return fail(B3G_ERR_INVALID_ARG, "null argument");
    *n = (int)h->joints.size();
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_constraints(b3g_handle h, void* host_joints, int capacity, int* n) {
    if (!h || (!host_joints && capacity > 0)) return fail(B3G_ERR_INVALID_ARG, "null argument");
    if (h->uploaded) CUDA_TRY(cudaSetDevice(h->device));
    TRY(sync_joint_flags(h));
    const int m = std::min(capacity, (int)h->joints.size());
    if (m > 0) std::memcpy(host_joints, h->joints.data(), sizeof(b3gJoint) * (size_t)m);
    if (n) *n = (int)h->joints.size();
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_joint_order(b3g_handle h, int* order, int capacity, int* batch_offsets,
                                          int offsets_capacity, int* num_batches) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (h->joints_dirty) return fail(B3G_ERR_INVALID_ARG, "joints changed since the last joint solve");
    const int n = (int)h->joint_order.size(), nb = (int)h->joint_batch_off.size();
    if ((order && capacity < n) || (batch_offsets && offsets_capacity < nb))
        return fail(B3G_ERR_CAPACITY, "need %d order and %d offset entries", n, nb);
    if (order && n) std::memcpy(order, h->joint_order.data(), sizeof(int) * (size_t)n);
    if (batch_offsets && nb) std::memcpy(batch_offsets, h->joint_batch_off.data(), sizeof(int) * (size_t)nb);
    if (num_batches) *num_batches = nb > 0 ? nb - 1 : 0;
    return B3G_OK;
}

static void enqueue_step(b3gWorld* h, float dt, bool with_events) {
    cudaStream_t s = h->stream;
    DeviceState& d = h->d;
    long long n = 0;
    if (with_events) record(h, 0);
    n += launch_aabbs(d, s);
    if (with_events) record(h, 1);
    n += launch_pairs(d, s);
    if (with_events) record(h, 2);
    n += launch_contacts(d, h->cfg.contact_friction, s);
    if (with_events) record(h, 3);
    // stage 3->4: the joints (contact batching is fused into the solver kernel)
    n += launch_joints(d, h->cfg, s);
    if (with_events) record(h, 4);
    n += launch_solver(d, h->cfg, dt, s);
    if (with_events) record(h, 5);
    if (with_events) record(h, 6);
    n += launch_integrate(d, h->cfg, dt, s);
    if (with_events) record(h, 7);
    h->launches += n;
}

extern "C" b3gStatus b3g_step(b3g_handle h, float dt) {
    REQUIRE_UPLOADED(h);
    if (!(dt > 0.f)) return fail(B3G_ERR_INVALID_ARG, "dt must be positive");
    CUDA_TRY(cudaSetDevice(h->device));
    TRY(prepare_joints(h));
    if (h->cfg.autotune && !h->tuned) TRY(b3g_autotune(h, dt, 3, nullptr));
    if (!h->cfg.use_cuda_graph) {
        enqueue_step(h, dt, h->profiling);
        TRY(check_launch(h));
        return B3G_OK;
    }
    b3gWorld::StepGraph& g = h->graphs[h->profiling ? 1 : 0];
    if (!g.exec || g.dt != dt || g.mode != h->cfg.solver_mode || g.iters != h->cfg.solver_iterations ||
        g.tol != h->cfg.residual_tol) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        cudaGraph_t graph;
        long long before = h->launches;
        CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(h, dt, h->profiling);
        CUDA_TRY(cudaStreamEndCapture(h->stream, &graph));
        {
            b3gStatus st = check_launch(h);
            if (st != B3G_OK) {
                cudaGraphDestroy(graph);
                return st;
            }
        }
        CUDA_TRY(cudaGraphInstantiate(&g.exec, graph, 0));
        cudaGraphDestroy(graph);
        g.dt = dt;
        g.mode = h->cfg.solver_mode;
        g.iters = h->cfg.solver_iterations;
        g.tol = h->cfg.residual_tol;
        g.kernels = h->launches - before;
        h->launches = before;
    }
    CUDA_TRY(cudaGraphLaunch(g.exec, h->stream));
    h->launches += g.kernels;
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- autotuner
// Times candidate launch shapes on the world's current state and keeps the fastest of each.
// Every candidate sees the same input: the bodies are saved first and put back before each timed
// run (and at the end), so tuning leaves the simulation state as it found it.
namespace {

struct TuneRun {
    float ms[4];  // aabbs, pairs, contacts, solve
};

b3gStatus tune_time(b3gWorld* h, float dt, int repeats, const b3gBody* saved, bool solve, TuneRun& out) {
    DeviceState& d = h->d;
    cudaStream_t s = h->stream;
    cudaEvent_t ev[5];
    for (int k = 0; k < 5; k++) CUDA_TRY(cudaEventCreate(&ev[k]));
    std::vector<float> t[4];
    for (int r = 0; r < repeats + 1; r++) {  // the first run warms caches and is not kept
        CUDA_TRY(cudaMemcpyAsync(d.bodies, saved, sizeof(b3gBody) * d.num_bodies, cudaMemcpyDeviceToDevice, s));
        cudaEventRecord(ev[0], s);
        launch_aabbs(d, s);
        cudaEventRecord(ev[1], s);
        launch_pairs(d, s);
        cudaEventRecord(ev[2], s);
        launch_contacts(d, h->cfg.contact_friction, s);
        cudaEventRecord(ev[3], s);
        if (solve) launch_solver(d, h->cfg, dt, s);
        cudaEventRecord(ev[4], s);
        CUDA_TRY(cudaStreamSynchronize(s));
        TRY(check_launch(h));
        if (r == 0) continue;
        for (int k = 0; k < 4; k++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            t[k].push_back(ms);
        }
    }
    for (int k = 0; k < 5; k++) cudaEventDestroy(ev[k]);
    for (int k = 0; k < 4; k++) {  // median
        std::sort(t[k].begin(), t[k].end());
        out.ms[k] = t[k][t[k].size() / 2];
    }
    return B3G_OK;
}

}  // namespace

extern "C" b3gStatus b3g_autotune(b3g_handle h, float dt, int repeats, b3gTuning* out) {
    REQUIRE_UPLOADED(h);
    if (!(dt > 0.f)) return fail(B3G_ERR_INVALID_ARG, "dt must be positive");
    if (repeats < 1 || repeats > 100) return fail(B3G_ERR_INVALID_ARG, "repeats must be in [1, 100]");
    CUDA_TRY(cudaSetDevice(h->device));
    DeviceState& d = h->d;
    cudaStream_t s = h->stream;
    b3gBody* saved = nullptr;
    CUDA_TRY(cudaMalloc(&saved, sizeof(b3gBody) * d.num_bodies));
    b3gStatus st = B3G_OK;
    b3gTuning res{};
    int timed = 0;
    do {
        if (cudaMemcpyAsync(saved, d.bodies, sizeof(b3gBody) * d.num_bodies, cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess) {
            st = fail(B3G_ERR_CUDA, "autotune: saving the bodies failed");
            break;
        }
        TuneRun run;
        // radix sort blocks, then the pair kernel's grid: both time the pair stage
        static const int sort_c[] = {2, 4, 8};
        float best = 1e30f;
        int best_v = d.tune.sort_blocks_per_sm;
        for (int v : sort_c) {
            d.tune.sort_blocks_per_sm = v;
            if ((st = tune_time(h, dt, repeats, saved, false, run)) != B3G_OK) break;
            timed++;
            if (run.ms[1] < best) { best = run.ms[1]; best_v = v; }
        }
        if (st != B3G_OK) break;
        d.tune.sort_blocks_per_sm = best_v;
        static const int grid_c[] = {2, 4, 8, 16};
        best = 1e30f;
        best_v = d.tune.pairs_blocks_per_sm;
        for (int v : grid_c) {
            d.tune.pairs_blocks_per_sm = v;
            if ((st = tune_time(h, dt, repeats, saved, false, run)) != B3G_OK) break;
            timed++;
            if (run.ms[1] < best) { best = run.ms[1]; best_v = v; }
        }
        if (st != B3G_OK) break;
        d.tune.pairs_blocks_per_sm = best_v;
        res.pairs_ms = best;
        // broadphase AUTO: the LBVH's pair stage over the same grid sizes; the faster search stays
        if (h->cfg.broadphase == B3G_BROADPHASE_AUTO && d.num_dynamic > 1) {
            if ((st = alloc_lbvh(d)) != B3G_OK) break;
            const int grid_best = best_v;
            float lbest = 1e30f;
            int lbest_v = grid_best;
            d.broadphase = B3G_BROADPHASE_LBVH;
            for (int v : grid_c) {
                d.tune.pairs_blocks_per_sm = v;
                if ((st = tune_time(h, dt, repeats, saved, false, run)) != B3G_OK) break;
                timed++;
                if (run.ms[1] < lbest) { lbest = run.ms[1]; lbest_v = v; }
            }
            if (st != B3G_OK) break;
            if (lbest < best) {
                d.tune.pairs_blocks_per_sm = lbest_v;
                res.pairs_ms = lbest;
            } else {
                d.broadphase = B3G_BROADPHASE_GRID;
                d.tune.pairs_blocks_per_sm = grid_best;
            }
        }
        // the thread-per-pair narrowphase kernel's grid: times the contact stage
        best = 1e30f;
        best_v = d.tune.narrow_blocks_per_sm;
        for (int v : grid_c) {
            d.tune.narrow_blocks_per_sm = v;
            if ((st = tune_time(h, dt, repeats, saved, false, run)) != B3G_OK) break;
            timed++;
            if (run.ms[2] < best) { best = run.ms[2]; best_v = v; }
        }
        if (st != B3G_OK) break;
        d.tune.narrow_blocks_per_sm = best_v;
        res.contacts_ms = best;
        // the PGS solver's work split (only when the configuration leaves it to AUTO)
        if (h->cfg.solver_mode == B3G_SOLVER_PGS && h->cfg.pgs_partitions == B3G_PGS_PARTITIONS_AUTO) {
            static const int split_c[] = {B3G_PGS_PARTITIONS_NONE, B3G_PGS_PARTITIONS_SHARED,
                                          B3G_PGS_PARTITIONS_GLOBAL_DELTAS, B3G_PGS_PARTITIONS_STREAMED};
            best = 1e30f;
            best_v = B3G_PGS_PARTITIONS_NONE;
            for (int v : split_c) {
                d.tune.pgs_partitions = v;
                if ((st = tune_time(h, dt, repeats, saved, true, run)) != B3G_OK) break;
                timed++;
                if (run.ms[3] < best) { best = run.ms[3]; best_v = v; }
            }
            if (st != B3G_OK) break;
            d.tune.pgs_partitions = best_v;
        } else {
            if ((st = tune_time(h, dt, repeats, saved, true, run)) != B3G_OK) break;
            timed++;
            best = run.ms[3];
        }
        res.solve_ms = best;
    } while (false);
    // the state is put back whatever happened
    cudaMemcpyAsync(d.bodies, saved, sizeof(b3gBody) * d.num_bodies, cudaMemcpyDeviceToDevice, s);
    cudaStreamSynchronize(s);
    cudaFree(saved);
    drop_graphs(h);  // the captured step used the old launch shapes
    h->tuned = true;
    if (st != B3G_OK) return st;
    res.pgs_partitions = d.tune.pgs_partitions;
    res.pairs_blocks_per_sm = d.tune.pairs_blocks_per_sm;
    res.narrow_blocks_per_sm = d.tune.narrow_blocks_per_sm;
    res.sort_blocks_per_sm = d.tune.sort_blocks_per_sm;
    res.candidates_timed = timed;
    res.broadphase = d.broadphase;
    h->tuning = res;
    if (out) *out = res;
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- ray casts
// Frees a buffer that dalloc made, after the stream has drained (work in flight may still read it).
template <typename T>
static void dfree(b3gWorld* w, T** p) {
    if (!*p) return;
    cudaStreamSynchronize(w->stream);
    auto it = std::find(w->allocations.begin(), w->allocations.end(), static_cast<void*>(*p));
    if (it != w->allocations.end()) {
        cudaFree(*p);
        w->allocations.erase(it);
    }
    *p = nullptr;
}

// Ray-cast scratch: the sort keys for every call; device copies of the rays and hits only for
// calls with host buffers (b3g_cast_rays).  Growth frees the smaller buffers.
static b3gStatus ray_buffers(b3gWorld* h, int n, bool host_copies) {
    DeviceState& d = h->d;
    if (n > d.ray_cap) {
        const int cap = std::max(n, 2 * d.ray_cap);
        dfree(h, &d.ray_order);
        TRY(dalloc(h, &d.ray_order, 4 * (size_t)cap));
        d.ray_cap = cap;
    }
    if (host_copies && d.ray_host_cap < n) {
        dfree(h, &d.ray_buf);
        dfree(h, &d.hit_buf);
        TRY(dalloc(h, &d.ray_buf, 2 * (size_t)d.ray_cap));
        TRY(dalloc(h, &d.hit_buf, (size_t)d.ray_cap));
        d.ray_host_cap = d.ray_cap;
    }
    if (!d.ray_n) TRY(dalloc(h, &d.ray_n, 1));
    return B3G_OK;
}

extern "C" b3gStatus b3g_cast_rays_device(b3g_handle h, const void* device_rays, void* device_hits, int n) {
    REQUIRE_UPLOADED(h);
    if (n < 0 || (n > 0 && (!device_rays || !device_hits))) return fail(B3G_ERR_INVALID_ARG, "invalid ray arguments");
    if ((reinterpret_cast<uintptr_t>(device_rays) | reinterpret_cast<uintptr_t>(device_hits)) & 15u)
        return fail(B3G_ERR_INVALID_ARG, "ray and hit buffers must be 16-byte aligned");
    CUDA_TRY(cudaSetDevice(h->device));
    TRY(ray_buffers(h, n, false));
    DeviceState& d = h->d;
    if (n > 0) {
        // the sort length, written by a kernel so that the call stays asynchronous
        b3g::launch_set_int(d.ray_n, n, h->stream);
    }
    h->launches += launch_cast_rays(d, reinterpret_cast<const float4*>(device_rays),
                                    reinterpret_cast<b3gRayHit*>(device_hits), n, h->stream) + (n > 0 ? 1 : 0);
    TRY(check_launch(h));
    return B3G_OK;
}

extern "C" b3gStatus b3g_cast_rays(b3g_handle h, const void* host_rays, void* host_hits, int n) {
    REQUIRE_UPLOADED(h);
    if (n < 0 || (n > 0 && (!host_rays || !host_hits))) return fail(B3G_ERR_INVALID_ARG, "invalid ray arguments");
    CUDA_TRY(cudaSetDevice(h->device));
    DeviceState& d = h->d;
    TRY(ray_buffers(h, n, true));
    cudaStream_t s = h->stream;
    if (n > 0) {
        CUDA_TRY(cudaMemcpyAsync(d.ray_buf, host_rays, sizeof(b3gRayInfo) * (size_t)n, cudaMemcpyHostToDevice, s));
        CUDA_TRY(cudaMemcpyAsync(d.hit_buf, host_hits, sizeof(b3gRayHit) * (size_t)n, cudaMemcpyHostToDevice, s));
    }
    const int count = n;  // the sort length; the stream is synchronised before this function returns
    if (n > 0) CUDA_TRY(cudaMemcpyAsync(d.ray_n, &count, sizeof(int), cudaMemcpyHostToDevice, s));
    h->launches += launch_cast_rays(d, d.ray_buf, d.hit_buf, n, s);
    TRY(check_launch(h));
    if (n > 0)
        CUDA_TRY(cudaMemcpyAsync(host_hits, d.hit_buf, sizeof(b3gRayHit) * (size_t)n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    return B3G_OK;
}

extern "C" b3gStatus b3g_profiler_range(int on) {
    CUDA_TRY(on ? cudaProfilerStart() : cudaProfilerStop());
    return B3G_OK;
}

extern "C" b3gStatus b3g_get_tuning(b3g_handle h, b3gTuning* out) {
    REQUIRE_UPLOADED(h);
    if (!out) return fail(B3G_ERR_INVALID_ARG, "null output");
    b3gTuning t = h->tuning;
    t.pgs_partitions = h->d.tune.pgs_partitions;
    t.pairs_blocks_per_sm = h->d.tune.pairs_blocks_per_sm;
    t.narrow_blocks_per_sm = h->d.tune.narrow_blocks_per_sm;
    t.sort_blocks_per_sm = h->d.tune.sort_blocks_per_sm;
    *out = t;
    return B3G_OK;
}

extern "C" b3gStatus b3g_setup_aabbs(b3g_handle h) {
    REQUIRE_UPLOADED(h);
    h->launches += launch_aabbs(h->d, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}
extern "C" b3gStatus b3g_calculate_overlapping_pairs(b3g_handle h) {
    REQUIRE_UPLOADED(h);
    h->launches += launch_pairs(h->d, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}
extern "C" b3gStatus b3g_compute_contacts(b3g_handle h) {
    REQUIRE_UPLOADED(h);
    h->launches += launch_contacts(h->d, h->cfg.contact_friction, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}
extern "C" b3gStatus b3g_compute_contacts_for_pairs(b3g_handle h, const void* d_pairs, int n) {
    REQUIRE_UPLOADED(h);
    if (n < 0 || (n > 0 && !d_pairs)) return fail(B3G_ERR_INVALID_ARG, "invalid pair buffer");
    if (reinterpret_cast<uintptr_t>(d_pairs) & 15u) return fail(B3G_ERR_INVALID_ARG, "pairs must be 16-byte aligned");
    CUDA_TRY(cudaSetDevice(h->device));
    h->launches += launch_pairs_external(h->d, static_cast<const b3gPair*>(d_pairs), n, h->stream);
    h->launches += launch_contacts(h->d, h->cfg.contact_friction, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}

extern "C" b3gStatus b3g_solve_joints(b3g_handle h) {
    REQUIRE_UPLOADED(h);
    TRY(prepare_joints(h));
    h->launches += launch_joints(h->d, h->cfg, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}
extern "C" b3gStatus b3g_solve_contacts(b3g_handle h, float dt) {
    REQUIRE_UPLOADED(h);
    h->launches += launch_solver(h->d, h->cfg, dt, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}
extern "C" b3gStatus b3g_integrate(b3g_handle h, float dt) {
    REQUIRE_UPLOADED(h);
    h->launches += launch_integrate(h->d, h->cfg, dt, h->stream);
    TRY(check_launch(h));
    return B3G_OK;
}
extern "C" b3gStatus b3g_synchronize(b3g_handle h) {
    REQUIRE_UPLOADED(h);
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return B3G_OK;
}

static b3gStatus read_counters(b3g_handle h, DevCounters& c) {
    CUDA_TRY(cudaMemcpyAsync(&c, h->d.counters, sizeof(DevCounters), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return B3G_OK;
}

extern "C" b3gStatus b3g_get_stats(b3g_handle h, b3gStepStats* out) {
    REQUIRE_UPLOADED(h);
    if (!out) return fail(B3G_ERR_INVALID_ARG, "null output");
    DevCounters c;
    TRY(read_counters(h, c));
    out->num_pairs = std::min(c.num_pairs, h->d.max_pairs);
    out->num_contacts = c.num_contacts;
    out->num_points = c.num_points;
    out->num_colors = c.num_colors;
    out->iterations = c.iterations;
    out->residual = c.residual;
    out->status = c.status;
    out->num_large = h->d.num_large + h->d.num_sap;
    out->num_child_pairs = h->d.num_children > 0 ? c.pad[4] : 0;
    out->num_concave_pairs = h->d.num_meshes > 0 ? c.pad[6] : 0;
    return B3G_OK;
}

extern "C" b3gStatus b3g_status(b3g_handle h, unsigned int* flags, int clear) {
    REQUIRE_UPLOADED(h);
    if (!flags) return fail(B3G_ERR_INVALID_ARG, "null output");
    DevCounters c;
    TRY(read_counters(h, c));
    *flags = c.status;
    if (clear) CUDA_TRY(cudaMemsetAsync(&h->d.counters->status, 0, sizeof(unsigned int), h->stream));
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- getters
extern "C" b3gStatus b3g_get_num_bodies(b3g_handle h, int* n) {
    if (!h || !n) return fail(B3G_ERR_INVALID_ARG, "null argument");
    *n = (int)h->bodies.size();
    return B3G_OK;
}
extern "C" b3gStatus b3g_get_body_buffer(b3g_handle h, void** p) {
    REQUIRE_UPLOADED(h);
    if (!p) return fail(B3G_ERR_INVALID_ARG, "null output");
    *p = h->d.bodies;
    return B3G_OK;
}
extern "C" b3gStatus b3g_get_inertia_buffer(b3g_handle h, void** p) {
    REQUIRE_UPLOADED(h);
    if (!p) return fail(B3G_ERR_INVALID_ARG, "null output");
    *p = h->d.inertias;
    return B3G_OK;
}
extern "C" b3gStatus b3g_get_aabb_buffer(b3g_handle h, void** p) {
    REQUIRE_UPLOADED(h);
    if (!p) return fail(B3G_ERR_INVALID_ARG, "null output");
    *p = h->d.aabbs;
    return B3G_OK;
}
extern "C" b3gStatus b3g_get_pair_buffer(b3g_handle h, void** p, int* n) {
    REQUIRE_UPLOADED(h);
    if (!p || !n) return fail(B3G_ERR_INVALID_ARG, "null output");
    DevCounters c;
    TRY(read_counters(h, c));
    *p = h->d.pairs;
    *n = std::min(c.num_pairs, h->d.max_pairs);
    return B3G_OK;
}
extern "C" b3gStatus b3g_get_contact_buffer(b3g_handle h, void** p, int* n) {
    REQUIRE_UPLOADED(h);
    if (!p || !n) return fail(B3G_ERR_INVALID_ARG, "null output");
    h->launches += launch_compact_contacts(h->d, h->stream);
    DevCounters c;
    TRY(read_counters(h, c));
    *p = h->d.contacts_compact;
    *n = c.num_contacts;
    return B3G_OK;
}
extern "C" b3gStatus b3g_get_stream(b3g_handle h, void** s) {
    REQUIRE_UPLOADED(h);
    if (!s) return fail(B3G_ERR_INVALID_ARG, "null output");
    *s = h->stream;
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- host copies
static b3gStatus copy_out(b3g_handle h, void* dst, const void* src, size_t bytes) {
    CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return B3G_OK;
}
static b3gStatus copy_in(b3g_handle h, void* dst, const void* src, size_t bytes) {
    CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_bodies(b3g_handle h, void* host, int n) {
    REQUIRE_UPLOADED(h);
    if (!host || n < 0 || n > h->d.num_bodies) return fail(B3G_ERR_INVALID_ARG, "bad body buffer");
    return copy_out(h, host, h->d.bodies, sizeof(b3gBody) * n);
}
extern "C" b3gStatus b3g_write_bodies(b3g_handle h, const void* host, int n) {
    REQUIRE_UPLOADED(h);
    if (!host || n < 0 || n > h->d.num_bodies) return fail(B3G_ERR_INVALID_ARG, "bad body buffer");
    TRY(copy_in(h, h->d.bodies, host, sizeof(b3gBody) * n));
    // a body state from the host may be anywhere: the next PGS solve colours from scratch rather
    // than carrying the last solve's colours over
    static const int recolour = 1;
    CUDA_TRY(cudaMemcpyAsync(h->d.prev_mn + 2, &recolour, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    return B3G_OK;
}
extern "C" b3gStatus b3g_read_inertias(b3g_handle h, void* host, int n) {
    REQUIRE_UPLOADED(h);
    if (!host || n < 0 || n > h->d.num_bodies) return fail(B3G_ERR_INVALID_ARG, "bad inertia buffer");
    return copy_out(h, host, h->d.inertias, sizeof(b3gInertia) * n);
}
extern "C" b3gStatus b3g_read_aabbs(b3g_handle h, void* host, int n) {
    REQUIRE_UPLOADED(h);
    if (!host || n < 0 || n > h->d.num_bodies) return fail(B3G_ERR_INVALID_ARG, "bad aabb buffer");
    return copy_out(h, host, h->d.aabbs, sizeof(b3gAabb) * n);
}
extern "C" b3gStatus b3g_write_aabbs(b3g_handle h, const void* host, int n) {
    REQUIRE_UPLOADED(h);
    if (!host || n != h->d.num_bodies) return fail(B3G_ERR_INVALID_ARG, "bad aabb buffer");
    return copy_in(h, h->d.aabbs, host, sizeof(b3gAabb) * n);
}
extern "C" b3gStatus b3g_read_pairs(b3g_handle h, void* host, int capacity, int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    DevCounters c;
    TRY(read_counters(h, c));
    int n = std::min(c.num_pairs, h->d.max_pairs);
    *num = n;
    if (host && capacity > 0) TRY(copy_out(h, host, h->d.pairs, sizeof(b3gPair) * std::min(n, capacity)));
    return B3G_OK;
}
extern "C" b3gStatus b3g_read_contacts(b3g_handle h, void* host, int capacity, int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    h->launches += launch_compact_contacts(h->d, h->stream);
    DevCounters c;
    TRY(read_counters(h, c));
    *num = c.num_contacts;
    if (host && capacity > 0)
        TRY(copy_out(h, host, h->d.contacts_compact, sizeof(b3gContact4) * std::min(c.num_contacts, capacity)));
    return B3G_OK;
}

__global__ void k_expand_contacts(const b3gContact4* __restrict__ in, int n, b3gContact4* __restrict__ slots,
                                  int* __restrict__ manifold_pair, int* __restrict__ flags, DevCounters* counters) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        slots[m] = in[m];
        manifold_pair[m] = m;
        flags[m] = 1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters->num_contacts = n;
        counters->pad[0] = n;  // every written manifold counts as a pair's (none as a compound child pair's)
    }
}

extern "C" b3gStatus b3g_write_contacts(b3g_handle h, const void* host, int n) {
    REQUIRE_UPLOADED(h);
    if (!host || n < 0 || n > h->d.max_contacts) return fail(B3G_ERR_INVALID_ARG, "bad contact buffer");
    if (n > 0) TRY(copy_in(h, h->d.contacts_compact, host, sizeof(b3gContact4) * n));
    k_expand_contacts<<<h->d.num_sms * 2, 256, 0, h->stream>>>(h->d.contacts_compact, n, h->d.contact_slots,
                                                              h->d.manifold_pair, h->d.contact_flag, h->d.counters);
    h->launches++;
    TRY(check_launch(h));
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_batches(b3g_handle h, int* host, int capacity, int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    DevCounters c;
    TRY(read_counters(h, c));
    *num = c.num_contacts;
    if (host && capacity > 0)
        TRY(copy_out(h, host, h->d.manifold_color, sizeof(int) * std::min(c.num_contacts, capacity)));
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_solve_order(b3g_handle h, int* host, int capacity, int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    DevCounters c;
    TRY(read_counters(h, c));
    *num = c.num_contacts;
    if (!host || capacity <= 0 || c.num_contacts == 0) return B3G_OK;
    const int n = std::min(c.num_contacts, capacity);
    if (h->cfg.solver_mode != B3G_SOLVER_PGS) {  // Jacobi: order-independent, manifold order
        for (int m = 0; m < n; m++) host[m] = m;
        return B3G_OK;
    }
    // the PGS kernel's processing order: groups by key, then the colour-overflow leftovers
    return copy_out(h, host, h->d.color_order, sizeof(int) * n);
}

__global__ void k_gather_impulses(const float4* __restrict__ imp, int n, float* __restrict__ out) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        for (int j = 0; j < 4; j++) {
            float4 v = imp[(size_t)m * 4 + j];
            out[(size_t)m * 12 + 3 * j + 0] = v.x;  // normal
            out[(size_t)m * 12 + 3 * j + 1] = v.z;  // lateral dir 1
            out[(size_t)m * 12 + 3 * j + 2] = v.y;  // lateral dir 2
        }
    }
}

extern "C" b3gStatus b3g_read_impulses(b3g_handle h, float* host, int capacity, int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    DevCounters c;
    TRY(read_counters(h, c));
    *num = c.num_contacts;
    int n = std::min(c.num_contacts, capacity);
    if (host && n > 0) {
        float* tmp = nullptr;
        CUDA_TRY(cudaMalloc(&tmp, sizeof(float) * 12 * (size_t)n));
        k_gather_impulses<<<h->d.num_sms * 2, 256, 0, h->stream>>>(h->d.sp.imp, n, tmp);
        b3gStatus st = copy_out(h, host, tmp, sizeof(float) * 12 * (size_t)n);
        cudaFree(tmp);
        return st;
    }
    return B3G_OK;
}

extern "C" b3gStatus b3g_get_num_collidables(b3g_handle h, int* n) {
    if (!h || !n) return fail(B3G_ERR_INVALID_ARG, "null argument");
    *n = (int)h->collidables.size();
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_registered_bodies(b3g_handle h, void* bodies, void* inertias, int n) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (n < 0 || n > (int)h->bodies.size()) return fail(B3G_ERR_INVALID_ARG, "bad body count");
    if (bodies && n) std::memcpy(bodies, h->bodies.data(), sizeof(b3gBody) * n);
    if (inertias && n) std::memcpy(inertias, h->inertias.data(), sizeof(b3gInertia) * n);
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_shape_tables(b3g_handle h, void* collidables, void* hulls, void* faces, int* indices,
                                           void* vertices, void* edges, void* local_aabbs, int* counts6) {
    if (!h || !counts6) return fail(B3G_ERR_INVALID_ARG, "null argument");
    int caps[6];
    std::memcpy(caps, counts6, sizeof(caps));
    counts6[0] = (int)h->collidables.size();
    counts6[1] = (int)h->hulls.size();
    counts6[2] = (int)h->faces.size();
    counts6[3] = (int)h->indices.size();
    counts6[4] = (int)h->vertices.size();
    counts6[5] = (int)h->edges.size();
    auto cp = [&](void* dst, const void* src, size_t esz, int n, int cap) {
        if (dst && n > 0 && cap >= n) std::memcpy(dst, src, esz * n);
    };
    cp(collidables, h->collidables.data(), sizeof(b3gCollidable), counts6[0], caps[0]);
    cp(local_aabbs, h->local_aabbs.data(), sizeof(b3gAabb), counts6[0], caps[0]);
    cp(hulls, h->hulls.data(), sizeof(b3gHull), counts6[1], caps[1]);
    cp(faces, h->faces.data(), sizeof(b3gFace), counts6[2], caps[2]);
    cp(indices, h->indices.data(), sizeof(int), counts6[3], caps[3]);
    cp(vertices, h->vertices.data(), sizeof(b3gFloat4), counts6[4], caps[4]);
    cp(edges, h->edges.data(), sizeof(b3gFloat4), counts6[5], caps[5]);
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- profiling
extern "C" b3gStatus b3g_set_profiling(b3g_handle h, int on) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    if (on && !h->events.created) {
        CUDA_TRY(cudaSetDevice(h->device));
        for (auto& e : h->events.ev) CUDA_TRY(cudaEventCreate(&e));
        h->events.created = true;
    }
    h->profiling = on != 0;
    return B3G_OK;
}

extern "C" b3gStatus b3g_get_stage_times(b3g_handle h, float* ms7) {
    REQUIRE_UPLOADED(h);
    if (!ms7) return fail(B3G_ERR_INVALID_ARG, "null output");
    if (!h->events.created) return fail(B3G_ERR_INVALID_ARG, "profiling was never enabled");
    CUDA_TRY(cudaEventSynchronize(h->events.ev[7]));
    for (int k = 0; k < 7; k++) {
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, h->events.ev[k], h->events.ev[k + 1]));
        ms7[k] = ms;
    }
    return B3G_OK;
}

extern "C" b3gStatus b3g_get_launch_count(b3g_handle h, long long* n) {
    if (!h || !n) return fail(B3G_ERR_INVALID_ARG, "null argument");
    *n = h->launches;
    return B3G_OK;
}

extern "C" b3gStatus b3g_record_event(b3g_handle h, int slot) {
    REQUIRE_UPLOADED(h);
    if (slot < 0 || slot >= 16) return fail(B3G_ERR_INVALID_ARG, "event slot out of range");
    if (!h->user_events[slot]) CUDA_TRY(cudaEventCreate(&h->user_events[slot]));
    CUDA_TRY(cudaEventRecord(h->user_events[slot], h->stream));
    return B3G_OK;
}

extern "C" b3gStatus b3g_event_elapsed(b3g_handle h, int a, int b, float* ms) {
    REQUIRE_UPLOADED(h);
    if (!ms || a < 0 || a >= 16 || b < 0 || b >= 16 || !h->user_events[a] || !h->user_events[b])
        return fail(B3G_ERR_INVALID_ARG, "event slots not recorded");
    CUDA_TRY(cudaEventSynchronize(h->user_events[b]));
    CUDA_TRY(cudaEventElapsedTime(ms, h->user_events[a], h->user_events[b]));
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- hull (host only)
extern "C" b3gStatus b3g_hull_compute(const float* verts, int stride_bytes, int num_verts, const float scaling[3],
                                      float* verts_out, float* planes_out, int* face_counts_out, int* indices_out,
                                      float* edges_out, float* center_out, int* counts6) {
    if (!verts || !counts6) return fail(B3G_ERR_INVALID_ARG, "null argument");
    HullTables t;
    if (build_hull(verts, stride_bytes, num_verts, scaling, t) != 0)
        return fail(B3G_ERR_DEGENERATE, "degenerate convex hull input (%d points)", num_verts);
    int nv = (int)t.vertices.size() / 3, nf = (int)t.face_counts.size(), ni = (int)t.indices.size(),
        ne = (int)t.edges.size() / 3;
    bool fits = counts6[0] >= nv && counts6[1] >= nf && counts6[2] >= ni && counts6[3] >= ne;
    counts6[0] = nv;
    counts6[1] = nf;
    counts6[2] = ni;
    counts6[3] = ne;
    if (!fits) return fail(B3G_ERR_CAPACITY, "hull output buffers too small");
    if (verts_out) std::memcpy(verts_out, t.vertices.data(), sizeof(float) * 3 * nv);
    if (planes_out) std::memcpy(planes_out, t.planes.data(), sizeof(float) * 4 * nf);
    if (face_counts_out) std::memcpy(face_counts_out, t.face_counts.data(), sizeof(int) * nf);
    if (indices_out) std::memcpy(indices_out, t.indices.data(), sizeof(int) * ni);
    if (edges_out && ne) std::memcpy(edges_out, t.edges.data(), sizeof(float) * 3 * ne);
    if (center_out) std::memcpy(center_out, t.center, sizeof(float) * 3);
    return B3G_OK;
}

// ---------------------------------------------------------------------------------- device buffers
extern "C" b3gStatus b3g_buffer_alloc(int cuda_device, size_t bytes, void** out) {
    if (!out) return fail(B3G_ERR_INVALID_ARG, "null output");
    *out = nullptr;
    CUDA_TRY(cudaSetDevice(cuda_device));
    if (bytes == 0) return B3G_OK;
    CUDA_TRY(cudaMalloc(out, bytes));
    return B3G_OK;
}

extern "C" b3gStatus b3g_buffer_free(int cuda_device, void* p) {
    if (!p) return B3G_OK;
    CUDA_TRY(cudaSetDevice(cuda_device));
    CUDA_TRY(cudaFree(p));
    return B3G_OK;
}

extern "C" b3gStatus b3g_buffer_copy(int cuda_device, void* dst, const void* src, size_t bytes, int kind) {
    if (bytes == 0) return B3G_OK;
    if (!dst || !src) return fail(B3G_ERR_INVALID_ARG, "null buffer");
    const cudaMemcpyKind k = kind == B3G_COPY_H2D   ? cudaMemcpyHostToDevice
                             : kind == B3G_COPY_D2H ? cudaMemcpyDeviceToHost
                             : kind == B3G_COPY_D2D ? cudaMemcpyDeviceToDevice
                                                    : cudaMemcpyDefault;
    if (k == cudaMemcpyDefault) return fail(B3G_ERR_INVALID_ARG, "unknown copy kind %d", kind);
    CUDA_TRY(cudaSetDevice(cuda_device));
    CUDA_TRY(cudaMemcpy(dst, src, bytes, k));
    return B3G_OK;
}

// ------------------------------------------------------------------ allocation-free broadphase
// Per device: the static scratch array's address and the SM count, looked up on the first call
// with that device current.
namespace {
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
void* g_na_scratch[NA_MAX_DEVICES] = {};
int g_na_sms[NA_MAX_DEVICES] = {};
}  // namespace

extern "C" b3gStatus b3g_grid_pairs_noalloc(const void* d_aabbs, int n, float cell_size, int grid_dim, void* d_pairs,
                                            int max_pairs, int* d_num_pairs, void* cuda_stream) {
    if (n < 0 || n > B3G_NOALLOC_MAX_AABBS)
        return fail(B3G_ERR_CAPACITY, "n = %d outside 0..%d (B3G_NOALLOC_MAX_AABBS)", n, B3G_NOALLOC_MAX_AABBS);
    if (max_pairs < 1 || max_pairs > B3G_NOALLOC_MAX_PAIRS)
        return fail(B3G_ERR_CAPACITY, "max_pairs = %d outside 1..%d (B3G_NOALLOC_MAX_PAIRS)", max_pairs,
                    B3G_NOALLOC_MAX_PAIRS);
    if (grid_dim < 4 || grid_dim > B3G_NOALLOC_MAX_GRID_DIM || (grid_dim & (grid_dim - 1)))
        return fail(B3G_ERR_CAPACITY, "grid_dim = %d: needs a power of two in 4..%d (B3G_NOALLOC_MAX_GRID_DIM)",
                    grid_dim, B3G_NOALLOC_MAX_GRID_DIM);
    if (!(cell_size > 0.f) || !std::isfinite(cell_size))
        return fail(B3G_ERR_INVALID_ARG, "cell_size must be positive and finite");
    if ((n > 0 && !d_aabbs) || !d_pairs || !d_num_pairs) return fail(B3G_ERR_INVALID_ARG, "null device buffer");
    if (reinterpret_cast<uintptr_t>(d_aabbs) % 16 != 0)
        return fail(B3G_ERR_INVALID_ARG, "d_aabbs must be 16-byte aligned");
    int dev = -1;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NA_MAX_DEVICES) return fail(B3G_ERR_UNSUPPORTED, "device index %d not supported", dev);
    void* scratch = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_scratch[dev]) {  // first call on this device: one-time lookups
            int s = 0;
            CUDA_TRY(cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev));
            if (s < 1 || s * 4 > B3G_NOALLOC_MAX_SORT_BLOCKS)
                return fail(B3G_ERR_UNSUPPORTED, "%d SMs: the static sort scratch covers at most %d", s,
                            B3G_NOALLOC_MAX_SORT_BLOCKS / 4);
            void* p = nullptr;
            CUDA_TRY(noalloc_scratch_address(&p));
            if (!p) return fail(B3G_ERR_CUDA, "cudaGetSymbolAddress returned a null scratch address");
            g_na_sms[dev] = s;
            g_na_scratch[dev] = p;
        }
        scratch = g_na_scratch[dev];
        sms = g_na_sms[dev];
    }
    int bits = 1;
    while ((1 << bits) < grid_dim) bits++;
    int body_bits = 1;
    while ((1 << body_bits) < n + 1) body_bits++;
    launch_grid_pairs_noalloc(scratch, sms, static_cast<const b3gAabb*>(d_aabbs), n, 1.f / cell_size, bits,
                              body_bits, static_cast<b3gPair*>(d_pairs), max_pairs, d_num_pairs,
                              static_cast<cudaStream_t>(cuda_stream));
    CUDA_TRY(cudaPeekAtLastError());
    return B3G_OK;
}

// ------------------------------------------------------------------ learned warm start
extern "C" b3gStatus b3g_set_warm_start_model(b3g_handle h, b3g_mlp m) {
    if (!h) return fail(B3G_ERR_INVALID_ARG, "null handle");
    mlp::Model* model = b3g_mlp_model(m);
    if (model && model->device != h->device) return fail(B3G_ERR_INVALID_ARG, "network and world on different devices");
    h->ws_mlp = m;
    if (h->uploaded) {
        CUDA_TRY(cudaSetDevice(h->device));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        h->d.ws_model = h->d.ws_features ? model : nullptr;
        if (h->d.ws_model) CUDA_TRY(mlp::ensure_infer(*h->d.ws_model, h->d.ws_rows_cap));
        CUDA_TRY(cudaSetDevice(h->device));
        drop_graphs(h);  // the captured step has (or lacks) the network's launches
    }
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_warm_samples(b3g_handle h, float* features, float* targets, int* is_new, int capacity,
                                           int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    if (!h->d.ws_features) return fail(B3G_ERR_INVALID_ARG, "warm_start records no features (LEARNED, RECORD or PERSISTENT_LEARNED do)");
    DevCounters c;
    TRY(read_counters(h, c));
    const int nc = c.num_contacts;
    const int slots = std::min(4 * nc, h->d.ws_rows_cap);
    std::vector<float> f((size_t)slots * 12);
    std::vector<float4> imp(slots);
    std::vector<int4> hdr(nc);
    std::vector<unsigned char> fresh(slots);
    if (slots > 0) {
        TRY(copy_out(h, f.data(), h->d.ws_features, sizeof(float) * f.size()));
        TRY(copy_out(h, imp.data(), h->d.sp.imp, sizeof(float4) * imp.size()));
        TRY(copy_out(h, hdr.data(), h->d.manifold_hdr, sizeof(int4) * hdr.size()));
        TRY(copy_out(h, fresh.data(), h->d.ws_new, fresh.size()));
    }
    int n = 0;
    for (int s = 0; s < slots; s++) {
        if (!((hdr[s / 4].z >> (s % 4)) & 1)) continue;
        if (n < capacity && features && targets) {
            std::memcpy(features + (size_t)n * 12, f.data() + (size_t)s * 12, sizeof(float) * 12);
            targets[(size_t)n * 3 + 0] = imp[s].x;
            targets[(size_t)n * 3 + 1] = imp[s].y;
            targets[(size_t)n * 3 + 2] = imp[s].z;
            if (is_new) is_new[n] = fresh[s];
        }
        n++;
    }
    *num = n;
    return B3G_OK;
}

extern "C" b3gStatus b3g_read_warm_start(b3g_handle h, float* host, int capacity, int* num) {
    REQUIRE_UPLOADED(h);
    if (!num) return fail(B3G_ERR_INVALID_ARG, "null count");
    DevCounters c;
    TRY(read_counters(h, c));
    *num = c.num_contacts;
    if (!host || capacity <= 0) return B3G_OK;
    const int nm = std::min(c.num_contacts, capacity);
    std::memset(host, 0, sizeof(float) * 12 * (size_t)nm);
    if (!h->d.ws_init) return B3G_OK;
    const int slots = std::min(4 * nm, h->d.ws_rows_cap);
    std::vector<float4> w(slots);
    if (slots > 0) TRY(copy_out(h, w.data(), h->d.ws_init, sizeof(float4) * w.size()));
    for (int s = 0; s < slots; s++) {
        float* o = host + (size_t)(s / 4) * 12 + 3 * (s % 4);
        o[0] = w[s].x;  // contact
        o[1] = w[s].z;  // lateral 1 = first friction direction
        o[2] = w[s].y;  // lateral 2 = second friction direction
    }
    return B3G_OK;
}
