// Contact solver: b3PgsJacobiSolver semantics on the GPU.
//
// Reference (paths relative to the reference's src/Bullet3Dynamics/ConstraintSolver/):
//   solveGroup                       b3PgsJacobiSolver.cpp:170-189
//   per-body split counts (Jacobi)   :1020-1042
//   convertContact                   :847-983   (2 friction directions, velocity dependent, no caching)
//   setupContactConstraint           :654-804   (erp 0.2, no split impulse, restitution 0, cold start)
//   setupFrictionConstraint          :457-536
//   solveSingleIteration             :1281-1486 (all contact rows, [Jacobi: average], all friction rows)
//   resolveSingleConstraintRowLowerLimit / Generic :236-317 (scalar path; USE_SIMD is not defined in Bullet3)
//   averageVelocities                :1552-1587
//   solveGroupCacheFriendlyFinish    :1589-1691 (PGS: v += dv; Jacobi: v += (S/count) once per split copy)
//
// GB300 design: compact per-point records are built one thread per manifold; the iterations run
// in ONE cooperative persistent kernel with a bounded grid barrier.  A manifold's whole working
// set (normal, up to 4 points, both inverse inertias, both body deltas) is loaded up front so the
// per-manifold latency is one memory round trip, not one per row.
//   PGS    : dynamic bodies are split into one contiguous range of the broadphase's cell order per
//            block.  Manifolds inside one range are solved by that block alone (shared-memory body
//            deltas, __syncthreads between colours); the rest run grid-wide with one grid barrier
//            per colour.  Both sets are Jones-Plassmann greedy coloured (a manifold holding the
//            highest hashed priority on both of its dynamic bodies takes the smallest colour free
//            on both, exact per-body 64-bit masks) and counting-sorted by (owner, colour).
//   Jacobi : per iteration: contact rows of every manifold on its own split copies, a per-body
//            ordered reduction (same summation order as the reference's solver-body pool), friction
//            rows, reduction.  Per-body lists come from a stable radix sort, so the arithmetic
//            matches the sequential reference order bit for bit.
#include <cfloat>

#include "common.cuh"
#include "warmstart.h"
#include "world_internal.h"

namespace b3g {

static constexpr int SV_THREADS = 256;   // setup kernels
static constexpr int PK_THREADS = 512;   // persistent solver kernels: one block per SM, 16 warps
static constexpr float LARGE_UPPER = 1e10f;

struct SolverArgs {
    const b3gBody* bodies;
    const b3gInertia* inertias;
    const b3gContact4* slots;
    const int* manifold_pair;
    const int* d_npairs;      // slots below this hold pairs' manifolds, the rest compound child pairs'
    const int* d_nc;          // number of manifolds
    SolverPoints sp;
    SolverPoints sp_ord;      // PGS: the same records in colour order
    int4* hdr;                // bodyA, bodyB, active point mask, num points
    float2* inv_mass;         // invMass A, B
    int4* hdr_ord;            // PGS: colour-ordered copies
    float4* inv_mass_ord;     // (invMass A, invMass B, 0, 0): 16 B so tiles copy in bulk
    float4* inertia_ord;      // PGS: per ordered manifold both bodies' inverse world inertia rows (6 float4)
    float4* dv;               // per body: [2b] lin, [2b+1] ang (PGS, and Jacobi averaged delta)
    float4* dv_sum;           // Jacobi: per body sum of split deltas from the last averaging
    float4* split;            // Jacobi: per manifold 4 float4: A lin, A ang, B lin, B ang
    const int* body_count;    // Jacobi split counts (manifolds per dynamic body)
    const int* list_off;      // Jacobi per-body list offsets (exclusive scan of counts)
    const uint32_t* list;     // Jacobi: entries 2*m+side grouped by body, in manifold order
    int* color;               // per manifold
    int* color_order;
    int* color_offsets;       // B3G_MAX_COLORS + 2
    int* color_fill;          // B3G_MAX_COLORS + 1: manifolds per colour
    int* color_cursor;        // B3G_MAX_COLORS + 1: scatter cursors for the counting sort
    int* remaining;           // per round
    const uint32_t* sorted_bodies;  // PGS: dynamic bodies in broadphase cell order (block partitions)
    int* body_slot;           // PGS: body -> position in sorted_bodies
    int* manifold_group;      // PGS: processing group of each manifold
    int* group_counts;        // PGS: 3 segments of group_seg ints: counts, offsets, cursors
    int group_seg;
    int num_dynamic;          // length of sorted_bodies (0: every manifold is cross-partition)
    int chunk;                // dynamic bodies per block partition
    int use_smem;             // block-local body deltas in shared memory
    int tile_R;               // > 0: block-local records streamed through shared memory, R per tile
    int interleave;           // PGS: each point's friction rows right after its contact row
    float* ws_features;       // learned warm start: 12 features per point slot 4m+j (nullptr: none)
    int ws_rows_cap;          // point slots that get features
    int* ws_rows;             // device: min(4 * manifolds, ws_rows_cap)
    float gx, gy, gz;         // gravity (the dt * (g . n) feature)
    int warm;                 // PGS: the records' initial impulses are a warm start (apply, then iterate)
    unsigned long long* claim;
    unsigned long long* mask;  // per body: colours already taken by its manifolds
    unsigned long long* claim_x;  // PGS: the same two arrays for the cross-partition colouring
    unsigned long long* mask_x;
    b3gBody* bodies_out;      // velocities written at finish
    DevCounters* counters;
    double* residual_acc;     // 2 per iteration
    int num_bodies;
    int mode;
    int iterations;
    float residual_tol;
    float dt;
    float erp;
    float threshold;
    GridBarrier bar;
    unsigned int spin_limit;
    // PGS in colour order from the setup on (k_manifold_prep / k_colour / k_pgs_sweeps)
    int* pos_of;                  // manifold -> position in colour order (nullptr: the in-kernel path)
    unsigned long long* prev_key; // last solve's manifold keys (ascending) and colours
    int* prev_color;
    int* d_prev_n;
    int* d_new;                   // manifolds without a carried colour
    int* color_goff;              // colour offsets of the ordered records: [c] start, [65] total
    int body_bits;
    int tail_max;                 // trailing colours of at most this many manifolds run in one block
    GridBarrier bar2;             // barrier of k_colour (separate counters from the sweeps')
    unsigned long long* flow_mask;  // per body: the colours of its manifolds (exact, from k_colour)
    unsigned int* version;        // per body: manifold updates applied so far in this solve (k_pgs_flow)
};

// b3PlaneSpace1 (Bullet3Common/b3Vector3.h:1184-1212)
__device__ __forceinline__ void plane_space(v3 n, v3& p, v3& q) {
    if (fabsf(n.z) > 0.7071067811865475244008443621048490f) {
        float a = n.y * n.y + n.z * n.z;
        float k = 1.0f / sqrtf(a);
        p = mk3(0.f, -n.z * k, n.y * k);
        q = mk3(a * k, -n.x * p.z, n.x * p.y);
    } else {
        float a = n.x * n.x + n.y * n.y;
        float k = 1.0f / sqrtf(a);
        p = mk3(-n.y * k, n.x * k, 0.f);
        q = mk3(-n.z * p.y, n.z * p.x, a * k);
    }
}

__device__ __forceinline__ float4 f4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ float4 f4v(b3gFloat4 r) { return make_float4(r.x, r.y, r.z, r.w); }
__device__ __forceinline__ v3 xyz(float4 a) { return mk3(a.x, a.y, a.z); }

// Jacobi split counts: number of manifolds touching each dynamic body.
__global__ void k_count_manifolds(const b3gContact4* __restrict__ slots, const int* __restrict__ manifold_pair,
                                  const int* __restrict__ d_nc, const b3gBody* __restrict__ bodies,
                                  int* __restrict__ body_count, uint32_t* __restrict__ keys,
                                  uint32_t* __restrict__ vals, uint32_t sentinel, int* __restrict__ d_n2) {
    const int nc = *d_nc;
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_n2 = 2 * nc;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nc; m += gridDim.x * blockDim.x) {
        const b3gContact4& c = slots[manifold_pair[m]];
        int a = abs(c.bodyA), b = abs(c.bodyB);
        bool da = bodies[a].invMass != 0.f, db = bodies[b].invMass != 0.f;
        if (da) atomicAdd(&body_count[a], 1);
        if (db) atomicAdd(&body_count[b], 1);
        keys[2 * m] = da ? (uint32_t)a : sentinel;
        vals[2 * m] = 2u * m;
        keys[2 * m + 1] = db ? (uint32_t)b : sentinel;
        vals[2 * m + 1] = 2u * m + 1u;
    }
}

// Row setup: setupContactConstraint + convertContact friction rows, stored as compact records.
// One thread per contact point (the 4 point slots of a manifold are 4 consecutive lanes of a
// warp): the point's contact row and two friction rows; lane 0 of the 4 writes the manifold's
// header with the point mask (a ballot over the 4).
__global__ void __launch_bounds__(SV_THREADS, 3) k_setup_rows(SolverArgs a) {
    const int nc = *a.d_nc;
    const bool pgs = a.mode == B3G_SOLVER_PGS;
    if (a.ws_rows && blockIdx.x == 0 && threadIdx.x == 0) *a.ws_rows = min(4 * nc, a.ws_rows_cap);
    const bool ordered = a.pos_of != nullptr;  // records straight into colour order
    SolverPoints& out = ordered ? a.sp_ord : a.sp;
    const int total = 4 * nc;
    const int lane = threadIdx.x & 31;
    // (warp-uniform loop: every lane reaches the ballot)
    for (int base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const int t = base + (int)threadIdx.x;
        const int k = t >> 2, j = t & 3;  // record slot (ordered: record i holds manifold color_order[i])
        bool active = false;
        int m = 0, iA = 0, iB = 0, np = 0;
        float imA = 0.f, imB = 0.f;
        v3 n = mk3(0.f, 0.f, 0.f);
        float fric = 0.f;
        if (t < total) {
            m = ordered ? __ldcg(&a.color_order[k]) : k;
            const b3gContact4* cp = a.slots + a.manifold_pair[m];
            const float4 nw = ldg4(&cp->worldNormalOnB);
            const int4 ids = __ldg(reinterpret_cast<const int4*>(&cp->worldNormalOnB) + 1);  // cmp, batch, A, B
            iA = abs(ids.z);
            iB = abs(ids.w);
            const float4* bA = reinterpret_cast<const float4*>(a.bodies + iA);
            const float4* bB = reinterpret_cast<const float4*>(a.bodies + iB);
            imA = __ldg(&bA[4]).y;
            imB = __ldg(&bB[4]).y;
            np = (int)nw.w;
            if (np > 4) np = 4;
            if (imA == 0.f && imB == 0.f) np = 0;  // static-static: no rows (b3PgsJacobiSolver.cpp:864-866)
            fric = (float)((unsigned)ids.x >> 16) / (float)0xffff;
            // getContactPoint: normalised normal
            n = normalize3(mk3(nw.x, nw.y, nw.z));
            const float4 wp = j < np ? ldg4(&cp->worldPosB[j]) : make_float4(0.f, 0.f, 0.f, 1e30f);
            const float dist = wp.w;
            active = j < np && dist <= a.threshold;
            if (active) {
                const size_t s = (size_t)k * 4 + j;     // record slot of the point
                const size_t sf = (size_t)m * 4 + j;    // feature slot (manifold order)
                const b3gMat3 IA = a.inertias[iA].invInertiaWorld;
                const b3gMat3 IB = a.inertias[iB].invInertiaWorld;
                const float4 pA = __ldg(&bA[0]), lA = __ldg(&bA[2]), wA = __ldg(&bA[3]);
                const float4 pB = __ldg(&bB[0]), lB = __ldg(&bB[2]), wB = __ldg(&bB[3]);
                const v3 posA = mk3(pA.x, pA.y, pA.z), posB = mk3(pB.x, pB.y, pB.z);
                const v3 linA = mk3(lA.x, lA.y, lA.z), angA = mk3(wA.x, wA.y, wA.z);
                const v3 linB = mk3(lB.x, lB.y, lB.z), angB = mk3(wB.x, wB.y, wB.z);
                float countA = 1.f, countB = 1.f;
                if (!pgs) {
                    if (imA != 0.f) countA = (float)a.body_count[iA];
                    if (imB != 0.f) countB = (float)a.body_count[iB];
                }
                const v3 pos2 = mk3(wp.x, wp.y, wp.z);
                const v3 pos1 = pos2 + n * dist;
                const v3 rel1 = pos1 - posA;
                const v3 rel2 = pos2 - posB;
                v3 ang[6];  // angular components: contact A / B, dir2 A / B, dir1 A / B
                // contact row (setupContactConstraint)
                {
                    v3 torqueAxis0 = cross3(rel1, n);
                    v3 angCompA = imul(IA, torqueAxis0);
                    v3 torqueAxis1 = cross3(rel2, n);
                    v3 angCompB = imul(IB, -torqueAxis1);
                    float denom0 = imA + dot3(n, cross3(angCompA, rel1));
                    float denom1 = imB + dot3(n, cross3(-angCompB, rel2));
                    float jac = 1.0f / (denom0 + denom1);
                    float scaled = pgs ? jac : 1.0f / (denom0 * countA + denom1 * countB);
                    v3 r1xn = torqueAxis0, r2xn = -torqueAxis1;
                    float penetration = dist + 0.0f;
                    float vel1Dotn = dot3(n, linA) + dot3(r1xn, angA);
                    float vel2Dotn = -dot3(n, linB) + dot3(r2xn, angB);
                    float rel_vel = vel1Dotn + vel2Dotn;
                    float positionalError = 0.f;
                    float velocityError = 0.0f - rel_vel;
                    if (penetration > 0.f)
                        velocityError -= penetration / a.dt;
                    else
                        positionalError = -penetration * a.erp / a.dt;
                    float rhs = positionalError * scaled + velocityError * scaled;
                    out.rel1[s] = f4(rel1, jac);
                    out.rel2[s] = f4(rel2, rhs);
                    ang[0] = angCompA;
                    ang[1] = angCompB;
                }
                // friction rows (convertContact: dir2 row first, then dir1)
                {
                    v3 vel1 = linA + cross3(angA, rel1);
                    v3 vel2 = linB + cross3(angB, rel2);
                    v3 vel = vel1 - vel2;
                    float rel_vel = dot3(n, vel);
                    v3 dir1 = vel - n * rel_vel;
                    float lat = dot3(dir1, dir1);
                    v3 dir2;
                    if (lat > FLT_EPSILON) {
                        float inv = 1.f / sqrtf(lat);
                        dir1 = dir1 * inv;
                        dir2 = cross3(dir1, n);
                        float l2 = sqrtf(dot3(dir2, dir2));
                        dir2 = dir2 * (1.f / l2);
                    } else {
                        plane_space(n, dir1, dir2);
                    }
                    v3 dirs[2] = {dir2, dir1};
                    float jacs[2], rhss[2];
                    for (int r = 0; r < 2; r++) {
                        v3 d = dirs[r];
                        v3 r1xn = cross3(rel1, d);
                        v3 angCompA = imul(IA, r1xn);
                        v3 r2xn = cross3(rel2, -d);
                        v3 angCompB = imul(IB, r2xn);
                        float denom0 = imA + dot3(d, cross3(angCompA, rel1));
                        float denom1 = imB + dot3(d, cross3(-angCompB, rel2));
                        float jac = 1.0f / (denom0 + denom1);
                        float scaled = pgs ? jac : 1.0f / (denom0 * countA + denom1 * countB);
                        float v1 = dot3(d, linA) + dot3(r1xn, angA);
                        float v2 = -dot3(d, linB) + dot3(r2xn, angB);
                        float rv = v1 + v2;
                        float velocityError = 0.0f - rv;
                        jacs[r] = jac;
                        rhss[r] = velocityError * scaled;
                        ang[2 + 2 * r] = angCompA;
                        ang[3 + 2 * r] = angCompB;
                    }
                    out.dir2[s] = f4(dir2, jacs[0]);
                    out.dir1[s] = f4(dir1, jacs[1]);
                    out.rhsf[s] = make_float2(rhss[0], rhss[1]);
                    out.imp[s] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (ordered) {
                        // the sweeps' angular components, computed above with their operations
                        out.angP[s] = make_float4(ang[0].x, ang[0].y, ang[0].z, ang[2].x);
                        out.angQ[s] = make_float4(ang[1].x, ang[1].y, ang[1].z, ang[2].y);
                        out.angR[s] = make_float4(ang[2].z, ang[3].x, ang[3].y, ang[3].z);
                        out.angS[s] = make_float4(ang[4].x, ang[4].y, ang[4].z, ang[5].x);
                        out.angT[s] = make_float2(ang[5].y, ang[5].z);
                    }
                    if (a.ws_features && sf < (size_t)a.ws_rows_cap) {
                        // warm-start features of this point (the network's input layout)
                        float* f = a.ws_features + sf * 12;
                        f[0] = vel.x; f[1] = vel.y; f[2] = vel.z;
                        f[3] = n.x; f[4] = n.y; f[5] = n.z;
                        f[6] = dist;
                        f[7] = imA; f[8] = imB;
                        f[9] = (float)np;
                        f[10] = sqrtf(lat);
                        f[11] = a.dt * (a.gx * n.x + a.gy * n.y + a.gz * n.z);
                    }
                }
            }
        }
        const int mask = (int)(__ballot_sync(0xffffffffu, active) >> (lane & 28)) & 15;
        if (t >= total || j != 0) continue;
        // the manifold: normal + friction, inverse masses, header
        out.nf[k] = f4(n, fric);
        if (!ordered) {
            a.color[m] = -1;
            a.inv_mass[m] = make_float2(imA, imB);
            a.hdr[m] = make_int4(iA, iB, mask, np);
            continue;
        }
        a.inv_mass_ord[k] = make_float4(imA, imB, 0.f, 0.f);
        // the dataflow sweeps' per-body update numbers, packed: for each dynamic body its
        // manifolds' colour count (7 bits) and the rank of this manifold's colour among them
        // (6 bits); A in the low 13 bits, B in the next 13
        unsigned flow = 0;
        if (a.flow_mask) {
            const int c = __ldcg(&a.color[m]);
            if (c >= 0) {
                const unsigned long long below = (1ull << c) - 1ull;
                if (imA != 0.f) {
                    const unsigned long long cm = __ldcg(&a.flow_mask[iA]);
                    flow |= (unsigned)__popcll(cm) | ((unsigned)__popcll(cm & below) << 7);
                }
                if (imB != 0.f) {
                    const unsigned long long cm = __ldcg(&a.flow_mask[iB]);
                    flow |= ((unsigned)__popcll(cm) | ((unsigned)__popcll(cm & below) << 7)) << 13;
                }
            }
        }
        a.hdr_ord[k] = make_int4(iA, iB, mask, (int)flow);
    }
}

// One row (resolveSingleConstraintRowLowerLimit / Generic): returns the new applied impulse.
template <bool FRICTION>
__device__ __forceinline__ float solve_row(v3 d, float jac, float rhs, float applied, v3 r1xn, v3 r2xn, v3 angA,
                                           v3 angB, float lower, float upper, v3& dlA, v3& daA, v3& dlB, v3& daB,
                                           float imA, float imB) {
    float deltaImpulse = rhs - applied * 0.0f;
    float dv1 = dot3(d, dlA) + dot3(r1xn, daA);
    float dv2 = -dot3(d, dlB) + dot3(r2xn, daB);
    deltaImpulse -= dv1 * jac;
    deltaImpulse -= dv2 * jac;
    float sum = applied + deltaImpulse;
    if (sum < lower) {
        deltaImpulse = lower - applied;
        applied = lower;
    } else if (FRICTION && sum > upper) {
        deltaImpulse = upper - applied;
        applied = upper;
    } else {
        applied = sum;
    }
    dlA = dlA + (d * imA) * deltaImpulse;
    daA = daA + angA * deltaImpulse;
    dlB = dlB + ((-d) * imB) * deltaImpulse;
    daB = daB + angB * deltaImpulse;
    return applied;
}

__device__ __forceinline__ b3gMat3 ld_mat(const b3gMat3* p) {
    b3gMat3 r;
    const float4* q = reinterpret_cast<const float4*>(p);
    float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    r.row[0] = b3gFloat4{a.x, a.y, a.z, a.w};
    r.row[1] = b3gFloat4{b.x, b.y, b.z, b.w};
    r.row[2] = b3gFloat4{c.x, c.y, c.z, c.w};
    return r;
}

// ---- bulk asynchronous copies (TMA, untiled) into shared memory, completed on an mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// global -> shared, `bytes` a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase with the given parity; false after `limit` polls
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, unsigned limit) {
    for (unsigned i = 0; i < limit; i++) {
        if (mbar_test(bar, parity)) return true;
        __nanosleep(20);
    }
    return false;
}
// generic-proxy accesses before async-proxy (bulk copy) accesses of the same memory
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Record loads: from shared memory (a streamed tile) or through L2 (ld.cg) -- records may have
// been written earlier in the same kernel, so never through the non-coherent read-only path.
template <bool SMEM, typename T>
__device__ __forceinline__ T ldrec(const T* p) {
    if constexpr (SMEM)
        return *p;
    else
        return __ldcg(p);
}

// Contact rows (pass 0) or friction rows (pass 1) of record m of `sp` against the given body
// deltas; the updated applied impulses go to imp_out[0..3] (global memory).  With LOAD_ALL every
// point slot is loaded whatever the active mask (slots are always allocated; the inactive ones are
// never used), so the loads do not wait for the manifold header.
template <bool LOAD_ALL, bool SMEM>
__device__ __forceinline__ void solve_manifold(const SolverPoints& sp, int m, float4* imp_out, int pass,
                                               const int4& h, float imA, float imB, const b3gMat3& IA,
                                               const b3gMat3& IB, v3& dlA, v3& daA, v3& dlB, v3& daB, float& res_d,
                                               float& res_l) {
    const int mask = h.z;
    const size_t base = (size_t)m * 4;
    const float4 nf = ldrec<SMEM>(&sp.nf[m]);
    const v3 n = xyz(nf);
    float4 r1[4], r2[4], im[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (LOAD_ALL || (mask & (1 << j))) {
            r1[j] = ldrec<SMEM>(&sp.rel1[base + j]);
            r2[j] = ldrec<SMEM>(&sp.rel2[base + j]);
            im[j] = ldrec<SMEM>(&sp.imp[base + j]);
        }
    }
    if (pass == 0) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (!(mask & (1 << j))) continue;
            const v3 rel1 = xyz(r1[j]), rel2 = xyz(r2[j]);
            v3 r1xn = cross3(rel1, n);
            v3 ta1 = cross3(rel2, n);
            v3 r2xn = -ta1;
            v3 angA = imul(IA, r1xn);
            v3 angB = imul(IB, -ta1);
            float old = im[j].x;
            float nw = solve_row<false>(n, r1[j].w, r2[j].w, old, r1xn, r2xn, angA, angB, 0.f, LARGE_UPPER, dlA, daA,
                                        dlB, daB, imA, imB);
            __stcg(&imp_out[j].x, nw);
            float nd = nw - old;
            res_d += nd * nd;
            res_l += nw * nw;
        }
    } else {
        const float fr = nf.w;
        float4 d2[4], d1[4];
        float2 rf[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (LOAD_ALL || (mask & (1 << j))) {
                d2[j] = ldrec<SMEM>(&sp.dir2[base + j]);
                d1[j] = ldrec<SMEM>(&sp.dir1[base + j]);
                rf[j] = ldrec<SMEM>(&sp.rhsf[base + j]);
            }
        }
        if (pass == 3) {
            // warm start: the initial impulses (contact, dir2, dir1) applied to the body deltas
            // as internalApplyImpulse does under B3_SOLVER_USE_WARMSTARTING
            // (b3PgsJacobiSolver.cpp:745-752, 815-843); same vectors as the rows' own updates
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (!(mask & (1 << j))) continue;
                const v3 rel1 = xyz(r1[j]), rel2 = xyz(r2[j]);
                {
                    const float w = im[j].x;
                    v3 r1xn = cross3(rel1, n);
                    v3 ta1 = cross3(rel2, n);
                    v3 angA = imul(IA, r1xn);
                    v3 angB = imul(IB, -ta1);
                    dlA = dlA + (n * imA) * w;
                    daA = daA + angA * w;
                    dlB = dlB + ((-n) * imB) * w;
                    daB = daB + angB * w;
                }
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    const v3 d = xyz(k == 0 ? d2[j] : d1[j]);
                    const float w = k == 0 ? im[j].y : im[j].z;
                    v3 r1xn = cross3(rel1, d);
                    v3 r2xn = cross3(rel2, -d);
                    v3 angA = imul(IA, r1xn);
                    v3 angB = imul(IB, r2xn);
                    dlA = dlA + (d * imA) * w;
                    daA = daA + angA * w;
                    dlB = dlB + ((-d) * imB) * w;
                    daB = daB + angB * w;
                }
            }
            return;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (!(mask & (1 << j))) continue;
            float total = im[j].x;
            const v3 rel1 = xyz(r1[j]), rel2 = xyz(r2[j]);
            float f2 = im[j].y, f1 = im[j].z;
            if (pass == 2) {
                // interleaved (B3_SOLVER_INTERLEAVE_CONTACT_AND_FRICTION_CONSTRAINTS,
                // b3PgsJacobiSolver.cpp:1334-1377): this point's contact row first, its friction
                // rows bounded by the new impulse
                v3 r1xn = cross3(rel1, n);
                v3 ta1 = cross3(rel2, n);
                v3 r2xn = -ta1;
                v3 angA = imul(IA, r1xn);
                v3 angB = imul(IB, -ta1);
                const float old = total;
                total = solve_row<false>(n, r1[j].w, r2[j].w, old, r1xn, r2xn, angA, angB, 0.f, LARGE_UPPER, dlA,
                                         daA, dlB, daB, imA, imB);
                const float nd = total - old;
                res_d += nd * nd;
                res_l += total * total;
            }
            if (total > 0.f) {
                const float lower = -(fr * total), upper = fr * total;
                {
                    v3 d = xyz(d2[j]);
                    v3 r1xn = cross3(rel1, d);
                    v3 r2xn = cross3(rel2, -d);
                    float nw = solve_row<true>(d, d2[j].w, rf[j].x, f2, r1xn, r2xn, imul(IA, r1xn), imul(IB, r2xn),
                                               lower, upper, dlA, daA, dlB, daB, imA, imB);
                    float nd = nw - f2;
                    res_d += nd * nd;
                    f2 = nw;
                }
                {
                    v3 d = xyz(d1[j]);
                    v3 r1xn = cross3(rel1, d);
                    v3 r2xn = cross3(rel2, -d);
                    float nw = solve_row<true>(d, d1[j].w, rf[j].y, f1, r1xn, r2xn, imul(IA, r1xn), imul(IB, r2xn),
                                               lower, upper, dlA, daA, dlB, daB, imA, imB);
                    float nd = nw - f1;
                    res_d += nd * nd;
                    f1 = nw;
                }
                __stcg(&imp_out[j], make_float4(total, f2, f1, 0.f));
            } else if (pass == 2) {
                __stcg(&imp_out[j].x, total);
            }
            res_l += f2 * f2 + f1 * f1;
        }
    }
}

// ---- one manifold of the colour-ordered records (k_pgs_sweeps, k_pgs_flow): the rows of
// solve_manifold with the angular components (inverse inertia x relpos x axis) read from the
// setup's precomputation, which used the same operations on the same values, so every row sees
// the same numbers bit for bit.  Points stream through two register sets: the records of point
// j + 1 are loaded while point j solves.
struct OrdPoint {
    float4 r1, r2, P, Q;      // rel_pos1 + jac, rel_pos2 + rhs, contact angular A / B (+ dir2 A.xy)
    float4 d2, d1, R, S;      // friction directions + jacs, remaining angular components
    float2 rf, T;
};

// The records are read-only while the sweeps run (k_setup_rows wrote them in an earlier launch),
// so they go through the non-coherent path and hit the lines prefetch_manifold brought into L1;
// the applied impulses, rewritten every sweep, are read from L2 (all points at once, beside the
// body deltas, by solve_ord).
__device__ __forceinline__ void ld_point(const SolverPoints& sp, size_t s, int pass, OrdPoint& p) {
    p.r1 = __ldg(&sp.rel1[s]);
    p.r2 = __ldg(&sp.rel2[s]);
    p.P = __ldg(&sp.angP[s]);
    p.Q = __ldg(&sp.angQ[s]);
    if (pass != 0) {
        p.d2 = __ldg(&sp.dir2[s]);
        p.d1 = __ldg(&sp.dir1[s]);
        p.rf = __ldg(&sp.rhsf[s]);
        p.R = __ldg(&sp.angR[s]);
        p.S = __ldg(&sp.angS[s]);
        p.T = __ldg(&sp.angT[s]);
    }
}

__device__ __forceinline__ void solve_point(const OrdPoint& p, float4 im, v3 n, float fr, int pass, float4* out, float imA,
                                            float imB, v3& dlA, v3& daA, v3& dlB, v3& daB, float& res_d,
                                            float& res_l) {
    const v3 rel1 = xyz(p.r1), rel2 = xyz(p.r2);
    const v3 cA = xyz(p.P), cB = xyz(p.Q);
    const v3 a2 = mk3(p.P.w, p.Q.w, p.R.x), b2 = mk3(p.R.y, p.R.z, p.R.w);
    const v3 a1 = xyz(p.S), b1 = mk3(p.S.w, p.T.x, p.T.y);
    if (pass == 3) {
        // warm start (b3PgsJacobiSolver.cpp:745-752, 815-843), as solve_manifold
        float w = im.x;
        dlA = dlA + (n * imA) * w;
        daA = daA + cA * w;
        dlB = dlB + ((-n) * imB) * w;
        daB = daB + cB * w;
        const v3 e2 = xyz(p.d2), e1 = xyz(p.d1);
        w = im.y;
        dlA = dlA + (e2 * imA) * w;
        daA = daA + a2 * w;
        dlB = dlB + ((-e2) * imB) * w;
        daB = daB + b2 * w;
        w = im.z;
        dlA = dlA + (e1 * imA) * w;
        daA = daA + a1 * w;
        dlB = dlB + ((-e1) * imB) * w;
        daB = daB + b1 * w;
        return;
    }
    float total = im.x;
    if (pass != 1) {
        const v3 r1xn = cross3(rel1, n);
        const v3 r2xn = -cross3(rel2, n);
        const float old = total;
        total = solve_row<false>(n, p.r1.w, p.r2.w, old, r1xn, r2xn, cA, cB, 0.f, LARGE_UPPER, dlA, daA, dlB, daB,
                                 imA, imB);
        const float nd = total - old;
        res_d += nd * nd;
        res_l += total * total;
        if (pass == 0) {
            __stcg(&out->x, total);
            return;
        }
    }
    float f2 = im.y, f1 = im.z;
    if (total > 0.f) {
        const float lower = -(fr * total), upper = fr * total;
        {
            const v3 d = xyz(p.d2);
            const float nw = solve_row<true>(d, p.d2.w, p.rf.x, f2, cross3(rel1, d), cross3(rel2, -d), a2, b2, lower,
                                             upper, dlA, daA, dlB, daB, imA, imB);
            const float nd = nw - f2;
            res_d += nd * nd;
            f2 = nw;
        }
        {
            const v3 d = xyz(p.d1);
            const float nw = solve_row<true>(d, p.d1.w, p.rf.y, f1, cross3(rel1, d), cross3(rel2, -d), a1, b1, lower,
                                             upper, dlA, daA, dlB, daB, imA, imB);
            const float nd = nw - f1;
            res_d += nd * nd;
            f1 = nw;
        }
        __stcg(out, make_float4(total, f2, f1, 0.f));
    } else if (pass == 2) {
        __stcg(&out->x, total);
    }
    res_l += f2 * f2 + f1 * f1;
}

__device__ __forceinline__ void solve_ord(const SolverPoints& sp, int k, int pass, int mask, float imA, float imB,
                                          v3& dlA, v3& daA, v3& dlB, v3& daB, float& res_d, float& res_l) {
    const float4 nf = __ldg(&sp.nf[k]);
    const v3 n = xyz(nf);
    const size_t base = (size_t)k * 4;
    if (!mask) return;
    float4 im[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
        if (mask & (1 << q)) im[q] = __ldcg(&sp.imp[base + q]);
    int j = __ffs(mask) - 1;
    OrdPoint cur, nxt;
    ld_point(sp, base + j, pass, cur);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (q != j) continue;  // q walks the set points in order (unrolled: im[] stays in registers)
        const int rest = mask & ~((2 << j) - 1);  // points after j
        const int jn = rest ? __ffs(rest) - 1 : -1;
        if (jn >= 0) ld_point(sp, base + jn, pass, nxt);
        solve_point(cur, im[q], n, nf.w, pass, sp.imp + base + j, imA, imB, dlA, daA, dlB, daB, res_d, res_l);
        if (jn < 0) break;
        cur = nxt;
        j = jn;
    }
}

__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// One manifold's colour-ordered records on their way into this SM's L1 (issued before the wait
// that precedes the manifold's solve, so that only the body deltas cost an L2 round trip after
// it); its applied impulses into L2.  A manifold's 4 point slots of one array are 64 contiguous
// bytes, one line.
__device__ __forceinline__ void prefetch_manifold(const SolverArgs& a, int k) {
    const size_t b4 = (size_t)k * 4;
    prefetch_l1(&a.hdr_ord[k]);
    prefetch_l1(&a.inv_mass_ord[k]);
    prefetch_l1(&a.sp_ord.nf[k]);
    prefetch_l1(&a.sp_ord.rel1[b4]);
    prefetch_l1(&a.sp_ord.rel2[b4]);
    prefetch_l1(&a.sp_ord.angP[b4]);
    prefetch_l1(&a.sp_ord.angQ[b4]);
    prefetch_l1(&a.sp_ord.dir2[b4]);
    prefetch_l1(&a.sp_ord.dir1[b4]);
    prefetch_l1(&a.sp_ord.rhsf[b4]);
    prefetch_l1(&a.sp_ord.angR[b4]);
    prefetch_l1(&a.sp_ord.angS[b4]);
    prefetch_l1(&a.sp_ord.angT[b4]);
    prefetch_l2(&a.sp_ord.imp[b4]);
}


__device__ __forceinline__ void block_accumulate(double* dst, float x, float y) {
    __shared__ float sx[PK_THREADS / 32], sy[PK_THREADS / 32];
    for (int o = 16; o; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sx[threadIdx.x >> 5] = x;
        sy[threadIdx.x >> 5] = y;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float tx = 0, ty = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) {
            tx += sx[w];
            ty += sy[w];
        }
        if (tx != 0.f) atomicAdd(&dst[0], (double)tx);
        if (ty != 0.f) atomicAdd(&dst[1], (double)ty);
    }
    __syncthreads();
}

// Warp-aggregated counters: lanes with the same key (key < 0: none) add their number with one
// atomic.  All 32 lanes must call.
__device__ __forceinline__ void warp_count(int* counts, int key) {
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&counts[key], __popc(peers));
}
// Warp-aggregated reservation: returns this lane's slot in the run reserved for its key.  All 32
// lanes must call.  Within a key, slots follow lane order.
__device__ __forceinline__ int warp_reserve(int* cursors, int key) {
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&cursors[key], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__device__ __forceinline__ unsigned int hash32(unsigned int x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ void load_dv(const SolverArgs& a, int b, v3& l, v3& w) {
    l = xyz(__ldcg(&a.dv[2 * b]));
    w = xyz(__ldcg(&a.dv[2 * b + 1]));
}
__device__ __forceinline__ void store_dv(const SolverArgs& a, int b, v3 l, v3 w) {
    __stcg(&a.dv[2 * b], f4(l, 0.f));
    __stcg(&a.dv[2 * b + 1], f4(w, 0.f));
}

// residual bookkeeping shared by both kernels; returns true when the tolerance stops the solve.
// `it` indexes the residual slots and counts the sweeps run so far (it + 1 after this one).
__device__ __forceinline__ bool end_iteration(const SolverArgs& a, int it, float res_d, float res_l, bool& ok,
                                              double* r_out = nullptr) {
    block_accumulate(a.residual_acc + 2 * it, res_d, res_l);
    if (!grid_barrier(a.bar, gridDim.x, a.spin_limit)) {
        ok = false;
        return true;
    }
    double dd = *((volatile double*)&a.residual_acc[2 * it]);
    double ll = *((volatile double*)&a.residual_acc[2 * it + 1]);
    double r = sqrt(dd) / fmax(sqrt(ll), 1e-12);
    if (r_out) *r_out = r;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.counters->residual = (float)r;
        a.counters->iterations = it + 1;
    }
    return a.residual_tol > 0.f && r <= (double)a.residual_tol;
}

// Block-wide exclusive scan of n ints (one block): out[i] = sum(in[0..i)), returns the total.
__device__ int block_exclusive_scan(const int* in, int* out, int n) {
    __shared__ int s_part[PK_THREADS];
    const int T = blockDim.x;
    const int per = (n + T - 1) / T;
    const int lo = threadIdx.x * per, hi = min(lo + per, n);
    int s = 0;
    for (int i = lo; i < hi; i++) s += __ldcg(&in[i]);
    s_part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        int v = threadIdx.x >= off ? s_part[threadIdx.x - off] : 0;
        __syncthreads();
        s_part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = threadIdx.x ? s_part[threadIdx.x - 1] : 0;
    for (int i = lo; i < hi; i++) {
        int v = __ldcg(&in[i]);
        out[i] = run;
        run += v;
    }
    int total = s_part[T - 1];
    __syncthreads();
    return total;
}

// Body deltas of the partitioned PGS: bodies owned by this block live in shared memory during
// the block-local phase (6 floats each), everything else in global memory.
__device__ __forceinline__ void load_dv_local(const SolverArgs& a, const float* s_dv, int body, int local, v3& l,
                                              v3& w) {
    if (local >= 0) {
        const float* p = s_dv + 6 * local;
        l = mk3(p[0], p[1], p[2]);
        w = mk3(p[3], p[4], p[5]);
    } else {
        load_dv(a, body, l, w);
    }
}
__device__ __forceinline__ void store_dv_local(const SolverArgs& a, float* s_dv, int body, int local, v3 l, v3 w) {
    if (local >= 0) {
        float* p = s_dv + 6 * local;
        p[0] = l.x; p[1] = l.y; p[2] = l.z;
        p[3] = w.x; p[4] = w.y; p[5] = w.z;
    } else {
        store_dv(a, body, l, w);
    }
}
// World inverse inertia of an owned body from shared memory (9 floats, staged once per solve),
// of any other body from global memory.
// rows written earlier in the same launch: read through L2, never the non-coherent path
__device__ __forceinline__ b3gMat3 ld_mat_cg(const float4* q) {
    b3gMat3 r;
    const float4 x = __ldcg(q), y = __ldcg(q + 1), z = __ldcg(q + 2);
    r.row[0] = b3gFloat4{x.x, x.y, x.z, x.w};
    r.row[1] = b3gFloat4{y.x, y.y, y.z, y.w};
    r.row[2] = b3gFloat4{z.x, z.y, z.z, z.w};
    return r;
}

__device__ __forceinline__ b3gMat3 load_inertia_local(const SolverArgs& a, const float* s_inv, int body, int local) {
    if (local >= 0) {
        const float* p = s_inv + 9 * local;
        b3gMat3 r;
        r.row[0] = b3gFloat4{p[0], p[1], p[2], 0.f};
        r.row[1] = b3gFloat4{p[3], p[4], p[5], 0.f};
        r.row[2] = b3gFloat4{p[6], p[7], p[8], 0.f};
        return r;
    }
    return ld_mat(&a.inertias[body].invInertiaWorld);
}

// ---- streamed tiles: one tile = up to R consecutive block-local manifolds of one colour, copied
// into a shared-memory buffer laid out as [hdr R][inv mass R][nf R][rel1 4R][rel2 4R][imp 4R]
// [dir2 4R][dir1 4R][rhsf 4R] (16-byte elements except rhsf's 8, so every piece is a 16-byte
// multiple at a 16-byte aligned offset); the contact pass copies only the first six pieces.
__device__ __forceinline__ unsigned tile_bytes(int cnt, int pass) { return (unsigned)cnt * (pass ? 400u : 240u); }

__device__ __forceinline__ void issue_tile(const SolverArgs& a, char* buf, int R, unsigned long long* bar, int k0,
                                           int cnt, int pass) {
    const unsigned c = (unsigned)cnt;
    mbar_expect_tx(bar, tile_bytes(cnt, pass));
    bulk_g2s(buf, a.hdr_ord + k0, 16u * c, bar);
    bulk_g2s(buf + 16 * R, a.inv_mass_ord + k0, 16u * c, bar);
    bulk_g2s(buf + 32 * R, a.sp_ord.nf + k0, 16u * c, bar);
    bulk_g2s(buf + 48 * R, a.sp_ord.rel1 + 4 * (size_t)k0, 64u * c, bar);
    bulk_g2s(buf + 112 * R, a.sp_ord.rel2 + 4 * (size_t)k0, 64u * c, bar);
    bulk_g2s(buf + 176 * R, a.sp_ord.imp + 4 * (size_t)k0, 64u * c, bar);
    if (pass) {
        bulk_g2s(buf + 240 * R, a.sp_ord.dir2 + 4 * (size_t)k0, 64u * c, bar);
        bulk_g2s(buf + 304 * R, a.sp_ord.dir1 + 4 * (size_t)k0, 64u * c, bar);
        bulk_g2s(buf + 368 * R, a.sp_ord.rhsf + 4 * (size_t)k0, 32u * c, bar);
    }
}

__device__ __forceinline__ void bulk_prefetch_l2(const void* p, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
// L2 prefetch of the ordered records [k0, k0 + cnt) one pass reads (no-op for cnt <= 0)
__device__ __forceinline__ void prefetch_records_l2(const SolverArgs& a, int k0, int cnt, int pass) {
    if (cnt <= 0) return;
    const unsigned c = (unsigned)cnt;
    bulk_prefetch_l2(a.hdr_ord + k0, 16u * c);
    bulk_prefetch_l2(a.inv_mass_ord + k0, 16u * c);
    bulk_prefetch_l2(a.sp_ord.nf + k0, 16u * c);
    bulk_prefetch_l2(a.inertia_ord + 6 * (size_t)k0, 96u * c);
    bulk_prefetch_l2(a.sp_ord.rel1 + 4 * (size_t)k0, 64u * c);
    bulk_prefetch_l2(a.sp_ord.rel2 + 4 * (size_t)k0, 64u * c);
    bulk_prefetch_l2(a.sp_ord.imp + 4 * (size_t)k0, 64u * c);
    if (pass) {
        bulk_prefetch_l2(a.sp_ord.dir2 + 4 * (size_t)k0, 64u * c);
        bulk_prefetch_l2(a.sp_ord.dir1 + 4 * (size_t)k0, 64u * c);
        bulk_prefetch_l2(a.sp_ord.rhsf + 4 * (size_t)k0, 32u * c);
    }
}

__device__ __forceinline__ SolverPoints tile_view(char* buf, int R) {
    SolverPoints v;
    v.nf = reinterpret_cast<float4*>(buf + 32 * R);
    v.rel1 = reinterpret_cast<float4*>(buf + 48 * R);
    v.rel2 = reinterpret_cast<float4*>(buf + 112 * R);
    v.imp = reinterpret_cast<float4*>(buf + 176 * R);
    v.dir2 = reinterpret_cast<float4*>(buf + 240 * R);
    v.dir1 = reinterpret_cast<float4*>(buf + 304 * R);
    v.rhsf = reinterpret_cast<float2*>(buf + 368 * R);
    return v;
}

// Partition owning a dynamic body: its cell-order position / chunk, or -2 when the body is not in
// the cell-sorted list (inverse mass changed after upload, or no broadphase ran this step).
__device__ __forceinline__ int owner_of(const SolverArgs& a, int body) {
    const int p = __ldcg(&a.body_slot[body]);
    if (p < 0 || p >= a.num_dynamic || (int)a.sorted_bodies[p] != body) return -2;
    return p / a.chunk;
}

// ------------------------------------------------------------------ persistent PGS kernel
// Processing order of one PGS pass (a valid Gauss-Seidel order: every group holds manifolds
// that share no dynamic body, and groups run in key order):
//   1. block-local groups: block g owns the dynamic bodies at positions [g*chunk, (g+1)*chunk) of
//      the broadphase's cell-sorted body list; a manifold whose dynamic bodies are all owned by g
//      (statics belong to nobody) is solved by block g, colour by colour, with __syncthreads
//      between colours and the owned body deltas in shared memory.  Different blocks touch
//      disjoint bodies, so running them concurrently equals running them in block order;
//   2. one grid barrier, then the cross-partition manifolds, coloured on their own, colour by
//      colour with a grid barrier per colour.
// Group key = owner * NC + colour (block-local) or nblocks * NC + colour (cross), NC = number of
// block-local colours; the solve order (b3g_read_solve_order) is the manifolds sorted by key.
// PARTS: block partitions (SHARED / STREAMED / GLOBAL_DELTAS splits); without it every manifold is
// solved grid-wide and the shared-memory and tile paths are compiled out.
template <bool PARTS>
__global__ void __launch_bounds__(PK_THREADS, 1) k_solve_pgs(SolverArgs a) {
    extern __shared__ __align__(128) float s_dv[];
    grid_barrier_begin();
    const int nc = *a.d_nc;
    const unsigned nb = gridDim.x;
    const int G = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    const int nd = a.num_dynamic;
    const int chunk = a.chunk;
    // slot map: position of every dynamic body in cell order (read after the first barrier below)
    for (int p = tid; p < nd; p += stride) a.body_slot[a.sorted_bodies[p]] = p;
    // ---- partition owner of every manifold: a block index when all of its dynamic bodies belong
    // to that block's partition, -1 (cross-partition) otherwise
    if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
    for (int m = tid; m < nc; m += stride) {
        const int4 h = a.hdr[m];
        const float2 im = a.inv_mass[m];
        const int oA = im.x != 0.f ? owner_of(a, h.x) : -1;
        const int oB = im.y != 0.f ? owner_of(a, h.y) : -1;
        // -2 (a dynamic body outside the partitioned list) and differing owners go cross-partition
        int owner = -1;
        if (oA != -2 && oB != -2) owner = (oA >= 0 && oB >= 0) ? (oA == oB ? oA : -1) : (oA >= 0 ? oA : oB);
        a.manifold_group[m] = owner;
    }
    // ---- colouring: Jones-Plassmann greedy, block-local and cross-partition manifolds coloured
    // independently (they never run in the same phase).  Per round a manifold that holds the
    // highest hashed priority on both of its dynamic bodies takes the smallest colour used by
    // neither body (exact per-body 64-bit masks, no aliasing); statics never conflict.  The
    // manifold_group reads below are the thread's own writes from the loop above (same m mapping).
    int rounds = 0;
    for (int r = 0; r < B3G_MAX_COLORS; r++) {
        const unsigned long long rk = (unsigned long long)r << 56;
        for (int m = tid; m < nc; m += stride) {
            if (a.color[m] >= 0) continue;
            const int4 h = a.hdr[m];
            const float2 im = a.inv_mass[m];
            unsigned long long* claim = a.manifold_group[m] < 0 ? a.claim_x : a.claim;
            unsigned long long key = rk | ((unsigned long long)(hash32((unsigned)m) & 0xFFFFFFu) << 32) | (unsigned)m;
            if (im.x != 0.f) atomicMax(&claim[h.x], key);
            if (im.y != 0.f) atomicMax(&claim[h.y], key);
        }
        if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
        int left = 0;
        // every lane runs the same trip count so the per-colour counts aggregate across the warp
        for (int m0 = tid - (threadIdx.x & 31); m0 < nc; m0 += stride) {
            const int m = m0 + (threadIdx.x & 31);
            int fill_key = -1;
            if (m >= nc || a.color[m] >= 0) {
                warp_count(a.color_fill, fill_key);
                continue;
            }
            const int4 h = a.hdr[m];
            const float2 im = a.inv_mass[m];
            const bool cross = a.manifold_group[m] < 0;
            unsigned long long* claim = cross ? a.claim_x : a.claim;
            unsigned long long* mask = cross ? a.mask_x : a.mask;
            unsigned long long key = rk | ((unsigned long long)(hash32((unsigned)m) & 0xFFFFFFu) << 32) | (unsigned)m;
            bool okA = im.x == 0.f || __ldcg(&claim[h.x]) == key;
            bool okB = im.y == 0.f || __ldcg(&claim[h.y]) == key;
            if (okA && okB) {
                unsigned long long used = 0ull;
                if (im.x != 0.f) used |= __ldcg(&mask[h.x]);
                if (im.y != 0.f) used |= __ldcg(&mask[h.y]);
                int c = __ffsll((long long)~used) - 1;
                if (c >= 0 && c < 64) {
                    a.color[m] = c;
                    fill_key = c + (cross ? 64 : 0);
                    if (im.x != 0.f) atomicOr(&mask[h.x], 1ull << c);
                    if (im.y != 0.f) atomicOr(&mask[h.y], 1ull << c);
                } else {
                    left++;
                }
            } else {
                left++;
            }
            warp_count(a.color_fill, fill_key);
        }
        for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
        if ((threadIdx.x & 31) == 0 && left) atomicAdd(&a.remaining[r], left);
        if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
        rounds = r + 1;
        if (*((volatile int*)&a.remaining[r]) == 0) break;
    }
    // highest used colour of each colouring: one L2 read per lane, then a warp vote
    int ncl = 0, ncx = 0;
    {
        const int lane = threadIdx.x & 31;
        const unsigned l0 = __ballot_sync(0xffffffffu, __ldcg(&a.color_fill[lane]) > 0);
        const unsigned l1 = __ballot_sync(0xffffffffu, __ldcg(&a.color_fill[lane + 32]) > 0);
        const unsigned x0 = __ballot_sync(0xffffffffu, __ldcg(&a.color_fill[lane + 64]) > 0);
        const unsigned x1 = __ballot_sync(0xffffffffu, __ldcg(&a.color_fill[lane + 96]) > 0);
        ncl = l1 ? 64 - __clz(l1) : (l0 ? 32 - __clz(l0) : 0);
        ncx = x1 ? 64 - __clz(x1) : (x0 ? 32 - __clz(x0) : 0);
    }
    const bool overflow = rounds > 0 && *((volatile int*)&a.remaining[rounds - 1]) != 0 && nc > 0;
    const int NC = ncl > 0 ? ncl : 1;  // key stride of the block-local groups
    const int ngroups = G * NC + ncx;
    int* gcount = a.group_counts;
    int* goff = gcount + a.group_seg;
    int* gcur = goff + a.group_seg;
    // ---- processing group of every manifold: owner * NC + colour (block-local) or
    // G * NC + colour (cross-partition).  Reported colours: block-local c, cross ncl + c, so the
    // batches stay legal as one colouring.
    for (int m0 = tid - (threadIdx.x & 31); m0 < nc; m0 += stride) {
        const int m = m0 + (threadIdx.x & 31);
        int key = -1;
        if (m < nc) {
            const int c = a.color[m];
            if (c >= 0) {
                const int owner = a.manifold_group[m];
                key = owner >= 0 ? owner * NC + c : G * NC + c;
                if (owner < 0) a.color[m] = ncl + c;
            }
            a.manifold_group[m] = key;
        }
        warp_count(gcount, key);
    }
    if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
    if (blockIdx.x == 0) {
        int total = block_exclusive_scan(gcount, goff, ngroups);
        if (threadIdx.x == 0) {
            goff[ngroups] = total;
            a.counters->num_colors = ncl + ncx;
            if (overflow) atomicOr(&a.counters->status, B3G_FLAG_BATCH_OVERFLOW);
        }
    }
    if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
    for (int m0 = tid - (threadIdx.x & 31); m0 < nc; m0 += stride) {
        const int m = m0 + (threadIdx.x & 31);
        const int key = m < nc ? a.manifold_group[m] : -1;
        const int pos = warp_reserve(gcur, key);
        if (key >= 0) a.color_order[__ldcg(&goff[key]) + pos] = m;
    }
    const int ncol = __ldcg(&goff[ngroups]);  // coloured manifolds; the rest are overflow leftovers
    if (overflow && tid == 0) {
        int k = ncol;
        for (int m = 0; m < nc; m++)
            if (a.color[m] < 0) a.color_order[k++] = m;
    }
    if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
    // ---- group-ordered copy of the records (coalesced phases, no order -> header indirection);
    // block-local manifolds carry their bodies' shared-memory slots in hdr.w (0xffff = not owned)
    // One thread per point slot: the four slots of a record are read and written as one
    // contiguous 64-byte run per array (slots of inactive points are copied too; never used).
    // Four slots per thread are in flight at once (all loads issued before the stores).
    const int nlocal = __ldcg(&goff[G * NC]);
    for (int t0 = tid; t0 < 4 * nc; t0 += 4 * stride) {
        float4 r1[4], r2[4], d2[4], d1[4], im[4];
        float2 rf[4];
        size_t dst[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int t = t0 + u * stride;
            dst[u] = ~(size_t)0;
            if (t >= 4 * nc) continue;
            const int k = t >> 2, j = t & 3;
            const size_t s = (size_t)__ldcg(&a.color_order[k]) * 4 + j;
            dst[u] = (size_t)k * 4 + j;
            r1[u] = __ldcg(&a.sp.rel1[s]);
            r2[u] = __ldcg(&a.sp.rel2[s]);
            d2[u] = __ldcg(&a.sp.dir2[s]);
            d1[u] = __ldcg(&a.sp.dir1[s]);
            rf[u] = __ldcg(&a.sp.rhsf[s]);
            im[u] = __ldcg(&a.sp.imp[s]);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (dst[u] == ~(size_t)0) continue;
            const size_t d = dst[u];
            a.sp_ord.rel1[d] = r1[u];
            a.sp_ord.rel2[d] = r2[u];
            a.sp_ord.dir2[d] = d2[u];
            a.sp_ord.dir1[d] = d1[u];
            a.sp_ord.rhsf[d] = rf[u];
            a.sp_ord.imp[d] = im[u];
        }
    }
    for (int k = tid; k < nc; k += stride) {
        const int m = __ldcg(&a.color_order[k]);
        const int4 h = a.hdr[m];
        const float2 im = a.inv_mass[m];
        int w = 0xffffffff;
        if (k < nlocal) {
            const int owner = __ldcg(&a.manifold_group[m]) / NC;
            const int la = im.x != 0.f ? __ldcg(&a.body_slot[h.x]) - owner * chunk : 0xffff;
            const int lb = im.y != 0.f ? __ldcg(&a.body_slot[h.y]) - owner * chunk : 0xffff;
            w = (int)(((unsigned)la & 0xffffu) | (((unsigned)lb & 0xffffu) << 16));
        }
        a.hdr_ord[k] = make_int4(h.x, h.y, h.z, w);
        a.inv_mass_ord[k] = make_float4(im.x, im.y, 0.f, 0.f);
        a.sp_ord.nf[k] = __ldcg(&a.sp.nf[m]);
        // both bodies' inverse inertias next to the record: the solve reads them by position
        // instead of gathering them through the header's body indices
        {
            const float4* IA = reinterpret_cast<const float4*>(&a.inertias[h.x].invInertiaWorld);
            const float4* IB = reinterpret_cast<const float4*>(&a.inertias[h.y].invInertiaWorld);
            float4* o = a.inertia_ord + 6 * (size_t)k;
            o[0] = __ldg(IA); o[1] = __ldg(IA + 1); o[2] = __ldg(IA + 2);
            o[3] = __ldg(IB); o[4] = __ldg(IB + 1); o[5] = __ldg(IB + 2);
        }
    }
    if (PARTS && a.tile_R > 0) fence_proxy_async();  // the ordered records are read by bulk copies below
    if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
    // ---- iterations.  Segments of one pass: the NC block-local colours (__syncthreads between
    // them), then the ncx cross-partition colours and the colour-overflow leftovers (grid barrier
    // after each).  One solve call site keeps the register budget of the kernel low.
    const int myLo = blockIdx.x * chunk;
    const int myN = max(0, min(chunk, nd - myLo));
    const int nseg = NC + ncx + (overflow ? 1 : 0);
    float* s_inv = s_dv + 6 * chunk;  // owned bodies' world inverse inertia (fixed during the solve)
    // streamed tiles: two buffers after the owned-body arrays, then two mbarriers and the tile list
    const int R = PARTS ? a.tile_R : 0;
    const bool use_smem = PARTS && a.use_smem;
    char* tbuf = reinterpret_cast<char*>(s_dv) + ((60 * (size_t)chunk + 15) & ~(size_t)15);
    unsigned long long* tbar = reinterpret_cast<unsigned long long*>(tbuf + 2 * (size_t)R * B3G_PGS_TILE_BYTES);
    int2* tiles = reinterpret_cast<int2*>(tbar + 2);
    __shared__ int s_ntiles;
    unsigned tpar0 = 0, tpar1 = 0;  // phase parity of each buffer's mbarrier
    if (R > 0) {
        if (threadIdx.x == 0) {
            int nt = 0;
            for (int c = 0; c < NC && nt >= 0; c++) {
                const int lo = __ldcg(&goff[blockIdx.x * NC + c]), hi = __ldcg(&goff[blockIdx.x * NC + c + 1]);
                for (int k0 = lo; k0 < hi; k0 += R) {
                    if (nt == B3G_PGS_MAX_TILES) {  // too many tiles: this block reads records directly
                        nt = -1;
                        break;
                    }
                    tiles[nt++] = make_int2(k0, min(R, hi - k0));
                }
            }
            s_ntiles = nt;
            mbar_init(&tbar[0], 1);
            mbar_init(&tbar[1], 1);
            fence_mbar_init();
        }
        __syncthreads();
    }
    const int ntiles = R > 0 ? s_ntiles : -1;
    // [lo, hi) of every segment, read once: block-local colours, cross colours, leftovers
    __shared__ int2 s_seg[2 * 64 + 2];
    for (int sg = threadIdx.x; sg < nseg; sg += blockDim.x) {
        int lo = ncol, hi = nc;
        if (sg < NC + ncx) {
            const int key = sg < NC ? blockIdx.x * NC + sg : G * NC + sg - NC;
            lo = __ldcg(&goff[key]);
            hi = __ldcg(&goff[key + 1]);
        }
        s_seg[sg] = make_int2(lo, hi);
    }
    __syncthreads();
    if (use_smem) {
        for (int l = threadIdx.x; l < myN; l += blockDim.x) {
            const b3gMat3 I = ld_mat(&a.inertias[a.sorted_bodies[myLo + l]].invInertiaWorld);
            float* p = s_inv + 9 * l;
            p[0] = I.row[0].x; p[1] = I.row[0].y; p[2] = I.row[0].z;
            p[3] = I.row[1].x; p[4] = I.row[1].y; p[5] = I.row[1].z;
            p[6] = I.row[2].x; p[7] = I.row[2].y; p[8] = I.row[2].z;
        }
    }
    bool ok = true;
    // passes of one iteration: contact rows then friction rows, or one interleaved pass (2);
    // a warm start adds one application pass (3) before the first iteration
    const int npasses = a.interleave ? 1 : 2;
    bool warm_live = a.warm != 0;
    int extra = 0;  // 1 after a dropped warm start: its sweep still counts
    for (int it = a.warm ? -1 : 0; it < a.iterations; it++) {
        float res_d = 0.f, res_l = 0.f;
        const bool warm_pass = it < 0;
        for (int ps = 0; ps < (warm_pass ? 1 : npasses); ps++) {
            const int pass = warm_pass ? 3 : (a.interleave ? 2 : ps);
            if (use_smem) {
                for (int l = threadIdx.x; l < myN; l += blockDim.x) {
                    v3 dl, dw;
                    load_dv(a, (int)a.sorted_bodies[myLo + l], dl, dw);
                    float* p = s_dv + 6 * l;
                    p[0] = dl.x; p[1] = dl.y; p[2] = dl.z;
                    p[3] = dw.x; p[4] = dw.y; p[5] = dw.z;
                }
                __syncthreads();
            }
            // block-local phase, streamed: tile t+1 is copied while tile t is solved
            if (ntiles > 0) {
                if (threadIdx.x == 0) {
                    fence_proxy_async();
                    issue_tile(a, tbuf, R, &tbar[0], tiles[0].x, tiles[0].y, pass);
                }
                for (int t = 0; t < ntiles; t++) {
                    const int b = t & 1;
                    char* buf = tbuf + (size_t)b * R * B3G_PGS_TILE_BYTES;
                    if (threadIdx.x == 0 && t + 1 < ntiles) {
                        fence_proxy_async();
                        issue_tile(a, tbuf + (size_t)(b ^ 1) * R * B3G_PGS_TILE_BYTES, R, &tbar[b ^ 1],
                                   tiles[t + 1].x, tiles[t + 1].y, pass);
                    }
                    const bool got = mbar_wait(&tbar[b], b ? tpar1 : tpar0, a.spin_limit);
                    if (b)
                        tpar1 ^= 1u;
                    else
                        tpar0 ^= 1u;
                    if (__syncthreads_or(!got)) {
                        // a copy never completed: raise the abort, drain what is still in flight
                        if (threadIdx.x == 0) {
                            atomicExch(a.bar.abort_flag, 1u);
                            atomicOr(a.bar.status, B3G_FLAG_BARRIER_TIMEOUT);
                            if (!got) mbar_wait(&tbar[b], b ? tpar1 ^ 1u : tpar0 ^ 1u, a.spin_limit);
                            if (t + 1 < ntiles) mbar_wait(&tbar[b ^ 1], b ? tpar0 : tpar1, a.spin_limit);
                        }
                        __syncthreads();
                        return;
                    }
                    const int2 tl = tiles[t];
                    const SolverPoints tv = tile_view(buf, R);
                    for (int i = threadIdx.x; i < tl.y; i += blockDim.x) {
                        const int4 h = reinterpret_cast<const int4*>(buf)[i];
                        const float4 im = reinterpret_cast<const float4*>(buf + 16 * R)[i];
                        const int la = (h.w & 0xffff) == 0xffff ? -1 : (h.w & 0xffff);
                        const int lb = ((unsigned)h.w >> 16) == 0xffffu ? -1 : (int)((unsigned)h.w >> 16);
                        v3 dlA = mk3(0, 0, 0), daA = mk3(0, 0, 0), dlB = mk3(0, 0, 0), daB = mk3(0, 0, 0);
                        if (im.x != 0.f) load_dv_local(a, s_dv, h.x, la, dlA, daA);
                        if (im.y != 0.f) load_dv_local(a, s_dv, h.y, lb, dlB, daB);
                        const b3gMat3 IA = load_inertia_local(a, s_inv, h.x, la);
                        const b3gMat3 IB = load_inertia_local(a, s_inv, h.y, lb);
                        solve_manifold<true, true>(tv, i, a.sp_ord.imp + 4 * (size_t)(tl.x + i), pass, h, im.x, im.y,
                                                   IA, IB, dlA, daA, dlB, daB, res_d, res_l);
                        if (im.x != 0.f) store_dv_local(a, s_dv, h.x, la, dlA, daA);
                        if (im.y != 0.f) store_dv_local(a, s_dv, h.y, lb, dlB, daB);
                    }
                    __syncthreads();
                }
            }
            for (int sg = 0; sg < nseg; sg++) {
                const bool local = sg < NC;
                const int2 seg = s_seg[sg];
                // warm L2 with this block's records of the next segment while this one runs
                if (threadIdx.x == 0) {
                    int ns = sg + 1, npass = pass;
                    if (ns == nseg) {
                        ns = 0;
                        if (!a.interleave) npass ^= 1;
                    }
                    if (ns < NC) {
                        if (ntiles < 0) prefetch_records_l2(a, s_seg[ns].x, s_seg[ns].y - s_seg[ns].x, npass);
                    } else if (ns < NC + ncx) {
                        const int k0 = s_seg[ns].x + blockIdx.x * blockDim.x;
                        prefetch_records_l2(a, k0, min((int)blockDim.x, s_seg[ns].y - k0), npass);
                    }
                }
                int first, hi, step;
                if (local) {
                    first = seg.x + threadIdx.x;
                    hi = seg.y;
                    step = blockDim.x;
                    if (ntiles >= 0) first = hi;  // already solved by the streamed tiles
                } else if (sg < NC + ncx) {
                    if (seg.x == seg.y) continue;  // uniform across blocks
                    first = seg.x + tid;
                    hi = seg.y;
                    step = stride;
                } else {  // leftovers: one thread, in manifold order (always correct, slow)
                    first = ncol;
                    hi = tid == 0 ? nc : ncol;
                    step = 1;
                }
                const bool smem_here = local && use_smem;
                for (int k = first; k < hi; k += step) {
                    // no early exit for manifolds without active points: their deltas are read and
                    // written back unchanged, and the record loads need not wait for the header
                    const int4 h = __ldcg(&a.hdr_ord[k]);
                    const float4 im = __ldcg(&a.inv_mass_ord[k]);
                    int la = -1, lb = -1;
                    if (smem_here) {
                        la = (h.w & 0xffff) == 0xffff ? -1 : (h.w & 0xffff);
                        lb = ((unsigned)h.w >> 16) == 0xffffu ? -1 : (int)((unsigned)h.w >> 16);
                    }
                    v3 dlA = mk3(0, 0, 0), daA = mk3(0, 0, 0), dlB = mk3(0, 0, 0), daB = mk3(0, 0, 0);
                    if (im.x != 0.f) load_dv_local(a, s_dv, h.x, la, dlA, daA);
                    if (im.y != 0.f) load_dv_local(a, s_dv, h.y, lb, dlB, daB);
                    const b3gMat3 IA = la >= 0 ? load_inertia_local(a, s_inv, h.x, la)
                                               : ld_mat_cg(a.inertia_ord + 6 * (size_t)k);
                    const b3gMat3 IB = lb >= 0 ? load_inertia_local(a, s_inv, h.y, lb)
                                               : ld_mat_cg(a.inertia_ord + 6 * (size_t)k + 3);
                    solve_manifold<true, false>(a.sp_ord, k, a.sp_ord.imp + 4 * (size_t)k, pass, h, im.x, im.y, IA,
                                                IB, dlA, daA, dlB, daB, res_d, res_l);
                    if (im.x != 0.f) store_dv_local(a, s_dv, h.x, la, dlA, daA);
                    if (im.y != 0.f) store_dv_local(a, s_dv, h.y, lb, dlB, daB);
                }
                if (local) {
                    __syncthreads();
                    if (sg < NC - 1) continue;
                    // without partitions the local phase is empty in every block: the barrier
                    // after the previous segment already orders the phases around it
                    if (!PARTS || nd == 0) continue;
                    if (use_smem) {
                        for (int l = threadIdx.x; l < myN; l += blockDim.x) {
                            const float* p = s_dv + 6 * l;
                            store_dv(a, (int)a.sorted_bodies[myLo + l], mk3(p[0], p[1], p[2]),
                                     mk3(p[3], p[4], p[5]));
                        }
                    }
                }
                if (R > 0) fence_proxy_async();  // impulses written above are read by later bulk copies
                if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
            }
        }
        if (warm_pass) continue;  // the application pass has no residual
        // the residual is read (one more grid barrier) only where it decides something: a
        // tolerance, the warm-start check after the first sweep, and the last sweep's statistics
        if (!(a.residual_tol > 0.f || (it == 0 && warm_live) || it == a.iterations - 1)) {
            block_accumulate(a.residual_acc + 2 * (it + extra), res_d, res_l);
            continue;
        }
        double r = 0.0;
        if (end_iteration(a, it + extra, res_d, res_l, ok, &r)) break;
        if (it == 0 && warm_live) {
            warm_live = false;
            // a cold first sweep has residual exactly 1: a warm start that does worse is dropped
            // and the solve restarts cold with the full iteration budget (every block sees the same r)
            if (r > 1.0) {
                for (int i = tid; i < 2 * a.num_bodies; i += stride) __stcg(&a.dv[i], make_float4(0.f, 0.f, 0.f, 0.f));
                for (int k = tid; k < nc; k += stride)
                    for (int j = 0; j < 4; j++) __stcg(&a.sp_ord.imp[(size_t)k * 4 + j], make_float4(0.f, 0.f, 0.f, 0.f));
                if (tid == 0) atomicOr(&a.counters->status, B3G_FLAG_WARM_DISCARDED);
                extra = 1;
                it = -1;
                if (R > 0) fence_proxy_async();
                if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
            }
        }
    }
    if (!ok) return;
    // ---- applied impulses back to manifold order (read by b3g_read_impulses)
    for (int k = tid; k < nc; k += stride) {
        const int m = __ldcg(&a.color_order[k]);
        const int4 h = __ldcg(&a.hdr_ord[k]);
        for (int j = 0; j < 4; j++)
            if (h.z & (1 << j)) a.sp.imp[(size_t)m * 4 + j] = __ldcg(&a.sp_ord.imp[(size_t)k * 4 + j]);
    }
    // ---- finish: v += dv for dynamic bodies
    for (int b = tid; b < a.num_bodies; b += stride) {
        if (a.bodies[b].invMass == 0.f) continue;
        v3 dl, da;
        load_dv(a, b, dl, da);
        b3gBody& B = a.bodies_out[b];
        B.linVel.x = B.linVel.x + dl.x;
        B.linVel.y = B.linVel.y + dl.y;
        B.linVel.z = B.linVel.z + dl.z;
        B.angVel.x = B.angVel.x + da.x;
        B.angVel.y = B.angVel.y + da.y;
        B.angVel.z = B.angVel.z + da.z;
    }
}

// ------------------------------------------------------------------ persistent Jacobi kernel
__device__ __forceinline__ void jacobi_average(const SolverArgs& a, int tid, int stride) {
    for (int b = tid; b < a.num_bodies; b += stride) {
        const int cnt = a.body_count[b];
        if (cnt <= 0) continue;
        const int off = a.list_off[b];
        v3 sl = mk3(0.f, 0.f, 0.f), sa = mk3(0.f, 0.f, 0.f);
        for (int k = 0; k < cnt; k++) {
            uint32_t e = a.list[off + k];
            uint32_t m = e >> 1, side = e & 1u;
            sl = sl + xyz(__ldcg(&a.split[4 * m + 2 * side]));
            sa = sa + xyz(__ldcg(&a.split[4 * m + 2 * side + 1]));
        }
        float factor = 1.f / (float)cnt;
        a.dv_sum[2 * b] = f4(sl, 0.f);
        a.dv_sum[2 * b + 1] = f4(sa, 0.f);
        store_dv(a, b, sl * factor, sa * factor);
    }
}

__global__ void __launch_bounds__(PK_THREADS, 1) k_solve_jacobi(SolverArgs a) {
    grid_barrier_begin();
    const int nc = *a.d_nc;
    const unsigned nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.counters->num_colors = 0;
    bool ok = true;
    for (int it = 0; it < a.iterations; it++) {
        float res_d = 0.f, res_l = 0.f;
        for (int pass = 0; pass < 2; pass++) {
            for (int m = tid; m < nc; m += stride) {
                const int4 h = a.hdr[m];
                const float2 im = a.inv_mass[m];
                v3 dlA = mk3(0, 0, 0), daA = mk3(0, 0, 0), dlB = mk3(0, 0, 0), daB = mk3(0, 0, 0);
                if (im.x != 0.f) load_dv(a, h.x, dlA, daA);
                if (im.y != 0.f) load_dv(a, h.y, dlB, daB);
                if (h.z) {
                    const b3gMat3 IA = ld_mat(&a.inertias[h.x].invInertiaWorld);
                    const b3gMat3 IB = ld_mat(&a.inertias[h.y].invInertiaWorld);
                    solve_manifold<false, false>(a.sp, m, a.sp.imp + (size_t)m * 4, pass, h, im.x, im.y, IA, IB, dlA,
                                                 daA, dlB, daB, res_d, res_l);
                }
                __stcg(&a.split[4 * m + 0], f4(dlA, 0.f));
                __stcg(&a.split[4 * m + 1], f4(daA, 0.f));
                __stcg(&a.split[4 * m + 2], f4(dlB, 0.f));
                __stcg(&a.split[4 * m + 3], f4(daB, 0.f));
            }
            if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
            jacobi_average(a, tid, stride);
            if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
        }
        if (end_iteration(a, it, res_d, res_l, ok)) break;
    }
    if (!ok) return;
    // finish: body velocity += (S * 1/count), applied once per split copy
    for (int b = tid; b < a.num_bodies; b += stride) {
        const int cnt = a.body_count[b];
        if (cnt <= 0) continue;
        float factor = 1.f / (float)cnt;
        v3 dl = xyz(a.dv_sum[2 * b]) * factor, da = xyz(a.dv_sum[2 * b + 1]) * factor;
        b3gBody& B = a.bodies_out[b];
        v3 lv = f4v3(B.linVel), av = f4v3(B.angVel);
        for (int k = 0; k < cnt; k++) {
            lv = lv + dl;
            av = av + da;
        }
        B.linVel.x = lv.x; B.linVel.y = lv.y; B.linVel.z = lv.z;
        B.angVel.x = av.x; B.angVel.y = av.y; B.angVel.z = av.z;
    }
}

// Initial impulses of the point records.  A point persists when the previous solve had a
// manifold for the same body pair (binary search of the ascending pair keys) with an active point
// on body B within 0.05 of it; it then starts from that point's converged impulses (persist).
// Other points start from the network's prediction (pred, normalised units, 16 per slot: contact
// impulse >= 0, friction impulses inside that impulse's friction cone, non-finite values cold)
// or cold.  With write_imp 0 only the persistence flags are recorded.  Slots beyond rows_cap
// start cold.
struct WarmFill {
    const float* pred;            // nullptr: no network
    const float* tnorm;           // target mean[3], 1/std[3]
    const int* d_nc;
    int rows_cap;
    const int4* hdr;
    SolverPoints sp;
    const b3gContact4* slots;
    const int* manifold_pair;
    const int* d_npairs;
    int body_bits;
    const unsigned long long* prev_keys;
    const float4* prev_pts;
    const float4* prev_imp;
    const int* prev_n;
    int persist;                  // take persisting points' previous impulses
    float factor;                 // ... scaled by this
    int predict_all;              // network also for persisting points
    int write_imp;
    float4* init;
    unsigned char* is_new;
    const int* pos_of;            // non-null: initial impulses go to the colour-ordered records
    float4* imp_ord;
};

// A compound child pair's manifold is never carried over (several share a body pair): its key
// sorts after every pair's and matches nothing.
__device__ __forceinline__ bool is_child_manifold(const int* manifold_pair, const int* d_npairs, int m) {
    return __ldcg(&manifold_pair[m]) >= __ldcg(d_npairs);
}

__device__ __forceinline__ unsigned long long pair_key(int a, int b, int bits) {
    const unsigned lo = (unsigned)min(a, b), hi = (unsigned)max(a, b);
    return ((unsigned long long)lo << bits) | hi;
}

__global__ void k_warm_fill(WarmFill w) {
    const int nc = *w.d_nc;
    const int pn = *w.prev_n;
    const int mmax = min(nc, w.rows_cap / 4);
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < mmax; m += gridDim.x * blockDim.x) {
        const int4 h = w.hdr[m];
        const int mask = h.z;
        float4* imp_out = w.pos_of ? w.imp_ord + 4 * (size_t)__ldcg(&w.pos_of[m]) : w.sp.imp + 4 * (size_t)m;
        const float fr = (float)w.slots[w.manifold_pair[m]].frictionCmp / (float)0xffff;
        // previous manifold of the same body pair
        const unsigned long long key = pair_key(h.x, h.y, w.body_bits);
        int lo = 0, hi = pn;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (w.prev_keys[mid] < key)
                lo = mid + 1;
            else
                hi = mid;
        }
        const int q = (lo < pn && w.prev_keys[lo] == key && !is_child_manifold(w.manifold_pair, w.d_npairs, m)) ? lo : -1;
        const b3gContact4& c = w.slots[w.manifold_pair[m]];
        for (int j = 0; j < 4; j++) {
            const size_t s = (size_t)m * 4 + j;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            bool matched = false;
            if (mask & (1 << j)) {
                if (q >= 0) {
                    float best = 0.05f * 0.05f;
                    int bj = -1;
                    for (int k = 0; k < 4; k++) {
                        const float4 p = w.prev_pts[(size_t)q * 4 + k];
                        if (p.w == 0.f) continue;
                        const float dx = p.x - c.worldPosB[j].x, dy = p.y - c.worldPosB[j].y, dz = p.z - c.worldPosB[j].z;
                        const float d2 = dx * dx + dy * dy + dz * dz;
                        if (d2 < best) {
                            best = d2;
                            bj = k;
                        }
                    }
                    if (bj >= 0) {
                        matched = true;
                        if (w.persist) {
                            const float4 pv = w.prev_imp[(size_t)q * 4 + bj];
                            v = w.factor == 1.f ? pv : make_float4(pv.x * w.factor, pv.y * w.factor, pv.z * w.factor, 0.f);
                        }
                    }
                }
                if (w.pred && (!matched || w.predict_all || !w.persist)) {
                    const float* y = w.pred + s * 16;
                    float lam = y[0] / w.tnorm[3] + w.tnorm[0];
                    float f2 = y[1] / w.tnorm[4] + w.tnorm[1];
                    float f1 = y[2] / w.tnorm[5] + w.tnorm[2];
                    if (!(lam > 0.f) || !isfinite(lam)) lam = 0.f;
                    const float lim = fr * lam;
                    f2 = isfinite(f2) ? fminf(fmaxf(f2, -lim), lim) : 0.f;
                    f1 = isfinite(f1) ? fminf(fmaxf(f1, -lim), lim) : 0.f;
                    v = make_float4(lam, f2, f1, 0.f);
                }
                if (w.write_imp) imp_out[j] = v;
            }
            if (w.init) w.init[s] = w.write_imp ? v : make_float4(0.f, 0.f, 0.f, 0.f);
            if (w.is_new) w.is_new[s] = matched ? 0 : 1;
        }
    }
}

// The solved manifolds (first rows_cap / 4) for the next step's persistence lookup.
__global__ void k_warm_store(const int* __restrict__ d_nc, int rows_cap, const int4* __restrict__ hdr,
                             const b3gContact4* __restrict__ slots, const int* __restrict__ manifold_pair,
                             const int* __restrict__ d_npairs, const float4* __restrict__ imp, int body_bits,
                             unsigned long long* __restrict__ keys, float4* __restrict__ pts,
                             float4* __restrict__ pimp, int* __restrict__ prev_n) {
    const int n = min(*d_nc, rows_cap / 4);
    if (blockIdx.x == 0 && threadIdx.x == 0) *prev_n = n;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        const int4 h = hdr[m];
        keys[m] = is_child_manifold(manifold_pair, d_npairs, m) ? ~0ull : pair_key(h.x, h.y, body_bits);
        const b3gContact4& c = slots[manifold_pair[m]];
        for (int j = 0; j < 4; j++) {
            const size_t s = (size_t)m * 4 + j;
            const bool on = (h.z >> j) & 1;
            pts[s] = make_float4(c.worldPosB[j].x, c.worldPosB[j].y, c.worldPosB[j].z, on ? 1.f : 0.f);
            pimp[s] = on ? imp[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// ------------------------------------------------------------------ PGS in colour order from the setup on
// The grid-wide PGS path (no block partitions) colours the manifolds BEFORE the row setup, so the
// setup writes every record at its position in colour order and the sweeps read them in order:
//   k_manifold_prep   per manifold: header, inverse masses, and the colour the same body pair had
//                     in the last solve (manifolds follow the sorted pair list, so the last
//                     solve's keys are sorted too: a binary search, tried at the same index first)
//   k_colour          carried colours claim their bits in the per-body colour masks (a clash,
//                     possible only when a body's inverse mass changed, drops the later one);
//                     Jones-Plassmann rounds colour the rest against those masks; counting sort by
//                     colour gives every manifold its record position
//   k_setup_rows      records straight into colour order (and the warm start's impulses)
//   k_pgs_sweeps      the iterations; colours up to the first of a run of small trailing colours
//                     are grid-wide phases with a grid barrier each, the trailing small colours
//                     run in one block with __syncthreads between them and one grid barrier after
//                     the run; then impulses back to manifold order, v += dv, and this solve's keys
//                     and colours for the next one
// Any legal colouring gives a legal Gauss-Seidel order (the solve order stays readable through
// b3g_read_solve_order); colours carried over keep the persisting contacts' batches stable from
// step to step, and a scene whose contact set does not change is coloured once.
__global__ void __launch_bounds__(SV_THREADS) k_manifold_prep(SolverArgs a) {
    const int nc = *a.d_nc;
    const int pn = a.d_prev_n[2] ? 0 : a.d_prev_n[0];  // a recolouring carries nothing over
    int fresh = 0;
    for (int m0 = blockIdx.x * blockDim.x; m0 < nc; m0 += gridDim.x * blockDim.x) {
        const int m = m0 + (int)threadIdx.x;
        int col = -1;
        if (m < nc) {
            const b3gContact4& c = a.slots[a.manifold_pair[m]];
            const int iA = abs(c.bodyA), iB = abs(c.bodyB);
            const float imA = a.bodies[iA].invMass, imB = a.bodies[iB].invMass;
            int np = (int)c.worldNormalOnB.w;
            if (np > 4) np = 4;
            if (imA == 0.f && imB == 0.f) np = 0;
            int mask = 0;
            for (int j = 0; j < np; j++)
                if (c.worldPosB[j].w <= a.threshold) mask |= 1 << j;
            a.hdr[m] = make_int4(iA, iB, mask, np);
            a.inv_mass[m] = make_float2(imA, imB);
            if (pn > 0 && a.manifold_pair[m] < *a.d_npairs) {
                const unsigned long long key = pair_key(iA, iB, a.body_bits);
                int q = min(m, pn - 1);
                if (__ldcg(&a.prev_key[q]) != key) {
                    int lo = 0, hi = pn;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (__ldcg(&a.prev_key[mid]) < key)
                            lo = mid + 1;
                        else
                            hi = mid;
                    }
                    q = (lo < pn && __ldcg(&a.prev_key[lo]) == key) ? lo : -1;
                }
                if (q >= 0) {
                    col = __ldcg(&a.prev_color[q]);
                    if (col >= 64) col = -1;
                }
            }
            a.color[m] = col;
            fresh += col < 0;
        }
    }
    for (int o = 16; o; o >>= 1) fresh += __shfl_xor_sync(0xffffffffu, fresh, o);
    if ((threadIdx.x & 31) == 0 && fresh) atomicAdd(a.d_new, fresh);
}

// Cooperative: carried colours, Jones-Plassmann for the rest, record positions.  Colour 64 holds
// the manifolds that found no colour below 64 (solved one after another by one thread).
// One Jones-Plassmann round over the uncoloured manifolds [first, nlist) step `step` of the list
// (or the manifold indices themselves when !listed): claim -- each manifold's key (round, hashed
// priority, index) into both dynamic bodies' claim words (atomic max); assign -- a manifold that
// holds both claims takes the smallest colour free on both bodies.  Returns the manifolds left.
constexpr int JP_LOCAL_MAX = 8192;
__device__ __forceinline__ unsigned long long jp_key(int r, int m) {
    return ((unsigned long long)r << 56) | ((unsigned long long)(hash32((unsigned)m) & 0xFFFFFFu) << 32) | (unsigned)m;
}
__device__ __forceinline__ void jp_claim(const SolverArgs& a, int r, const int* list, bool listed, int nlist,
                                         int first, int step) {
    for (int idx = first; idx < nlist; idx += step) {
        const int m = listed ? __ldcg(&list[idx]) : idx;
        if (a.color[m] >= 0) continue;
        const int4 h = a.hdr[m];
        const float2 im = a.inv_mass[m];
        const unsigned long long key = jp_key(r, m);
        if (im.x != 0.f) atomicMax(&a.claim[h.x], key);
        if (im.y != 0.f) atomicMax(&a.claim[h.y], key);
    }
}
__device__ __forceinline__ int jp_assign(const SolverArgs& a, int r, const int* list, bool listed, int nlist,
                                         int first, int step) {
    int left = 0;
    for (int idx = first; idx < nlist; idx += step) {
        const int m = listed ? __ldcg(&list[idx]) : idx;
        if (a.color[m] >= 0) continue;
        const int4 h = a.hdr[m];
        const float2 im = a.inv_mass[m];
        const unsigned long long key = jp_key(r, m);
        const bool okA = im.x == 0.f || __ldcg(&a.claim[h.x]) == key;
        const bool okB = im.y == 0.f || __ldcg(&a.claim[h.y]) == key;
        if (okA && okB) {
            unsigned long long used = 0ull;
            if (im.x != 0.f) used |= __ldcg(&a.mask[h.x]);
            if (im.y != 0.f) used |= __ldcg(&a.mask[h.y]);
            const int c = __ffsll((long long)~used) - 1;
            if (c >= 0 && c < 64) {
                a.color[m] = c;
                if (im.x != 0.f) atomicOr(&a.mask[h.x], 1ull << c);
                if (im.y != 0.f) atomicOr(&a.mask[h.y], 1ull << c);
            } else {
                left++;
            }
        } else {
            left++;
        }
    }
    return left;
}

__global__ void __launch_bounds__(PK_THREADS, 1) k_colour(SolverArgs a) {
    grid_barrier_begin();
    const int nc = *a.d_nc;
    const unsigned nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    // carried colours claim their mask bits; a clash on a body drops the manifold to recolouring.
    // The manifolds left without a colour (new ones, dropped ones) are listed (in pos_of, which the
    // scatter below overwrites), so that the colouring rounds visit only them.
    int dropped = 0;
    const bool carried = *((volatile int*)a.d_new) < nc;
    int* list = a.pos_of;
    unsigned int* list_n = a.bar2.count + 8;  // zeroed by k_reset_solver
    if (carried) {
        const int lane = threadIdx.x & 31;
        for (int m0 = tid - lane; m0 < nc; m0 += stride) {  // warp-uniform: every lane reaches the ballot
            const int m = m0 + lane;
            bool unc = false;
            if (m < nc) {
                const int c = a.color[m];
                if (c < 0) {
                    unc = true;
                } else {
                    const int4 h = a.hdr[m];
                    const float2 im = a.inv_mass[m];
                    const unsigned long long bit = 1ull << c;
                    bool clash = false;
                    if (im.x != 0.f) clash |= (atomicOr(&a.mask[h.x], bit) & bit) != 0ull;
                    if (im.y != 0.f) clash |= (atomicOr(&a.mask[h.y], bit) & bit) != 0ull;
                    if (clash) {
                        a.color[m] = -1;
                        dropped++;
                        unc = true;
                    }
                }
            }
            const unsigned bal = __ballot_sync(0xffffffffu, unc);
            if (bal) {
                int base = 0;
                if (lane == 0) base = (int)atomicAdd(list_n, (unsigned)__popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (unc) list[base + __popc(bal & ((1u << lane) - 1u))] = m;
            }
        }
    }
    for (int o = 16; o; o >>= 1) dropped += __shfl_xor_sync(0xffffffffu, dropped, o);
    if ((threadIdx.x & 31) == 0 && dropped) atomicAdd(a.d_new, dropped);
    if (!grid_barrier(a.bar2, nb, a.spin_limit)) return;
    const int nlist = carried ? (int)*((volatile unsigned int*)list_n) : nc;
    // Jones-Plassmann rounds over the uncoloured manifolds (the highest hashed priority on both of
    // its dynamic bodies takes the smallest colour free on both); statics never conflict.  A short
    // list (new contacts between colourings from scratch) is coloured by block 0 alone, with
    // __syncthreads between the halves of a round instead of grid barriers.
    bool overflow = false;
    if (*((volatile int*)a.d_new) > 0) {
        if (carried && nlist <= JP_LOCAL_MAX) {
            if (blockIdx.x == 0) {
                __shared__ int s_left;
                for (int r = 0; r < B3G_MAX_COLORS; r++) {
                    if (threadIdx.x == 0) s_left = 0;
                    jp_claim(a, r, list, true, nlist, threadIdx.x, blockDim.x);
                    __syncthreads();
                    int left = jp_assign(a, r, list, true, nlist, threadIdx.x, blockDim.x);
                    for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
                    if ((threadIdx.x & 31) == 0 && left) atomicAdd(&s_left, left);
                    __syncthreads();
                    const int l = s_left;
                    __syncthreads();
                    if (l == 0) break;
                    overflow = r == B3G_MAX_COLORS - 1;
                }
            }
            if (!grid_barrier(a.bar2, nb, a.spin_limit)) return;
        } else {
            for (int r = 0; r < B3G_MAX_COLORS; r++) {
                jp_claim(a, r, list, carried, nlist, tid, stride);
                if (!grid_barrier(a.bar2, nb, a.spin_limit)) return;
                int left = jp_assign(a, r, list, carried, nlist, tid, stride);
                for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
                if ((threadIdx.x & 31) == 0 && left) atomicAdd(&a.remaining[r], left);
                if (!grid_barrier(a.bar2, nb, a.spin_limit)) return;
                if (*((volatile int*)&a.remaining[r]) == 0) break;
                overflow = r == B3G_MAX_COLORS - 1;
            }
        }
    }
    // the exact colour set of every body (the masks above may hold bits of dropped carried
    // colours), for the dataflow sweeps; and a stable counting sort by colour (key 64: the
    // manifolds left without one): block g ranks the contiguous chunk [g*chunk, (g+1)*chunk) of
    // manifolds, so that within a colour the records keep manifold order -- the order of the
    // sorted pair list, in which neighbouring manifolds share bodies -- and a warp's manifolds of
    // consecutive colours lie in the same region
    const int G = gridDim.x;
    const int chunk = (nc + G - 1) / G;
    const int lo = min(nc, blockIdx.x * chunk), hi = min(nc, lo + chunk);
    int* cb = a.group_counts;        // [key * G + g]: manifolds of key in block g's chunk
    int* cb_off = cb + 65 * G;       // exclusive scan of cb (key-major)
    __shared__ int s_cnt[65];
    __shared__ int s_warp[PK_THREADS / 32][65];
    for (int k = threadIdx.x; k < 65; k += blockDim.x) s_cnt[k] = 0;
    __syncthreads();
    for (int m = lo + threadIdx.x; m < hi; m += blockDim.x) {
        const int c = a.color[m];
        if (c >= 0 && a.flow_mask) {
            const int4 h = a.hdr[m];
            const float2 im = a.inv_mass[m];
            if (im.x != 0.f) atomicOr(&a.flow_mask[h.x], 1ull << c);
            if (im.y != 0.f) atomicOr(&a.flow_mask[h.y], 1ull << c);
        }
        atomicAdd(&s_cnt[c >= 0 ? c : 64], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 65; k += blockDim.x) cb[k * G + blockIdx.x] = s_cnt[k];
    if (!grid_barrier(a.bar2, nb, a.spin_limit)) return;
    if (blockIdx.x == 0) {
        const int total = block_exclusive_scan(cb, cb_off, 65 * G);
        for (int k = threadIdx.x; k < 65; k += blockDim.x) {
            // (key-major scan: a key's count is the step to the next key's first offset)
            const int o = __ldcg(&cb_off[k * G]);
            a.color_goff[k] = o;
            a.color_fill[k] = (k < 64 ? __ldcg(&cb_off[(k + 1) * G]) : total) - o;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            a.color_goff[65] = total;
            int ncl = 0;
            for (int c = 0; c < 64; c++)
                if (a.color_fill[c] > 0) ncl = c + 1;
            a.counters->num_colors = ncl;
            if (overflow || a.color_fill[64] > 0) atomicOr(&a.counters->status, B3G_FLAG_BATCH_OVERFLOW);
            // carried colours drift upwards as contacts come and go (a new manifold takes the
            // smallest colour its bodies leave free): the next solve colours from scratch again
            // when this one has more than one colour past the last colouring from scratch, and
            // every 8 solves in any case, so that the baseline follows the scene (a colouring
            // from scratch costs about one colour's sweep time on a 262k-box pile; a drifted
            // colouring costs one per extra colour and sweep)
            if (*((volatile int*)a.d_new) >= nc) {
                a.d_prev_n[1] = ncl;
                a.d_prev_n[2] = 0;
                a.d_prev_n[3] = 0;
            } else {
                const int since = ++a.d_prev_n[3];
                if (ncl > a.d_prev_n[1] + 1 || since >= 8) a.d_prev_n[2] = 1;
            }
        }
    }
    if (!grid_barrier(a.bar2, nb, a.spin_limit)) return;
    // positions, in manifold order within each colour: per 512-manifold slice, lane ranks within
    // the warp (match_any), warp offsets from a per-colour scan over the block's warps
    __shared__ int s_run[65];
    for (int k = threadIdx.x; k < 65; k += blockDim.x) s_run[k] = __ldcg(&cb_off[k * G + blockIdx.x]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    for (int base = lo; base < hi; base += blockDim.x) {
        for (int i = threadIdx.x; i < nwarps * 65; i += blockDim.x) (&s_warp[0][0])[i] = 0;
        __syncthreads();
        const int m = base + (int)threadIdx.x;
        const int key = m < hi ? (a.color[m] >= 0 ? a.color[m] : 64) : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (key >= 0 && lane == __ffs(peers) - 1) s_warp[warp][key] = __popc(peers);
        __syncthreads();
        for (int k = threadIdx.x; k < 65; k += blockDim.x) {
            int run = s_run[k];
            for (int w = 0; w < nwarps; w++) {
                const int t = s_warp[w][k];
                s_warp[w][k] = run;
                run += t;
            }
            s_run[k] = run;
        }
        __syncthreads();
        if (key >= 0) {
            const int pos = s_warp[warp][key] + rank;
            a.color_order[pos] = m;
            a.pos_of[m] = pos;
        }
        __syncthreads();
    }
}

// One record of the ordered sweeps: the manifold at position k against the global body deltas.
__device__ __forceinline__ void sweep_record(const SolverArgs& a, int k, int pass, float& res_d, float& res_l) {
    const int4 h = __ldg(&a.hdr_ord[k]);
    const float4 im = __ldg(&a.inv_mass_ord[k]);
    v3 dlA = mk3(0, 0, 0), daA = mk3(0, 0, 0), dlB = mk3(0, 0, 0), daB = mk3(0, 0, 0);
    if (im.x != 0.f) load_dv(a, h.x, dlA, daA);
    if (im.y != 0.f) load_dv(a, h.y, dlB, daB);
    solve_ord(a.sp_ord, k, pass, h.z, im.x, im.y, dlA, daA, dlB, daB, res_d, res_l);
    if (im.x != 0.f) store_dv(a, h.x, dlA, daA);
    if (im.y != 0.f) store_dv(a, h.y, dlB, daB);
}

// the same, as a real call: for the rare uncoloured remainder of k_pgs_flow, whose hot loop keeps
// its registers for the inlined copy
__device__ __noinline__ void sweep_record_call(const SolverArgs& a, int k, int pass, float& res_d, float& res_l) {
    sweep_record(a, k, pass, res_d, res_l);
}

__global__ void __launch_bounds__(PK_THREADS, 1) k_pgs_sweeps(SolverArgs a) {
    grid_barrier_begin();
    const int nc = *a.d_nc;
    const unsigned nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    // position in a grid-wide colour: warp w of block b takes the 32-manifold groups
    // (w * gridDim.x + b) + j * (stride / 32), so a colour smaller than the grid spreads over every SM
    const int ptid = (((int)threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x) * 32 + ((int)threadIdx.x & 31);
    // colour ranges, read once; the trailing run of colours with at most tail_max manifolds each
    // (and the uncoloured remainder) is solved by block 0 alone
    __shared__ int s_off[66];
    for (int i = threadIdx.x; i < 66; i += blockDim.x) s_off[i] = __ldcg(&a.color_goff[i]);
    __syncthreads();
    int ncol = 0;
    for (int c = 0; c < 64; c++)
        if (s_off[c + 1] > s_off[c]) ncol = c + 1;
    int tail = ncol;
    while (tail > 0 && s_off[tail] - s_off[tail - 1] <= a.tail_max) tail--;
    const bool leftovers = s_off[65] > s_off[64];
    // phases per pass: the grid-wide colours, and when there is a tail, its colours plus one
    // phase for the remainder (which ends with the grid barrier)
    const int nphase = (tail < ncol || leftovers) ? ncol + 1 : tail;
    // this thread's first manifold of phase ph (-1: none); its records are prefetched into L1
    // before the barrier that precedes the phase
    auto first_item = [&](int ph) -> int {
        if (ph < tail) {
            const int k = s_off[ph] + ptid;
            return k < s_off[ph + 1] ? k : -1;
        }
        if (ph < ncol && blockIdx.x == 0) {
            const int k = s_off[ph] + (int)threadIdx.x;
            return k < s_off[ph + 1] ? k : -1;
        }
        return -1;
    };
    {
        const int k = first_item(0);
        if (k >= 0) prefetch_manifold(a, k);
    }
    bool ok = true;
    const int npasses = a.interleave ? 1 : 2;
    bool warm_live = a.warm != 0;
    int extra = 0;  // 1 after a dropped warm start: its sweep still counts
    for (int it = a.warm ? -1 : 0; it < a.iterations; it++) {
        float res_d = 0.f, res_l = 0.f;
        const bool warm_pass = it < 0;
        for (int ps = 0; ps < (warm_pass ? 1 : npasses); ps++) {
            const int pass = warm_pass ? 3 : (a.interleave ? 2 : ps);
            // phases of one pass: grid-wide colours [0, tail), then (block 0 only) the trailing
            // colours [tail, ncol) and the uncoloured remainder; one solve call site keeps the
            // register budget of the kernel low
            for (int ph = 0; ph < nphase; ph++) {
                int first, hi, step;
                if (ph < tail) {
                    first = s_off[ph];
                    hi = s_off[ph + 1];
                    if (first == hi) continue;  // uniform across blocks
                    first += ptid;
                    step = stride;
                } else if (ph < ncol) {
                    if (blockIdx.x != 0) continue;
                    first = s_off[ph] + (int)threadIdx.x;
                    hi = s_off[ph + 1];
                    step = blockDim.x;
                } else {  // uncoloured remainder: in order, one thread
                    first = s_off[64];
                    hi = blockIdx.x == 0 && threadIdx.x == 0 ? s_off[65] : first;
                    step = 1;
                }
                for (int k = first; k < hi; k += step) {
                    if (k + step < hi) prefetch_manifold(a, k + step);
                    sweep_record(a, k, pass, res_d, res_l);
                }
                {
                    const int nk = first_item(ph + 1 < nphase ? ph + 1 : 0);
                    if (nk >= 0) prefetch_manifold(a, nk);
                }
                if (ph < tail || ph == ncol) {
                    if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
                } else {
                    __syncthreads();  // block 0 between trailing colours
                }
            }
        }
        if (warm_pass) continue;  // the application pass has no residual
        if (!(a.residual_tol > 0.f || (it == 0 && warm_live) || it == a.iterations - 1)) {
            block_accumulate(a.residual_acc + 2 * (it + extra), res_d, res_l);
            continue;
        }
        double r = 0.0;
        if (end_iteration(a, it + extra, res_d, res_l, ok, &r)) break;
        if (it == 0 && warm_live) {
            warm_live = false;
            // a cold first sweep has residual exactly 1: a warm start that does worse is dropped
            // and the solve restarts cold with the full iteration budget (every block sees the same r)
            if (r > 1.0) {
                for (int i = tid; i < 2 * a.num_bodies; i += stride) __stcg(&a.dv[i], make_float4(0.f, 0.f, 0.f, 0.f));
                for (int k = tid; k < nc; k += stride)
                    for (int j = 0; j < 4; j++) __stcg(&a.sp_ord.imp[(size_t)k * 4 + j], make_float4(0.f, 0.f, 0.f, 0.f));
                if (tid == 0) atomicOr(&a.counters->status, B3G_FLAG_WARM_DISCARDED);
                extra = 1;
                it = -1;
                if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
            }
        }
    }
    if (!ok) return;
    // applied impulses back to manifold order (b3g_read_impulses, the warm-start store), and this
    // solve's manifold keys and colours for the next solve
    for (int k = tid; k < nc; k += stride) {
        const int m = __ldcg(&a.color_order[k]);
        const int4 h = __ldcg(&a.hdr_ord[k]);
        for (int j = 0; j < 4; j++)
            if (h.z & (1 << j)) a.sp.imp[(size_t)m * 4 + j] = __ldcg(&a.sp_ord.imp[(size_t)k * 4 + j]);
        a.prev_key[m] = is_child_manifold(a.manifold_pair, a.d_npairs, m) ? ~0ull : pair_key(h.x, h.y, a.body_bits);
        a.prev_color[m] = a.color[m];
    }
    if (tid == 0) *a.d_prev_n = nc;
    // finish: v += dv for dynamic bodies
    for (int b = tid; b < a.num_bodies; b += stride) {
        if (a.bodies[b].invMass == 0.f) continue;
        v3 dl, da;
        load_dv(a, b, dl, da);
        b3gBody& B = a.bodies_out[b];
        B.linVel.x = B.linVel.x + dl.x;
        B.linVel.y = B.linVel.y + dl.y;
        B.linVel.z = B.linVel.z + dl.z;
        B.angVel.x = B.angVel.x + da.x;
        B.angVel.y = B.angVel.y + da.y;
        B.angVel.z = B.angVel.z + da.z;
    }
}


// ---- dataflow sweeps: the same Gauss-Seidel order as k_pgs_sweeps without a grid barrier per colour.
// A body's manifolds run in colour order, one per colour (a colour holds at most one manifold of a
// dynamic body), so in sweep `it` the manifold of colour c on body b is that body's update number
//   it * popcount(colours of b) + popcount(colours of b below c)
// of the solve.  Each body carries a counter of the updates applied to it; a warp (32 manifolds of
// one colour, which share no dynamic body) waits until both bodies of every lane have reached
// their numbers, solves, and bumps the counters with release semantics after its delta stores.
// The result equals the colour-by-colour sweep bit for bit (every body sees the same sequence of
// updates); a warp only waits on manifolds earlier in (sweep, colour) order, so the earliest
// unfinished warp of the whole grid can always run: no deadlock while every block is resident
// (cooperative launch).  Waits are bounded (spin_limit polls, then the abort flag and the timeout
// status); the records a warp needs are prefetched into L2 before it waits.  The update numbers
// come packed in the record header (k_setup_rows), so a manifold's wait needs no other load.  Used
// when no sweep result decides anything during the solve (no residual tolerance, no warm start to
// check).

__global__ void __launch_bounds__(PK_THREADS, 1) k_pgs_flow(SolverArgs a) {
    grid_barrier_begin();
    const int nc = *a.d_nc;
    const unsigned nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    // warps interleaved across the blocks (as in k_pgs_sweeps): a small colour spreads over every SM
    const int warp = ((int)threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x, nwarps = stride >> 5;
    __shared__ int s_off[66];
    for (int i = threadIdx.x; i < 66; i += blockDim.x) s_off[i] = __ldcg(&a.color_goff[i]);
    __syncthreads();
    int ncol = 0;
    for (int c = 0; c < 64; c++)
        if (s_off[c + 1] > s_off[c]) ncol = c + 1;
    const bool remainder = s_off[65] > s_off[64];
    const int npasses = a.interleave ? 1 : 2;
    bool ok = true;
    for (int it = 0; it < a.iterations && ok; it++) {
        float res_d = 0.f, res_l = 0.f;
        for (int ps = 0; ps < npasses && ok; ps++) {
            const int sweep = it * npasses + ps;  // updates per body so far: sweep * popcount
            const int pass = a.interleave ? 2 : ps;
            for (int c = 0; c < ncol && ok; c++) {
                const int hi = s_off[c + 1];
                for (int k0 = s_off[c] + warp * 32; k0 < hi; k0 += nwarps * 32) {
                    const int k = k0 + lane;
                    const bool act = k < hi;
                    // the dynamic bodies to wait for (-1: none) and their update numbers; the
                    // solve reloads the header from L1
                    int wA = -1, wB = -1;
                    unsigned tA = 0, tB = 0;
                    if (act) {
                        prefetch_manifold(a, k);
                        const int4 h = __ldg(&a.hdr_ord[k]);
                        const float4 im = __ldg(&a.inv_mass_ord[k]);
                        const unsigned f = (unsigned)h.w;
                        if (im.x != 0.f) {
                            wA = h.x;
                            tA = (unsigned)sweep * (f & 127u) + ((f >> 7) & 63u);
                        }
                        if (im.y != 0.f) {
                            wB = h.y;
                            tB = (unsigned)sweep * ((f >> 13) & 127u) + ((f >> 20) & 63u);
                        }
                    }
                    // wait until both bodies of every lane have had their earlier updates
                    unsigned spins = 0;
                    for (;;) {
                        const bool ready = (wA < 0 || ld_acquire_gpu(&a.version[wA]) >= tA) &&
                                           (wB < 0 || ld_acquire_gpu(&a.version[wB]) >= tB);
                        if (__all_sync(0xffffffffu, ready)) break;
                        if (*(volatile unsigned int*)a.bar.abort_flag) {
                            ok = false;
                            break;
                        }
                        if (++spins >= a.spin_limit) {
                            if (lane == 0) {
                                atomicExch(a.bar.abort_flag, 1u);
                                atomicOr(a.bar.status, B3G_FLAG_BARRIER_TIMEOUT);
                            }
                            ok = false;
                            break;
                        }
                        if (spins > 16) __nanosleep(64);
                    }
                    if (!ok) break;
                    if (act) {
                        sweep_record(a, k, pass, res_d, res_l);
                        // release: this thread's delta stores are visible before the counter bump
                        if (wA >= 0) red_release_add_gpu(&a.version[wA], 1u);
                        if (wB >= 0) red_release_add_gpu(&a.version[wB], 1u);
                    }
                }
                ok = ok && !*(volatile unsigned int*)a.bar.abort_flag;
            }
            if (remainder && ok) {
                // manifolds without a colour: after every coloured one of this pass, in order, one
                // thread (they update no counter; the barriers order them)
                if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
                if (tid == 0)
                    for (int k = s_off[64]; k < s_off[65]; k++) sweep_record_call(a, k, pass, res_d, res_l);
                if (!grid_barrier(a.bar, nb, a.spin_limit)) return;
            }
        }
        // this sweep's residual sums (read after the solve; nothing decides on them during it)
        for (int o = 16; o; o >>= 1) {
            res_d += __shfl_xor_sync(0xffffffffu, res_d, o);
            res_l += __shfl_xor_sync(0xffffffffu, res_l, o);
        }
        if (lane == 0) {
            if (res_d != 0.f) atomicAdd(&a.residual_acc[2 * it], (double)res_d);
            if (res_l != 0.f) atomicAdd(&a.residual_acc[2 * it + 1], (double)res_l);
        }
    }
    if (!grid_barrier(a.bar, nb, a.spin_limit) || !ok) return;
    if (tid == 0) {
        const int last = a.iterations - 1;
        const double dd = *((volatile double*)&a.residual_acc[2 * last]);
        const double ll = *((volatile double*)&a.residual_acc[2 * last + 1]);
        a.counters->residual = (float)(sqrt(dd) / fmax(sqrt(ll), 1e-12));
        a.counters->iterations = a.iterations;
    }
    for (int k = tid; k < nc; k += stride) {
        const int m = __ldcg(&a.color_order[k]);
        const int4 h = __ldcg(&a.hdr_ord[k]);
        for (int j = 0; j < 4; j++)
            if (h.z & (1 << j)) a.sp.imp[(size_t)m * 4 + j] = __ldcg(&a.sp_ord.imp[(size_t)k * 4 + j]);
        a.prev_key[m] = is_child_manifold(a.manifold_pair, a.d_npairs, m) ? ~0ull : pair_key(h.x, h.y, a.body_bits);
        a.prev_color[m] = a.color[m];
    }
    if (tid == 0) *a.d_prev_n = nc;
    for (int b = tid; b < a.num_bodies; b += stride) {
        if (a.bodies[b].invMass == 0.f) continue;
        v3 dl, da;
        load_dv(a, b, dl, da);
        b3gBody& B = a.bodies_out[b];
        B.linVel.x = B.linVel.x + dl.x;
        B.linVel.y = B.linVel.y + dl.y;
        B.linVel.z = B.linVel.z + dl.z;
        B.angVel.x = B.angVel.x + da.x;
        B.angVel.y = B.angVel.y + da.y;
        B.angVel.z = B.angVel.z + da.z;
    }
}

__global__ void k_reset_solver(int* color_fill, int* remaining, int* color_cursor, unsigned int* barrier,
                               double* residual_acc, int nres, DevCounters* counters) {
    for (int i = threadIdx.x; i < B3G_MAX_COLORS + 1; i += blockDim.x) {
        color_fill[i] = 0;
        remaining[i] = 0;
        color_cursor[i] = 0;
    }
    for (int i = threadIdx.x; i < nres; i += blockDim.x) residual_acc[i] = 0.0;
    if (threadIdx.x < 4) {
        barrier[threadIdx.x] = 0;       // the sweeps' grid barrier
        barrier[16 + threadIdx.x] = 0;  // k_colour's
    }
    if (threadIdx.x == 0) barrier[24] = 0;  // k_colour's count of manifolds to colour
    if (threadIdx.x == 0) {
        counters->iterations = 0;
        counters->residual = 0.f;
        counters->num_colors = 0;
        counters->new_manifolds = 0;
    }
}

static int solver_grid(DeviceState& d, const void* fn, int blocks_per_sm, size_t smem) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, PK_THREADS, smem);
    if (per_sm < 1) per_sm = 1;
    int want = blocks_per_sm > 0 ? blocks_per_sm : 2;
    if (want > per_sm) want = per_sm;  // cooperative launch: every block must be co-resident
    if (want > B3G_PGS_MAX_BLOCKS_PER_SM) want = B3G_PGS_MAX_BLOCKS_PER_SM;
    return want * d.num_sms;
}

cudaError_t solver_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_solve_pgs<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         B3G_PGS_MAX_SMEM);
    if (e != cudaSuccess) return e;
    // the colour-ordered sweeps use < 1 KB of shared memory: the rest of the SM's 256 KB as L1
    // for the prefetched records
    e = cudaFuncSetAttribute(k_pgs_sweeps, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_pgs_flow, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_solve_pgs<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, B3G_PGS_MAX_SMEM);
}

int launch_solver(DeviceState& d, const b3gConfig& cfg, float dt, cudaStream_t s) {
    int launches = 0;
    long long ll = 0;
    const int grid = d.num_sms * 4;
    int iters = cfg.solver_iterations > 0 ? cfg.solver_iterations : 1;
    // residual_acc holds 2 doubles per sweep for 4096 sweeps: a dropped warm start adds one sweep
    if (iters > 4095) iters = 4095;
    int* d_nc = &d.counters->num_contacts;
    int* d_n2 = &d.counters->pad[1];
    // per-step resets
    cudaMemsetAsync(d.dv, 0, sizeof(float4) * 2 * (size_t)d.num_bodies, s);
    const bool jac = cfg.solver_mode == B3G_SOLVER_JACOBI;
    cudaMemsetAsync(d.color_claim, 0, sizeof(unsigned long long) * (jac ? 2 : 4) * (size_t)d.num_bodies, s);
    cudaMemsetAsync(d.body_manifold_count, 0, sizeof(int) * (size_t)d.num_bodies, s);
    int* color_fill = d.color_offsets + (B3G_MAX_COLORS + 2);
    int* remaining = color_fill + (B3G_MAX_COLORS + 1);
    int* color_cursor = remaining + (B3G_MAX_COLORS + 1);
    k_reset_solver<<<1, 256, 0, s>>>(color_fill, remaining, color_cursor, d.barrier, d.residual_acc, 2 * (iters + 1),
                                     d.counters);
    launches++;

    SolverArgs a;
    a.bodies = d.bodies;
    a.inertias = d.inertias;
    a.slots = d.contact_slots;
    a.manifold_pair = d.manifold_pair;
    a.d_npairs = &d.counters->pad[0];
    a.d_nc = d_nc;
    a.sp = d.sp;
    a.sp_ord = d.sp_ord;
    a.hdr = d.manifold_hdr;
    a.inv_mass = d.manifold_inv_mass;
    a.hdr_ord = d.manifold_hdr_ord;
    a.inv_mass_ord = d.manifold_inv_mass_ord;
    a.inertia_ord = d.inertia_ord;
    a.dv = d.dv;
    a.dv_sum = d.dv_sum;
    a.split = d.split_dv;
    a.body_count = d.body_manifold_count;
    a.list_off = d.body_list_offsets;
    a.list = nullptr;
    a.color = d.manifold_color;
    a.color_order = d.color_order;
    a.color_offsets = d.color_offsets;
    a.color_fill = color_fill;
    a.color_cursor = color_cursor;
    a.remaining = remaining;
    a.sorted_bodies = nullptr;
    a.body_slot = d.body_slot;
    a.manifold_group = d.manifold_group;
    a.group_counts = d.group_counts;
    a.group_seg = 0;
    a.num_dynamic = 0;
    a.chunk = 1;
    a.use_smem = 0;
    a.tile_R = 0;
    a.interleave = cfg.pgs_interleave ? 1 : 0;
    a.ws_features = cfg.warm_start != 0 ? d.ws_features : nullptr;
    a.ws_rows_cap = d.ws_rows_cap;
    a.ws_rows = a.ws_features ? d.ws_rows : nullptr;
    a.gx = cfg.gravity[0];
    a.gy = cfg.gravity[1];
    a.gz = cfg.gravity[2];
    const int wm = cfg.warm_start;
    const bool ws_learned = (wm == B3G_WARM_LEARNED || wm == B3G_WARM_PERSISTENT_LEARNED) && d.ws_model && a.ws_features;
    const bool ws_persist = wm == B3G_WARM_PERSISTENT || wm == B3G_WARM_PERSISTENT_LEARNED;
    a.warm = (cfg.solver_mode == B3G_SOLVER_PGS && (ws_learned || ws_persist)) ? 1 : 0;
    a.claim = d.color_claim;
    a.mask = d.color_claim + d.num_bodies;
    a.claim_x = d.color_claim + 2 * (size_t)d.num_bodies;
    a.mask_x = d.color_claim + 3 * (size_t)d.num_bodies;
    a.bodies_out = d.bodies;
    a.counters = d.counters;
    a.residual_acc = d.residual_acc;
    a.num_bodies = d.num_bodies;
    a.mode = cfg.solver_mode;
    a.iterations = iters;
    a.residual_tol = cfg.residual_tol;
    a.dt = dt;
    a.erp = cfg.erp;
    a.threshold = cfg.contact_threshold;
    a.bar.count = d.barrier;
    a.bar.gen = d.barrier + 1;
    a.bar.abort_flag = d.barrier + 2;
    a.bar.status = &d.counters->status;
    a.spin_limit = cfg.barrier_spin_limit > 0 ? (unsigned)cfg.barrier_spin_limit : B3G_BARRIER_SPIN_LIMIT;
    a.pos_of = nullptr;
    a.prev_key = d.prev_mkey;
    a.prev_color = d.prev_mcolor;
    a.d_prev_n = d.prev_mn;
    a.d_new = &d.counters->new_manifolds;
    a.color_goff = d.color_offsets;
    a.body_bits = d.body_bits;
    a.tail_max = cfg.pgs_tail_manifolds > 0 ? cfg.pgs_tail_manifolds : 32;
    a.bar2.count = d.barrier + 16;
    a.bar2.gen = d.barrier + 17;
    a.bar2.abort_flag = d.barrier + 18;
    a.bar2.status = &d.counters->status;
    a.flow_mask = nullptr;
    a.version = nullptr;
    // PGS work split: the autotuner's choice (b3g_autotune) when the config says AUTO, else the
    // split measured fastest on GB300 for 256k-box piles -- grid-wide colours, coloured before
    // the row setup (records written in colour order)
    const int pgs_mode = cfg.pgs_partitions != B3G_PGS_PARTITIONS_AUTO ? cfg.pgs_partitions
                         : d.tune.pgs_partitions > 0                   ? d.tune.pgs_partitions
                                                                       : B3G_PGS_PARTITIONS_NONE;
    const bool ordered = cfg.solver_mode == B3G_SOLVER_PGS && pgs_mode == B3G_PGS_PARTITIONS_NONE;
    const int cgrid = ordered ? solver_grid(d, (const void*)k_pgs_sweeps, cfg.solver_blocks_per_sm, 0) : 0;
    // dataflow sweeps where no sweep's residual decides anything during the solve
    const bool flow = ordered && !(cfg.residual_tol > 0.f) && !a.warm && cfg.pgs_flow == 1;
    if (ordered) {
        a.pos_of = d.manifold_pos;
        a.color_fill = color_fill;
        a.color_cursor = color_cursor;
        if (flow) {  // the per-body colour sets and update counters of the dataflow sweeps
            a.flow_mask = d.color_claim + 2 * (size_t)d.num_bodies;            // zeroed above each solve
            a.version = reinterpret_cast<unsigned int*>(d.body_manifold_count);  // zeroed above each solve
        }
        k_manifold_prep<<<grid, SV_THREADS, 0, s>>>(a);
        launches++;
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(cgrid);
        lc.blockDim = dim3(PK_THREADS);
        lc.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        cudaError_t e = cudaLaunchKernelEx(&lc, k_colour, a);
        if (e != cudaSuccess && d.launch_error == cudaSuccess) d.launch_error = e;
        launches++;
    }

    if (cfg.solver_mode == B3G_SOLVER_JACOBI) {
        const uint32_t sentinel = (1u << d.body_bits) - 1u;
        k_count_manifolds<<<grid, SV_THREADS, 0, s>>>(d.contact_slots, d.manifold_pair, d_nc, d.bodies,
                                                      d.body_manifold_count, d.jac_keys[0], d.jac_vals[0], sentinel,
                                                      d_n2);
        launches++;
        int w = radix_sort_u32(d.prim, d.jac_keys[0], d.jac_keys[1], d.jac_vals[0], d.jac_vals[1], d_n2, d.body_bits,
                               d.sort_scratch, s, &ll);
        a.list = d.jac_vals[w];
        exclusive_scan_i32(d.prim, d.body_manifold_count, d.body_list_offsets, d.d_num_bodies, nullptr,
                           d.scan_scratch, s, &ll);
    }
    k_setup_rows<<<grid * 4, SV_THREADS, 0, s>>>(a);  // a thread per contact point
    launches++;
    if (wm != B3G_WARM_COLD && d.ws_init) {
        // initial impulses: persisting points from the previous solve, the others from the network
        WarmFill w;
        w.pred = nullptr;
        w.tnorm = nullptr;
        if (ws_learned && a.warm) {
            launches += mlp::forward_device(*d.ws_model, d.ws_features, 12, d.ws_rows, d.ws_rows_cap, s);
            w.pred = mlp::last_predictions(*d.ws_model);
            w.tnorm = mlp::target_norm(*d.ws_model);
        }
        w.d_nc = d_nc;
        w.rows_cap = d.ws_rows_cap;
        w.hdr = d.manifold_hdr;
        w.sp = d.sp;
        w.slots = d.contact_slots;
        w.manifold_pair = d.manifold_pair;
        w.d_npairs = &d.counters->pad[0];
        w.body_bits = d.body_bits;
        w.prev_keys = d.prev_keys;
        w.prev_pts = d.prev_pts;
        w.prev_imp = d.prev_imp;
        w.prev_n = d.prev_n;
        w.persist = ws_persist ? 1 : 0;
        w.factor = cfg.warm_start_factor > 0.f ? cfg.warm_start_factor : 1.f;
        w.predict_all = wm == B3G_WARM_LEARNED ? 1 : 0;
        w.write_imp = a.warm;
        w.init = d.ws_init;
        w.is_new = d.ws_new;
        w.pos_of = a.pos_of;
        w.imp_ord = d.sp_ord.imp;
        k_warm_fill<<<grid, SV_THREADS, 0, s>>>(w);
        launches++;
    }

    // PGS partitions: a contiguous range of the cell-ordered dynamic bodies per block, the range's
    // body deltas and world inverse inertias in shared memory when they fit (60 B per body)
    size_t smem = 0;
    int sgrid = 0;
    const int bps = cfg.solver_blocks_per_sm;
    if (jac) {
        sgrid = solver_grid(d, (const void*)k_solve_jacobi, bps, 0);
    } else if (ordered) {
        sgrid = cgrid;
    } else {
        const int mode = pgs_mode;
        const bool parts = mode != B3G_PGS_PARTITIONS_NONE;
        const int nd = parts && d.cell_sorted_bodies ? d.num_dynamic : 0;
        sgrid = solver_grid(d, (const void*)k_solve_pgs<true>, bps, 0);
        const int chunk = nd > 0 ? (nd + sgrid - 1) / sgrid : 1;
        const size_t owned = ((size_t)chunk * 15 * sizeof(float) + 15) & ~(size_t)15;
        const bool shared_mode = mode == B3G_PGS_PARTITIONS_SHARED || mode == B3G_PGS_PARTITIONS_STREAMED;
        smem = owned;
        if (nd == 0 || !shared_mode || chunk >= 0xffff || smem > (size_t)B3G_PGS_MAX_SMEM) smem = 0;
        // streamed tiles: two buffers of R manifolds in what shared memory is left
        int R = 0;
        const size_t tile_extra = 16 + 8 * (size_t)B3G_PGS_MAX_TILES;  // mbarriers, tile list
        if (smem > 0 && mode == B3G_PGS_PARTITIONS_STREAMED && owned + tile_extra < (size_t)B3G_PGS_MAX_SMEM) {
            size_t r = ((size_t)B3G_PGS_MAX_SMEM - owned - tile_extra) / (2 * (size_t)B3G_PGS_TILE_BYTES);
            if (r > (size_t)PK_THREADS) r = PK_THREADS;
            R = (int)(r & ~(size_t)31);
            if (R < 32) R = 0;
        }
        if (R > 0) smem = owned + 2 * (size_t)R * B3G_PGS_TILE_BYTES + tile_extra;
        // keep the grid co-resident: drop the shared-memory use if it would cost occupancy
        if (smem > 0 && solver_grid(d, (const void*)k_solve_pgs<true>, bps, smem) != sgrid) {
            smem = 0;
            R = 0;
        }
        a.sorted_bodies = d.cell_sorted_bodies;
        a.num_dynamic = nd;
        a.chunk = chunk;
        a.use_smem = smem > 0 ? 1 : 0;
        a.tile_R = R;
        a.group_seg = sgrid * 64 + 64 + 2;
        cudaMemsetAsync(d.group_counts, 0, sizeof(int) * 3 * (size_t)a.group_seg, s);
    }
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(sgrid);
    lc.blockDim = dim3(PK_THREADS);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    cudaError_t e = jac                 ? cudaLaunchKernelEx(&lc, k_solve_jacobi, a)
                    : flow              ? cudaLaunchKernelEx(&lc, k_pgs_flow, a)
                    : ordered           ? cudaLaunchKernelEx(&lc, k_pgs_sweeps, a)
                    : a.num_dynamic > 0 ? cudaLaunchKernelEx(&lc, k_solve_pgs<true>, a)
                                        : cudaLaunchKernelEx(&lc, k_solve_pgs<false>, a);
    if (e != cudaSuccess && d.launch_error == cudaSuccess) d.launch_error = e;
    launches++;
    if (wm != B3G_WARM_COLD && d.prev_keys) {  // this solve's impulses for the next step's persisting points
        k_warm_store<<<grid, SV_THREADS, 0, s>>>(d_nc, d.ws_rows_cap, d.manifold_hdr, d.contact_slots, d.manifold_pair,
                                                 &d.counters->pad[0], d.sp.imp, d.body_bits, d.prev_keys, d.prev_pts, d.prev_imp,
                                                 d.prev_n);
        launches++;
    }
    return launches + (int)ll;
}

}  // namespace b3g
