// Joint stage: point-to-point and fixed joints, solved right before the contacts.
//
// The reference solves joints in a separate PGS pass before the contact solver
// (b3GpuRigidBodyPipeline.cpp:361-374 -> b3GpuPgsConstraintSolver::solveJoints,
// b3GpuPgsConstraintSolver.cpp:927-944): 4 iterations at dt 1/60, erp 0.2, damping 1, cfm 0,
// one kernel launch per batch and iteration over a greedy batching of the joints, then the
// break check and the velocity write-back.  Here the whole stage is ONE launch:
//
//   1. rows: one thread per joint builds its 3 (point to point) or 6 (fixed) rows from the
//      bodies' current state (getInfo2Kernel, kernels/jointSolver.cl:651-870) and zeroes both
//      bodies' velocity deltas;
//   2. iterations x batches: the joints of a batch share no dynamic body, so a batch is one
//      parallel sweep (solveJointConstraintRows, jointSolver.cl:303-329), then a block or grid
//      barrier;
//   3. break check (breakViolatedConstraintsKernel, jointSolver.cl:352-371) and write-back of the
//      deltas into the bodies' velocities (writeBackVelocitiesKernel, jointSolver.cl:631-648).
//
// Small joint sets run as one block (__syncthreads between batches); large ones as a cooperative
// grid with the bounded grid barrier.  Arithmetic follows the reference kernels operation by
// operation (float, no contraction), so results equal the CPU restatement bit for bit.
#include <cfloat>

#include "common.cuh"
#include "world_internal.h"

namespace b3g {

namespace {

constexpr int JT_THREADS = 256;
constexpr float JT_INFINITY = 1e30f;  // B3_INFINITY of jointSolver.cl

struct JArgs {
    b3gBody* bodies;
    const b3gInertia* inertias;
    b3gJoint* joints;
    JointHdr* hdr;       // 1 per joint
    JointRow* rows;      // 6 per joint
    float* imp;          // 6 per joint: applied impulses
    float4* dv;          // 2 per body: delta linear, delta angular velocity
    const int* order;    // joint indices, batch by batch
    const int* batch_off;
    const int* uniq;     // every body some joint names, once
    int num_joints, num_batches, num_uniq, iterations;
    float dt, erp, damping, cfm;
    GridBarrier bar;
    unsigned int spin_limit;
};

struct v3j {
    float x, y, z;
};
__device__ __forceinline__ v3j mkj(float x, float y, float z) { return v3j{x, y, z}; }
__device__ __forceinline__ float dotj(v3j a, v3j b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3j xyz(float4 a) { return mkj(a.x, a.y, a.z); }
__device__ __forceinline__ v3j xyz(const b3gFloat4& a) { return mkj(a.x, a.y, a.z); }
__device__ __forceinline__ float4 q4(const b3gFloat4& a) { return make_float4(a.x, a.y, a.z, a.w); }

// qtMul / qtRotate / qtInvert of jointSolver.cl:222-262
__device__ __forceinline__ float4 jq_mul(float4 a, float4 b) {
    float4 r;
    r.x = (a.y * b.z - a.z * b.y) + (a.w * b.x + b.w * a.x);
    r.y = (a.z * b.x - a.x * b.z) + (a.w * b.y + b.w * a.y);
    r.z = (a.x * b.y - a.y * b.x) + (a.w * b.z + b.w * a.z);
    r.w = a.w * b.w - (a.x * b.x + a.y * b.y + a.z * b.z);
    return r;
}
__device__ __forceinline__ float4 jq_inv(float4 q) { return make_float4(-q.x, -q.y, -q.z, q.w); }
__device__ __forceinline__ v3j jq_rot(float4 q, float4 v) {
    const float4 t = jq_mul(jq_mul(q, make_float4(v.x, v.y, v.z, 0.f)), jq_inv(q));
    return mkj(t.x, t.y, t.z);
}

// mtMul1 (matrix x column vector) and mtMul3 (row vector x matrix), jointSolver.cl:54-76
__device__ __forceinline__ v3j mt_mul1(const b3gMat3& m, v3j b) {
    return mkj(dotj(xyz(m.row[0]), b), dotj(xyz(m.row[1]), b), dotj(xyz(m.row[2]), b));
}
__device__ __forceinline__ v3j mt_mul3(v3j a, const b3gMat3& m) {
    return mkj(dotj(a, mkj(m.row[0].x, m.row[1].x, m.row[2].x)), dotj(a, mkj(m.row[0].y, m.row[1].y, m.row[2].y)),
               dotj(a, mkj(m.row[0].z, m.row[1].z, m.row[2].z)));
}

// acos for the fixed joints' angle: asin's Maclaurin series (coefficients (2n)!/(4^n n!^2 (2n+1)),
// 12 terms, Horner form) with the half-angle identities acos(x) = 2 asin(sqrt((1-x)/2)) for
// x > 1/2, pi - 2 asin(sqrt((1+x)/2)) for x < -1/2 and pi/2 - asin(x) between.  Within 1.3 ulp of
// the exact value on [-1, 1]; the CPU restatement evaluates the same operations, so the two agree
// bit for bit.
__constant__ float c_asin[11] = {0.166666672f,   0.075000003f,   0.0446428582f,  0.030381944f,
                                 0.0223721582f,  0.0173527636f,  0.0139648439f,  0.0115518011f,
                                 0.00976160914f, 0.00839033537f, 0.007312526f};
__device__ __forceinline__ float asin_series(float z) {
    const float t = z * z;
    float p = c_asin[10];
#pragma unroll
    for (int i = 9; i >= 0; --i) p = c_asin[i] + t * p;
    return z + (z * t) * p;
}
__device__ __forceinline__ float joint_acos(float x) {
    if (x > 0.5f) return 2.0f * asin_series(sqrtf((1.0f - x) * 0.5f));
    if (x < -0.5f) return 3.14159274f - 2.0f * asin_series(sqrtf((1.0f + x) * 0.5f));
    return 1.57079637f - asin_series(x);
}

// calculateDiffAxisAngleQuaternion with nearest / getAngle / b3Acos (jointSolver.cl:543-590)
__device__ void diff_axis_angle(float4 orn0, float4 orn1a, v3j& axis, float& angle) {
    const float4 d = make_float4(orn0.x - orn1a.x, orn0.y - orn1a.y, orn0.z - orn1a.z, orn0.w - orn1a.w);
    const float4 s = make_float4(orn0.x + orn1a.x, orn0.y + orn1a.y, orn0.z + orn1a.z, orn0.w + orn1a.w);
    const float dd = d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w;
    const float ss = s.x * s.x + s.y * s.y + s.z * s.z + s.w * s.w;
    const float4 orn1 = dd < ss ? orn1a : make_float4(-orn1a.x, -orn1a.y, -orn1a.z, -orn1a.w);
    const float4 dorn = jq_mul(orn1, jq_inv(orn0));
    float w = dorn.w;
    if (w >= 1.f) w = 1.f;
    if (w < -1.f) w = -1.f;
    angle = 2.f * joint_acos(w);
    axis = mkj(dorn.x, dorn.y, dorn.z);
    const float len = dotj(axis, axis);
    if (len < FLT_EPSILON * FLT_EPSILON) {
        axis = mkj(1.f, 0.f, 0.f);
    } else {
        const float r = sqrtf(len);
        axis = mkj(axis.x / r, axis.y / r, axis.z / r);
    }
}

__device__ __forceinline__ int joint_rows(int type) {
    return type == B3G_JOINT_FIXED ? 6 : type == B3G_JOINT_POINT2POINT ? 3 : 0;
}

// Axes of row j: linear Jacobian n, angular Jacobians r1 (body A) and r2 (body B).  Rows 0-2 of
// getInfo2Point2Point: n = unit axis, r1 = skew row of -a1, r2 = skew row of a2; rows 3-5 of
// getInfo2FixedOrientation: n = 0, r1 = unit axis, r2 = -unit axis (jointSolver.cl:479-486,
// 488-541, 592-628).  Setup and sweeps both rebuild the rows through this function.
__device__ __forceinline__ void row_axes(int j, v3j m1, v3j a2, v3j& n, v3j& r1, v3j& r2) {
    const int e = j < 3 ? j : j - 3;
    if (j < 3) {
        n = mkj(e == 0 ? 1.f : 0.f, e == 1 ? 1.f : 0.f, e == 2 ? 1.f : 0.f);
        r1 = e == 0 ? mkj(0.f, -m1.z, m1.y) : e == 1 ? mkj(m1.z, 0.f, -m1.x) : mkj(-m1.y, m1.x, 0.f);
        r2 = e == 0 ? mkj(0.f, -a2.z, a2.y) : e == 1 ? mkj(a2.z, 0.f, -a2.x) : mkj(-a2.y, a2.x, 0.f);
    } else {
        n = mkj(0.f, 0.f, 0.f);
        r1 = mkj(e == 0 ? 1.f : 0.f, e == 1 ? 1.f : 0.f, e == 2 ? 1.f : 0.f);
        r2 = mkj(e == 0 ? -1.f : 0.f, e == 1 ? -1.f : 0.f, e == 2 ? -1.f : 0.f);
    }
}

// getInfo2Kernel for joint i: rows, then the finalize loop (limits, angular components,
// jacDiagABInv, rhs from the positional error and the bodies' current velocities)
__device__ void joint_setup(const JArgs& a, int i) {
    const b3gJoint c = a.joints[i];
    const int nr = joint_rows(c.type);
    if (nr == 0) return;
    const int A = c.rbA, B = c.rbB;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    a.dv[2 * A] = z4;
    a.dv[2 * A + 1] = z4;
    a.dv[2 * B] = z4;
    a.dv[2 * B + 1] = z4;
    const b3gBody bA = a.bodies[A], bB = a.bodies[B];
    const float k = (1.f / a.dt) * a.erp;
    // getInfo2Point2Point: J1 linear = identity rows, J1 angular = skew(-a1), J2 angular = skew(a2),
    // rhs k (a2 + posB - a1 - posA); getInfo2FixedOrientation: J1 angular = identity rows, J2
    // angular = -identity rows, rhs k axis (-angle).  Each row is rebuilt inside the finalize loop.
    const float4 qA = q4(bA.quat), qB = q4(bB.quat);
    const v3j a1 = jq_rot(qA, q4(c.pivotInA)), a2 = jq_rot(qB, q4(c.pivotInB));
    const v3j m1 = mkj(-a1.x, -a1.y, -a1.z);
    const v3j err = mkj(((a2.x + bB.pos.x) - a1.x) - bA.pos.x, ((a2.y + bB.pos.y) - a1.y) - bA.pos.y,
                        ((a2.z + bB.pos.z) - a1.z) - bA.pos.z);
    v3j ang = mkj(0.f, 0.f, 0.f);
    if (nr == 6) {
        v3j axis;
        float angle;
        diff_axis_angle(q4(c.relTargetAB), jq_mul(qA, jq_inv(qB)), axis, angle);
        const float na = -angle;
        ang = mkj(axis.x * na, axis.y * na, axis.z * na);
    }
    const b3gMat3 IA = a.inertias[A].invInertiaWorld, IB = a.inertias[B].invInertiaWorld;
    const v3j vA = xyz(bA.linVel), wA = xyz(bA.angVel), vB = xyz(bB.linVel), wB = xyz(bB.angVel);
    JointRow* out = a.rows + 6 * (size_t)i;
    float* imp = a.imp + 6 * (size_t)i;
    // every row's limits: +-infinity clamped to the breaking threshold
    float lo = -JT_INFINITY, hi = JT_INFINITY;
    if (hi >= c.breakingImpulseThreshold) hi = c.breakingImpulseThreshold;
    if (lo <= -c.breakingImpulseThreshold) lo = -c.breakingImpulseThreshold;
#pragma unroll 1
    for (int j = 0; j < nr; ++j) {
        v3j n, r1, r2;
        row_axes(j, m1, a2, n, r1, r2);
        const int e = j < 3 ? j : j - 3;
        const float rhs = j < 3 ? k * (e == 0 ? err.x : e == 1 ? err.y : err.z)
                                : k * (e == 0 ? ang.x : e == 1 ? ang.y : ang.z);
        const v3j angA = mt_mul1(IA, r1), angB = mt_mul1(IB, r2);
        const v3j lA = mkj(n.x * bA.invMass, n.y * bA.invMass, n.z * bA.invMass);
        const v3j lB = mkj(n.x * bB.invMass, n.y * bB.invMass, n.z * bB.invMass);
        float sum = dotj(lA, n);
        sum += dotj(mt_mul3(r1, IA), r1);
        sum += dotj(lB, n);
        sum += dotj(mt_mul3(r2, IB), r2);
        const float jinv = fabsf(sum) > FLT_EPSILON ? 1.f / sum : 0.f;
        const float vel1 = dotj(n, vA) + dotj(r1, wA);
        const float vel2 = -dotj(n, vB) + dotj(r2, wB);
        const float rel = vel1 + vel2;
        const float pen = rhs * jinv;
        const float vimp = (0.f - rel * a.damping) * jinv;
        JointRow r;
        r.angA_rhs = make_float4(angA.x, angA.y, angA.z, pen + vimp);
        r.angB_jinv = make_float4(angB.x, angB.y, angB.z, jinv);
        out[j] = r;
        imp[j] = 0.f;
    }
    JointHdr h;
    h.m1_lo = make_float4(m1.x, m1.y, m1.z, lo);
    h.a2_hi = make_float4(a2.x, a2.y, a2.z, hi);
    h.A = A;
    h.B = B;
    h.active_rows = (c.flags & 1) ? nr : 0;  // the flags change only in the break check, after the sweeps
    h.imA = bA.invMass;
    h.imB = bB.invMass;
    h.pad[0] = h.pad[1] = h.pad[2] = 0;
    a.hdr[i] = h;
}

// resolveSingleConstraintRowGeneric over a joint's rows (jointSolver.cl:273-301); the deltas stay in
// registers across the rows.  A static body's deltas stay exactly zero (its inverse mass and world
// inverse inertia are zero), so they are not stored: joints of one batch may share a static body.
__device__ void joint_solve(const JArgs& a, int ci) {
    const JointHdr h = a.hdr[ci];
    const int nr = h.active_rows;
    if (nr == 0) return;
    const int A = h.A, B = h.B;
    const float imA = h.imA, imB = h.imB;
    const v3j m1 = xyz(h.m1_lo), a2 = xyz(h.a2_hi);
    const float lo = h.m1_lo.w, hi = h.a2_hi.w;
    float4 dlA = a.dv[2 * A], daA = a.dv[2 * A + 1], dlB = a.dv[2 * B], daB = a.dv[2 * B + 1];
    const JointRow* rows = a.rows + 6 * (size_t)ci;
    float* imp = a.imp + 6 * (size_t)ci;
    for (int j = 0; j < nr; ++j) {
        v3j n, r1, r2;
        row_axes(j, m1, a2, n, r1, r2);
        const JointRow r = rows[j];
        const float applied = imp[j], jinv = r.angB_jinv.w;
        float delta = r.angA_rhs.w - applied * a.cfm;
        const float d1 = dotj(n, xyz(dlA)) + dotj(r1, xyz(daA));
        const float d2 = -dotj(n, xyz(dlB)) + dotj(r2, xyz(daB));
        delta -= d1 * jinv;
        delta -= d2 * jinv;
        const float sum = applied + delta;
        float now;
        if (sum < lo) {
            delta = lo - applied;
            now = lo;
        } else if (sum > hi) {
            delta = hi - applied;
            now = hi;
        } else {
            now = sum;
        }
        imp[j] = now;
        dlA.x += (n.x * imA) * delta;
        dlA.y += (n.y * imA) * delta;
        dlA.z += (n.z * imA) * delta;
        daA.x += r.angA_rhs.x * delta;
        daA.y += r.angA_rhs.y * delta;
        daA.z += r.angA_rhs.z * delta;
        dlB.x += (-n.x * imB) * delta;
        dlB.y += (-n.y * imB) * delta;
        dlB.z += (-n.z * imB) * delta;
        daB.x += r.angB_jinv.x * delta;
        daB.y += r.angB_jinv.y * delta;
        daB.z += r.angB_jinv.z * delta;
    }
    if (imA != 0.f) {
        a.dv[2 * A] = dlA;
        a.dv[2 * A + 1] = daA;
    }
    if (imB != 0.f) {
        a.dv[2 * B] = dlB;
        a.dv[2 * B + 1] = daB;
    }
}

__device__ __forceinline__ bool sync_all(const JArgs& a) {
    if (gridDim.x == 1) {
        __syncthreads();
        return true;
    }
    return grid_barrier(a.bar, gridDim.x, a.spin_limit);
}

__global__ void __launch_bounds__(JT_THREADS) k_joints(JArgs a) {
    grid_barrier_begin();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nth = gridDim.x * blockDim.x;
    for (int i = tid; i < a.num_joints; i += nth) joint_setup(a, i);
    if (!sync_all(a)) return;
    for (int it = 0; it < a.iterations; ++it) {
        for (int b = 0; b < a.num_batches; ++b) {
            const int lo = a.batch_off[b], hi = a.batch_off[b + 1];
            for (int k = lo + tid; k < hi; k += nth) joint_solve(a, a.order[k]);
            if (!sync_all(a)) return;
        }
    }
    // breakViolatedConstraintsKernel: any row whose accumulated impulse reached the threshold
    for (int i = tid; i < a.num_joints; i += nth) {
        const int nr = joint_rows(a.joints[i].type);
        const float thr = a.joints[i].breakingImpulseThreshold;
        for (int j = 0; j < nr; ++j)
            if (fabsf(a.imp[6 * (size_t)i + j]) >= thr) a.joints[i].flags = 0;
    }
    // writeBackVelocitiesKernel for the bodies the joints name (the others' deltas are zero)
    for (int u = tid; u < a.num_uniq; u += nth) {
        const int b = a.uniq[u];
        b3gBody& body = a.bodies[b];
        if (body.invMass != 0.f) {
            const float4 dl = a.dv[2 * b], da = a.dv[2 * b + 1];
            body.linVel.x += dl.x;
            body.linVel.y += dl.y;
            body.linVel.z += dl.z;
            body.angVel.x += da.x;
            body.angVel.y += da.y;
            body.angVel.z += da.z;
        }
    }
}

// inverse masses of both bodies of every joint, for the host batching
__global__ void k_joint_masses(const b3gBody* bodies, const b3gJoint* joints, int n, float2* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float2(bodies[joints[i].rbA].invMass, bodies[joints[i].rbB].invMass);
}

}  // namespace

long long launch_joint_masses(const DeviceState& d, int n, float2* out, cudaStream_t s) {
    if (n <= 0) return 0;
    k_joint_masses<<<(n + 255) / 256, 256, 0, s>>>(d.bodies, d.joints, n, out);
    return 1;
}

long long launch_joints(DeviceState& d, const b3gConfig& cfg, cudaStream_t s) {
    if (d.num_joints <= 0) return 0;
    JArgs a;
    a.bodies = d.bodies;
    a.inertias = d.inertias;
    a.joints = d.joints;
    a.hdr = d.joint_hdr;
    a.rows = d.joint_rows;
    a.imp = d.joint_imp;
    a.dv = d.joint_dv;
    a.order = d.joint_order;
    a.batch_off = d.joint_batch_off;
    a.uniq = d.joint_uniq;
    a.num_joints = d.num_joints;
    a.num_batches = d.num_joint_batches;
    a.num_uniq = d.num_joint_uniq;
    // b3GpuPgsConstraintSolver::solveJoints' fixed solver settings (b3GpuPgsConstraintSolver.cpp:930-937,
    // b3ContactSolverInfo defaults erp 0.2, damping 1, globalCfm 0)
    a.iterations = 4;
    a.dt = 1.f / 60.f;
    a.erp = 0.2f;
    a.damping = 1.f;
    a.cfm = 0.f;
    a.bar.count = d.barrier + 8;
    a.bar.gen = d.barrier + 9;
    a.bar.abort_flag = d.barrier + 10;
    a.bar.status = &d.counters->status;
    a.spin_limit = cfg.barrier_spin_limit > 0 ? (unsigned)cfg.barrier_spin_limit : B3G_BARRIER_SPIN_LIMIT;
    // one block while the widest batch fits it; else a co-resident grid of up to two blocks per SM
    // (262,144 joints in 2 batches: 0.35 ms at one block per SM, 0.27 ms at two, 0.33 ms at three,
    // where the extra arrivals at each grid barrier cost more than the extra warps hide)
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_joints, JT_THREADS, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        if (per_sm > 2) per_sm = 2;
    }
    int grid = (d.max_joint_batch + JT_THREADS - 1) / JT_THREADS;
    if (grid < 1) grid = 1;
    if (grid > d.num_sms * per_sm) grid = d.num_sms * per_sm;
    long long n = 0;
    if (grid > 1) {
        cudaMemsetAsync(d.barrier + 8, 0, 3 * sizeof(unsigned int), s);
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(grid);
        lc.blockDim = dim3(JT_THREADS);
        lc.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        cudaError_t e = cudaLaunchKernelEx(&lc, k_joints, a);
        if (e != cudaSuccess && d.launch_error == cudaSuccess) d.launch_error = e;
    } else {
        k_joints<<<1, JT_THREADS, 0, s>>>(a);
    }
    n++;
    return n;
}

}  // namespace b3g
