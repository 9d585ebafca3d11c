// Shared device helpers for the GPU rigid-body step.
//
// Arithmetic convention: every physics translation unit is compiled with --fmad=false
// and IEEE division/square root, and every formula below fixes its evaluation order.
// The CPU oracle restates the same formulas in the same order (compiled with
// -ffp-contract=off), so the AABB, broadphase, SAT, clipping, reduction and solver
// stages reproduce the oracle bit-for-bit; only the integrator's sinf/cosf differ.
#ifndef B3G_COMMON_CUH
#define B3G_COMMON_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include "b3g_types.h"
#include "b3g_capi.h"

#define B3G_DEV __device__ __forceinline__
#define B3G_HD __host__ __device__ __forceinline__

struct v3 {
    float x, y, z;
};

B3G_HD v3 mk3(float x, float y, float z) { return v3{x, y, z}; }
B3G_HD v3 f4v3(const b3gFloat4& a) { return v3{a.x, a.y, a.z}; }
B3G_HD v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
B3G_HD v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
B3G_HD v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
B3G_HD v3 operator*(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
B3G_HD v3 operator*(float s, v3 a) { return v3{s * a.x, s * a.y, s * a.z}; }
B3G_HD float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
B3G_HD v3 cross3(v3 a, v3 b) {
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// v * (1/|v|): b3Vector3::normalized / normalize scale by the reciprocal length
// (Bullet3Common/b3Vector3.h:260-300, :791-803)
B3G_HD v3 normalize3(v3 a) {
    float inv = 1.0f / sqrtf(dot3(a, a));
    return v3{a.x * inv, a.y * inv, a.z * inv};
}

struct quat {
    float x, y, z, w;
};
B3G_HD quat f4q(const b3gFloat4& a) { return quat{a.x, a.y, a.z, a.w}; }

// Hamilton product a*b
B3G_HD quat qmul(quat a, quat b) {
    quat r;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
    r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    return r;
}
B3G_HD quat qconj(quat a) { return quat{-a.x, -a.y, -a.z, a.w}; }

// 3x3 rotation matrix rows from a quaternion (b3Matrix3x3::setRotation order).
struct m33 {
    v3 r0, r1, r2;
};
B3G_HD m33 qmat(quat q) {
    float d = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    float s = 2.0f / d;
    float xs = q.x * s, ys = q.y * s, zs = q.z * s;
    float wx = q.w * xs, wy = q.w * ys, wz = q.w * zs;
    float xx = q.x * xs, xy = q.x * ys, xz = q.x * zs;
    float yy = q.y * ys, yz = q.y * zs, zz = q.z * zs;
    m33 m;
    m.r0 = v3{1.0f - (yy + zz), xy - wz, xz + wy};
    m.r1 = v3{xy + wz, 1.0f - (xx + zz), yz - wx};
    m.r2 = v3{xz - wy, yz + wx, 1.0f - (xx + yy)};
    return m;
}
B3G_HD v3 mmul(const m33& m, v3 v) { return v3{dot3(m.r0, v), dot3(m.r1, v), dot3(m.r2, v)}; }
// transpose(m) * v
B3G_HD v3 mtmul(const m33& m, v3 v) {
    return v3{m.r0.x * v.x + m.r1.x * v.y + m.r2.x * v.z, m.r0.y * v.x + m.r1.y * v.y + m.r2.y * v.z,
              m.r0.z * v.x + m.r1.z * v.y + m.r2.z * v.z};
}
// rotate v by q: matrix form, used everywhere a world/local transform is needed
B3G_HD v3 qrot(quat q, v3 v) { return mmul(qmat(q), v); }
B3G_HD v3 qrot_inv(quat q, v3 v) { return mtmul(qmat(q), v); }
B3G_HD v3 xform(v3 p, v3 pos, quat q) { return qrot(q, p) + pos; }

// b3Quaternion * b3Vector3 (Bullet3Common/b3Quaternion.h:651-729, scalar branch)
B3G_HD quat qmulv(quat q, v3 w) {
    return quat{q.w * w.x + q.y * w.z - q.z * w.y, q.w * w.y + q.z * w.x - q.x * w.z,
                q.w * w.z + q.x * w.y - q.y * w.x, -q.x * w.x - q.y * w.y - q.z * w.z};
}
// b3QuatRotate (b3Quaternion.h:868-879): (q * v) * q^-1, the form the SAT and clipping code uses
B3G_HD v3 qrotq(quat q, v3 v) {
    quat t = qmul(qmulv(q, v), qconj(q));
    return v3{t.x, t.y, t.z};
}
// b3Matrix3x3::getRotation (b3Matrix3x3.h:392-491, scalar branch): matrix -> quaternion
B3G_HD quat quat_from_mat(const m33& m) {
    float e[3][3] = {{m.r0.x, m.r0.y, m.r0.z}, {m.r1.x, m.r1.y, m.r1.z}, {m.r2.x, m.r2.y, m.r2.z}};
    float t[4];
    float trace = e[0][0] + e[1][1] + e[2][2];
    if (trace > 0.0f) {
        float s = sqrtf(trace + 1.0f);
        t[3] = s * 0.5f;
        s = 0.5f / s;
        t[0] = (e[2][1] - e[1][2]) * s;
        t[1] = (e[0][2] - e[2][0]) * s;
        t[2] = (e[1][0] - e[0][1]) * s;
    } else {
        int i = e[0][0] < e[1][1] ? (e[1][1] < e[2][2] ? 2 : 1) : (e[0][0] < e[2][2] ? 2 : 0);
        int j = (i + 1) % 3, k = (i + 2) % 3;
        float s = sqrtf(e[i][i] - e[j][j] - e[k][k] + 1.0f);
        t[i] = s * 0.5f;
        s = 0.5f / s;
        t[3] = (e[k][j] - e[j][k]) * s;
        t[j] = (e[j][i] + e[i][j]) * s;
        t[k] = (e[k][i] + e[i][k]) * s;
    }
    return quat{t[0], t[1], t[2], t[3]};
}
// transpose, product and rigid-transform helpers with b3Matrix3x3 / b3Transform operation order
B3G_HD m33 mtrans(const m33& m) {
    m33 r;
    r.r0 = v3{m.r0.x, m.r1.x, m.r2.x};
    r.r1 = v3{m.r0.y, m.r1.y, m.r2.y};
    r.r2 = v3{m.r0.z, m.r1.z, m.r2.z};
    return r;
}
// m1 * m2: element (i,j) = m2.tdot_j(m1[i]) (b3Matrix3x3.h:1190-1272)
B3G_HD v3 mrow_times(const v3& a, const m33& m2) {
    return v3{m2.r0.x * a.x + m2.r1.x * a.y + m2.r2.x * a.z, m2.r0.y * a.x + m2.r1.y * a.y + m2.r2.y * a.z,
              m2.r0.z * a.x + m2.r1.z * a.y + m2.r2.z * a.z};
}
B3G_HD m33 mmul33(const m33& m1, const m33& m2) {
    m33 r;
    r.r0 = mrow_times(m1.r0, m2);
    r.r1 = mrow_times(m1.r1, m2);
    r.r2 = mrow_times(m1.r2, m2);
    return r;
}
// b3Transform::inverse applied to a point: basis^T p + basis^T (-origin) (b3Transform.h:182-186)
B3G_HD v3 xform_inv(const m33& R, v3 origin, v3 p) {
    m33 t = mtrans(R);
    return mmul(t, p) + mmul(t, -origin);
}

// inverse inertia matrix (3 float4 rows in memory)
// b3TransformAabb2 (Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h:24-43): a local box moved
// by a pose, centre by the rotation matrix, extent by its absolute value
B3G_HD void transform_aabb(const b3gAabb& local, v3 pos, quat q, float margin, v3& mn, v3& mx) {
    v3 lmin = mk3(local.minv[0], local.minv[1], local.minv[2]);
    v3 lmax = mk3(local.maxv[0], local.maxv[1], local.maxv[2]);
    v3 he = 0.5f * (lmax - lmin);
    he = he + mk3(margin, margin, margin);
    v3 lc = 0.5f * (lmax + lmin);
    m33 m = qmat(q);
    m33 a;
    a.r0 = mk3(fabsf(m.r0.x), fabsf(m.r0.y), fabsf(m.r0.z));
    a.r1 = mk3(fabsf(m.r1.x), fabsf(m.r1.y), fabsf(m.r1.z));
    a.r2 = mk3(fabsf(m.r2.x), fabsf(m.r2.y), fabsf(m.r2.z));
    v3 c = mmul(m, lc) + pos;
    v3 e = mk3(dot3(he, a.r0), dot3(he, a.r1), dot3(he, a.r2));
    mn = c - e;
    mx = c + e;
}

B3G_HD v3 imul(const b3gMat3& m, v3 v) {
    return v3{m.row[0].x * v.x + m.row[0].y * v.y + m.row[0].z * v.z,
              m.row[1].x * v.x + m.row[1].y * v.y + m.row[1].z * v.z,
              m.row[2].x * v.x + m.row[2].y * v.y + m.row[2].z * v.z};
}

// ---- uniform grid hashing (broadphase and ray casts)
B3G_DEV uint32_t cell_hash(int x, int y, int z, int bits, int mask) {
    return ((uint32_t)(z & mask) << (2 * bits)) | ((uint32_t)(y & mask) << bits) | (uint32_t)(x & mask);
}

// Per-scene shift of the integer cell coordinates (batched independent scenes).  A constant shift
// keeps a scene's neighbour cells neighbours after the wrap of cell_hash, so the 27-cell search
// stays complete within the scene, while different scenes that occupy the same region of space
// land in different cells of the hashed grid.  Cross-scene entries that still share a cell are
// rejected by the scene test of the pair kernel.
struct CellShift {
    int x, y, z;
};
B3G_DEV CellShift scene_shift(int scene, int bits) {
    uint32_t r = (uint32_t)scene * 0x9E3779B1u;
    r ^= r >> 15;
    r *= 0x85EBCA77u;
    r ^= r >> 13;
    const int mask = (1 << bits) - 1;
    return CellShift{(int)(r & mask), (int)((r >> bits) & mask), (int)((r >> (2 * bits)) & mask)};
}

B3G_DEV float4 ldg4(const b3gFloat4* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// ----------------------------------------------------------------------------------------
// Bounded grid barrier for persistent cooperative kernels.
//
// Every wait is capped: after B3G_BARRIER_SPIN_LIMIT polls a block raises the abort flag
// and the barrier returns false in every block (they all poll the abort flag), so a
// kernel can unwind and the host sees B3G_FLAG_BARRIER_TIMEOUT instead of a hang.
struct GridBarrier {
    unsigned int* count;      // arrivals since the launch started (reset to 0 before each launch)
    unsigned int* gen;        // unused (kept for layout)
    unsigned int* abort_flag; // non-zero once any block gave up
    unsigned int* status;     // device status word
};

#ifndef B3G_BARRIER_SPIN_LIMIT
#define B3G_BARRIER_SPIN_LIMIT (1u << 22)
#endif

B3G_DEV unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

B3G_DEV void red_release_add_gpu(unsigned int* p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Barriers this block has passed in the current launch (thread 0's count; the kernel zeroes it
// with grid_barrier_begin before its first barrier).
B3G_DEV unsigned int& grid_barrier_epoch() {
    __shared__ unsigned int s_epoch;
    return s_epoch;
}
B3G_DEV void grid_barrier_begin() {
    if (threadIdx.x == 0) grid_barrier_epoch() = 0;
}

// Grid-wide barrier of a cooperative launch: one arrival counter that only grows during the
// launch (zeroed before the launch); the n-th barrier completes when it reaches n * nblocks.
// Arrival is a fire-and-forget release add, waiting is acquire loads of the counter.  A wait
// gives up after spin_limit polls (or when another block gave up): it raises the abort flag and
// the timeout status bit and returns false, and every later barrier of the launch returns false.
B3G_DEV bool grid_barrier(const GridBarrier& b, unsigned int nblocks, unsigned int spin_limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned int target = (++grid_barrier_epoch()) * nblocks;
        red_release_add_gpu(b.count, 1u);
        unsigned int spins = 0;
        while (ld_acquire_gpu(b.count) < target) {
            if (*(volatile unsigned int*)b.abort_flag) { ok = 0; break; }
            if (++spins >= spin_limit) {
                atomicExch(b.abort_flag, 1u);
                atomicOr(b.status, B3G_FLAG_BARRIER_TIMEOUT);
                ok = 0;
                break;
            }
            if (spins > 64) __nanosleep(32);
        }
        // (a block that reaches the target without waiting needs no abort check: every block
        // arrived, so none gave up before this barrier; a later barrier sees any later abort)
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

#endif
