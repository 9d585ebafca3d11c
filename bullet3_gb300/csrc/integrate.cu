// Transform integration.
//
// Reference: integrateTransformsKernel (src/Bullet3OpenCL/RigidBody/kernels/integrateKernel.cl:24-32) ->
// integrateSingleTransform (src/Bullet3Dynamics/shared/b3IntegrateTransforms.h:5-55): angular damping,
// angular motion clamp |w|*dt <= pi/4, exponential-map quaternion update (Taylor branch for |w| < 0.001),
// normalisation, then x += v*dt, then v += g*dt; bodies with invMass 0 are skipped.
// Optional (off by default, as in the reference which freezes it at registration,
// b3GpuNarrowPhase.cpp:899-901): refresh the world inverse inertia R diag(I0^-1) R^T.
#include <algorithm>

#include "common.cuh"
#include "world_internal.h"

namespace b3g {

// One step of one dynamic body on its 5 float4 (pos, quat, linVel, angVel, [collidable, invMass,
// restitution, friction]) in place.
__device__ __forceinline__ void integrate_body(float4* b, float dt, float damping, float gx, float gy, float gz,
                                               unsigned int* status) {
    const float threshold = 0.25f * 3.14159254f;
    float4 av = b[3];
    av.x *= damping;
    av.y *= damping;
    av.z *= damping;
    v3 w = mk3(av.x, av.y, av.z);
    float fAngle = sqrtf(dot3(w, w));
    if (fAngle * dt > threshold) fAngle = threshold / dt;
    v3 axis;
    if (fAngle < 0.001f)
        axis = w * (0.5f * dt - (dt * dt * dt) * 0.020833333333f * fAngle * fAngle);
    else
        axis = w * (sinf(0.5f * fAngle * dt) / fAngle);
    const float4 q0 = b[1];
    quat dorn{axis.x, axis.y, axis.z, cosf(fAngle * dt * 0.5f)};
    quat q = qmul(dorn, quat{q0.x, q0.y, q0.z, q0.w});
    float len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (len > 0.f) {
        float inv = 1.f / len;
        q = quat{q.x * inv, q.y * inv, q.z * inv, q.w * inv};
    } else {
        q = quat{0.f, 0.f, 0.f, 1.f};
    }
    float4 p = b[0], lv = b[2];
    p.x = p.x + lv.x * dt;
    p.y = p.y + lv.y * dt;
    p.z = p.z + lv.z * dt;
    lv.x = lv.x + gx * dt;
    lv.y = lv.y + gy * dt;
    lv.z = lv.z + gz * dt;
    if (!(p.x == p.x && p.y == p.y && p.z == p.z)) atomicOr(status, B3G_FLAG_NAN);
    b[0] = p;
    b[1] = make_float4(q.x, q.y, q.z, q.w);
    b[2] = lv;
    b[3] = av;
}

// A block stages its 256 bodies (80 B each, 20 KB) through shared memory so that the global reads
// and writes are coalesced float4 streams; each thread integrates one body there.
constexpr int IT_THREADS = 256;
__global__ void __launch_bounds__(IT_THREADS) k_integrate(b3gBody* __restrict__ bodies,
                                                          b3gInertia* __restrict__ inertias, int n, float dt,
                                                          float damping, float gx, float gy, float gz,
                                                          int update_inertia, unsigned int* __restrict__ status) {
    __shared__ float4 s[IT_THREADS * 5];
    float4* g = reinterpret_cast<float4*>(bodies);
    for (int base = blockIdx.x * IT_THREADS; base < n; base += gridDim.x * IT_THREADS) {
        const int cnt = min(IT_THREADS, n - base);
        for (int j = threadIdx.x; j < 5 * cnt; j += IT_THREADS) s[j] = g[5 * (size_t)base + j];
        __syncthreads();
        const int i = base + (int)threadIdx.x;
        if ((int)threadIdx.x < cnt && s[5 * threadIdx.x + 4].y != 0.f) {  // invMass: skip statics
            float4* b = s + 5 * threadIdx.x;
            integrate_body(b, dt, damping, gx, gy, gz, status);
            if (update_inertia) {
                b3gInertia I = inertias[i];
                const float4 qq = b[1];
                m33 R = qmat(quat{qq.x, qq.y, qq.z, qq.w});
                v3 d = mk3(I.initInvInertia.row[0].x, I.initInvInertia.row[1].y, I.initInvInertia.row[2].z);
                v3 c0 = mk3(R.r0.x * d.x, R.r1.x * d.x, R.r2.x * d.x);
                v3 c1 = mk3(R.r0.y * d.y, R.r1.y * d.y, R.r2.y * d.y);
                v3 c2 = mk3(R.r0.z * d.z, R.r1.z * d.z, R.r2.z * d.z);
                // (R diag(d)) R^T: row r of the product = sum_k (R diag d)[r][k] * R[c][k]
                v3 rows[3] = {mk3(c0.x, c1.x, c2.x), mk3(c0.y, c1.y, c2.y), mk3(c0.z, c1.z, c2.z)};
                for (int r = 0; r < 3; r++) {
                    I.invInertiaWorld.row[r].x = dot3(rows[r], R.r0);
                    I.invInertiaWorld.row[r].y = dot3(rows[r], R.r1);
                    I.invInertiaWorld.row[r].z = dot3(rows[r], R.r2);
                }
                inertias[i] = I;
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < 5 * cnt; j += IT_THREADS) g[5 * (size_t)base + j] = s[j];
        __syncthreads();
    }
}

int launch_integrate(DeviceState& d, const b3gConfig& cfg, float dt, cudaStream_t s) {
    // one body per thread in a single wave
    const int grid = std::max(1, std::min((d.num_bodies + IT_THREADS - 1) / IT_THREADS, d.num_sms * 32));
    k_integrate<<<grid, IT_THREADS, 0, s>>>(d.bodies, d.inertias, d.num_bodies, dt, cfg.angular_damping,
                                              cfg.gravity[0], cfg.gravity[1], cfg.gravity[2], cfg.update_world_inertia,
                                              &d.counters->status);
    return 1;
}

}  // namespace b3g
