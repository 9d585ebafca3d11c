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

__global__ void __launch_bounds__(256) k_integrate(b3gBody* __restrict__ bodies, b3gInertia* __restrict__ inertias,
                                                   int n, float dt, float damping, float gx, float gy, float gz,
                                                   int update_inertia, unsigned int* __restrict__ status) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        b3gBody b = bodies[i];
        if (b.invMass == 0.f) continue;
        const float threshold = 0.25f * 3.14159254f;
        b.angVel.x *= damping;
        b.angVel.y *= damping;
        b.angVel.z *= damping;
        v3 w = mk3(b.angVel.x, b.angVel.y, b.angVel.z);
        float fAngle = sqrtf(dot3(w, w));
        if (fAngle * dt > threshold) fAngle = threshold / dt;
        v3 axis;
        if (fAngle < 0.001f)
            axis = w * (0.5f * dt - (dt * dt * dt) * 0.020833333333f * fAngle * fAngle);
        else
            axis = w * (sinf(0.5f * fAngle * dt) / fAngle);
        quat dorn{axis.x, axis.y, axis.z, cosf(fAngle * dt * 0.5f)};
        quat q = qmul(dorn, f4q(b.quat));
        float len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
        if (len > 0.f) {
            float inv = 1.f / len;
            q = quat{q.x * inv, q.y * inv, q.z * inv, q.w * inv};
        } else {
            q = quat{0.f, 0.f, 0.f, 1.f};
        }
        b.quat = b3gFloat4{q.x, q.y, q.z, q.w};
        b.pos.x = b.pos.x + b.linVel.x * dt;
        b.pos.y = b.pos.y + b.linVel.y * dt;
        b.pos.z = b.pos.z + b.linVel.z * dt;
        b.linVel.x = b.linVel.x + gx * dt;
        b.linVel.y = b.linVel.y + gy * dt;
        b.linVel.z = b.linVel.z + gz * dt;
        if (!(b.pos.x == b.pos.x && b.pos.y == b.pos.y && b.pos.z == b.pos.z)) atomicOr(status, B3G_FLAG_NAN);
        bodies[i] = b;
        if (update_inertia) {
            b3gInertia I = inertias[i];
            m33 R = qmat(q);
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
}

int launch_integrate(DeviceState& d, const b3gConfig& cfg, float dt, cudaStream_t s) {
    // one body per thread in a single wave (the kernel is latency-bound: a dependent chain per body)
    const int grid = std::max(1, std::min((d.num_bodies + 255) / 256, d.num_sms * 32));
    k_integrate<<<grid, 256, 0, s>>>(d.bodies, d.inertias, d.num_bodies, dt, cfg.angular_damping,
                                              cfg.gravity[0], cfg.gravity[1], cfg.gravity[2], cfg.update_world_inertia,
                                              &d.counters->status);
    return 1;
}

}  // namespace b3g
