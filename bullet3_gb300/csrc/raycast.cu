// Ray casts against the world's bodies.
//
// Reference: b3GpuRigidBodyPipeline::castRays -> b3GpuRaycast::castRays
// (src/Bullet3OpenCL/Raycast/b3GpuRaycast.cpp:248-373); per ray, rayCastPairsKernel / rayCastKernel
// (kernels/rayCastKernels.cl:261-439): the closest hit among hulls (rayConvex, :157-217, in the
// body's frame) and spheres (sphere_intersect, :224-248); planes and other shapes are skipped; a body
// equal to the input hit's m_hitResult2 is skipped.  The reference finds candidate bodies with a
// parallel linear BVH over the AABBs; here the candidates come from the broadphase's own uniform
// grid: one thread per ray walks the grid cells the segment crosses, in order (3-D DDA in double
// precision), and tests the bodies of each crossed cell's 3x3x3 neighbourhood -- a body's AABB never
// reaches beyond the neighbours of its centre's cell, so every body the segment can hit is seen.
// The walk stops once the next cell starts beyond the best hit so far.  Static bodies are tested by
// every ray of their scene.  The closest hit wins; equal fractions go to the lower body index (the
// reference's sequential loop keeps the first).  Every test uses the reference kernel's arithmetic
// (qtRotate quaternion form, the same operation order), so results match the CPU restatement bit for
// bit.  The grid is rebuilt from the current bodies first (AABBs, cell sort, run starts).
#include <algorithm>
#include <cfloat>
#include <climits>

#include "common.cuh"
#include "world_internal.h"

namespace b3g {

struct RayArgs {
    const float4* rays;     // 2 per ray: from, to
    b3gRayHit* hits;
    const uint32_t* order;  // rays in Morton order of their origin cell (thread i casts ray order[i])
    const b3gAabb* aabbs;   // world AABBs of the current poses
    int n;
    const b3gBody* bodies;
    const b3gCollidable* cols;
    const b3gHull* hulls;
    const b3gFace* faces;
    const uint32_t* keys;   // cell hashes in sorted order
    const uint32_t* vals;   // dynamic bodies in cell order
    const uint32_t* cell_start;
    int n_dyn;
    float inv_cell;
    int bits;
    const int* body_scene;  // nullptr: one scene
    int num_scenes;
    const int* large_list;
    const int* large_off;   // nullptr: [0, num_large)
    int num_large;
    const int* sap_list;
    const int* sap_off;
};

// qtMul / qtRotate of rayCastKernels.cl:101-131
__device__ __forceinline__ quat cl_qmul(quat a, quat b) {
    quat r;
    r.x = (a.y * b.z - a.z * b.y) + (a.w * b.x + b.w * a.x);
    r.y = (a.z * b.x - a.x * b.z) + (a.w * b.y + b.w * a.y);
    r.z = (a.x * b.y - a.y * b.x) + (a.w * b.z + b.w * a.z);
    r.w = a.w * b.w - (a.x * b.x + a.y * b.y + a.z * b.z);
    return r;
}
__device__ __forceinline__ v3 cl_qrot(quat q, v3 v) {
    const quat t = cl_qmul(cl_qmul(q, quat{v.x, v.y, v.z, 0.f}), quat{-q.x, -q.y, -q.z, q.w});
    return mk3(t.x, t.y, t.z);
}

// rayConvex with the fraction starting at 1 (the caller keeps the closest)
__device__ bool ray_convex(v3 from, v3 to, const b3gFace* faces, int nf, float& hit, v3& normal) {
    float exitFraction = 1.f, enterFraction = -0.3f;
    v3 cur = mk3(0.f, 0.f, 0.f);
    bool result = true;
    for (int i = 0; i < nf && result; i++) {
        const float4 p = __ldg(reinterpret_cast<const float4*>(&faces[i].plane));
        const v3 n = mk3(p.x, p.y, p.z);
        const float fromd = dot3(from, n) + p.w;
        const float tod = dot3(to, n) + p.w;
        if (fromd < 0.f) {
            if (tod >= 0.f) {
                const float fraction = fromd / (fromd - tod);
                if (exitFraction > fraction) exitFraction = fraction;
            }
        } else {
            if (tod < 0.f) {
                const float fraction = fromd / (fromd - tod);
                if (enterFraction <= fraction) {
                    enterFraction = fraction;
                    cur = n;
                }
            } else {
                result = false;
            }
        }
        if (exitFraction <= enterFraction) result = false;
    }
    if (enterFraction < 0.f) result = false;
    if (result) {
        hit = enterFraction;
        normal = cur;
    }
    return result;
}

__device__ __forceinline__ bool ray_sphere(v3 c, float radius, v3 from, v3 to, float& hit) {
    const v3 rs = from - c, d = to - from;
    const float A = dot3(d, d), B = dot3(rs, d), C = dot3(rs, rs) - radius * radius;
    const float D = B * B - A * C;
    if (D > 0.f) {
        const float t = (-B - sqrtf(D)) / A;
        if (t >= 0.f && t < 1.f) {
            hit = t;
            return true;
        }
    }
    return false;
}

struct RayBest {
    float t;
    int b;
    v3 normal;  // hull: face normal (body frame); sphere: from the centre to the hit point
};

// Conservative rejection: does the segment, up to the best fraction so far, come within a margin
// of the body's world AABB?  The body lies inside that AABB, so a body rejected here cannot be
// hit at a fraction <= best; the margin (1e-3 + 1e-4 x the coordinate's magnitude) is far above
// the rounding of the exact tests, so no hit is lost and the results do not change.
__device__ __forceinline__ bool ray_near_aabb(const RayArgs& a, int j, v3 from, v3 to, float tmax) {
    const float4 mn = __ldg(reinterpret_cast<const float4*>(a.aabbs) + 2 * j);
    const float4 mx = __ldg(reinterpret_cast<const float4*>(a.aabbs) + 2 * j + 1);
    const float f[3] = {from.x, from.y, from.z}, d[3] = {to.x - from.x, to.y - from.y, to.z - from.z};
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    float t0 = 0.f, t1 = tmax;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float m = 1e-3f + 1e-4f * fmaxf(fabsf(lo[k]), fabsf(hi[k]));
        const float l = lo[k] - m, h = hi[k] + m;
        if (fabsf(d[k]) < 1e-20f) {
            if (f[k] < l || f[k] > h) return false;
            continue;
        }
        const float inv = 1.f / d[k];
        float ta = (l - f[k]) * inv, tb = (h - f[k]) * inv;
        if (ta > tb) { const float t = ta; ta = tb; tb = t; }
        t0 = fmaxf(t0, ta - 1e-4f);
        t1 = fminf(t1, tb + 1e-4f);
        if (t0 > t1) return false;
    }
    return true;
}

__device__ __forceinline__ void ray_test(const RayArgs& a, int j, v3 from, v3 to, int ignore, RayBest& best) {
    if (j == ignore) return;
    const b3gBody& B = a.bodies[j];
    const b3gCollidable c = a.cols[B.collidableIdx];
    float t;
    v3 n;
    if (c.shapeType == B3G_SHAPE_CONVEX_HULL) {
        const float4 q4 = ldg4(&B.quat), p4 = ldg4(&B.pos);
        const quat inv{-q4.x, -q4.y, -q4.z, q4.w};
        const v3 invPos = cl_qrot(inv, mk3(-p4.x, -p4.y, -p4.z));
        const v3 lf = cl_qrot(inv, from) + invPos, lt = cl_qrot(inv, to) + invPos;
        const b3gHull& h = a.hulls[c.shapeIndex];
        if (h.numFaces == 0 || !ray_convex(lf, lt, a.faces + h.faceOffset, h.numFaces, t, n)) return;
    } else if (c.shapeType == B3G_SHAPE_SPHERE) {
        const float4 p4 = ldg4(&B.pos);
        const v3 centre = mk3(p4.x, p4.y, p4.z);
        if (!ray_sphere(centre, c.radius, from, to, t)) return;
        const float s = 1.f - t;
        const v3 hp = mk3(s * from.x + t * to.x, s * from.y + t * to.y, s * from.z + t * to.z);
        n = hp - centre;
    } else {
        return;  // planes and other shapes are not ray-cast (rayCastKernels.cl)
    }
    if (t < best.t || (t == best.t && j < best.b)) {
        best.t = t;
        best.b = j;
        best.normal = n;
    }
}

__global__ void __launch_bounds__(128) k_cast_rays(RayArgs a) {
    const int mask = (1 << a.bits) - 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const int r = (int)a.order[i];
        const float4 f4 = a.rays[2 * r], t4 = a.rays[2 * r + 1];
        const v3 from = mk3(f4.x, f4.y, f4.z), to = mk3(t4.x, t4.y, t4.z);
        const int ignore = a.hits[r].hitResult2;
        int scene = 0;
        if (a.num_scenes > 1) {
            scene = (int)f4.w;
            if (scene < 0 || scene >= a.num_scenes) scene = -1;  // no scene: nothing to hit
        }
        RayBest best{1.f, INT_MAX, mk3(0.f, 0.f, 0.f)};
        if (scene >= 0) {
            // static bodies of the ray's scene
            const int l0 = a.large_off ? a.large_off[scene] : 0, l1 = a.large_off ? a.large_off[scene + 1] : a.num_large;
            for (int l = l0; l < l1; l++) ray_test(a, a.large_list[l], from, to, ignore, best);
            for (int l = a.sap_off[scene]; l < a.sap_off[scene + 1]; l++) ray_test(a, a.sap_list[l], from, to, ignore, best);
            // dynamic bodies: walk the grid cells along the segment
            CellShift sh{0, 0, 0};
            if (a.body_scene) sh = scene_shift(scene, a.bits);
            const double ic = (double)a.inv_cell;
            const double o[3] = {(double)from.x * ic, (double)from.y * ic, (double)from.z * ic};
            const double d[3] = {((double)to.x - (double)from.x) * ic, ((double)to.y - (double)from.y) * ic,
                                 ((double)to.z - (double)from.z) * ic};
            int c[3], step[3];
            double tmax[3], tdelta[3];
            for (int k = 0; k < 3; k++) {
                c[k] = (int)floor(o[k]);
                if (d[k] > 0.0) {
                    step[k] = 1;
                    tdelta[k] = 1.0 / d[k];
                    tmax[k] = ((double)c[k] + 1.0 - o[k]) / d[k];
                } else if (d[k] < 0.0) {
                    step[k] = -1;
                    tdelta[k] = -1.0 / d[k];
                    tmax[k] = ((double)c[k] - o[k]) / d[k];
                } else {
                    step[k] = 0;
                    tdelta[k] = DBL_MAX;
                    tmax[k] = DBL_MAX;
                }
            }
            const int max_cells = (int)(fabs(d[0]) + fabs(d[1]) + fabs(d[2])) + 4;
            // the bodies whose centre cell lies within one cell of a visited cell: the whole 3x3x3
            // neighbourhood of the first cell, then per step only the 3x3 slab that enters it (the
            // union is the same set, each cell scanned once; the best hit is the minimum of
            // (fraction, body index), so the order of the tests does not matter)
            int entered = -1;  // axis of the last step (-1: the first cell)
            const int step0 = step[0], step1 = step[1], step2 = step[2];
            for (int visit = 0; visit < max_cells; visit++) {
                const int ulo = entered < 0 ? -1 : 0, uhi = entered < 0 ? 1 : 0;
                for (int u = ulo; u <= uhi; u++)
                    for (int v = -1; v <= 1; v++)
                        for (int w = -1; w <= 1; w++) {
                            // offsets from the cell: the full cube, or the entered slab (fixed one
                            // step ahead along the stepped axis, the other two axes spanning -1..1)
                            const int ox = entered == 0 ? step0 : w;
                            const int oy = entered == 1 ? step1 : (entered == 0 ? w : v);
                            const int oz = entered == 2 ? step2 : (entered < 0 ? u : v);
                            const uint32_t h = cell_hash(c[0] + ox + sh.x, c[1] + oy + sh.y, c[2] + oz + sh.z,
                                                         a.bits, mask);
                            const uint32_t s0 = __ldg(&a.cell_start[h]);
                            if (s0 >= (uint32_t)a.n_dyn || __ldg(&a.keys[s0]) != h) continue;
                            if (s0 > 0 && __ldg(&a.keys[s0 - 1]) == h) continue;
                            for (uint32_t q = s0; q < (uint32_t)a.n_dyn && __ldg(&a.keys[q]) == h; q++) {
                                const int j = (int)__ldg(&a.vals[q]);
                                if (a.body_scene && __ldg(&a.body_scene[j]) != scene) continue;
                                if (!ray_near_aabb(a, j, from, to, best.t)) continue;
                                ray_test(a, j, from, to, ignore, best);
                            }
                        }
                // the next cell along the segment; stop once it starts beyond the best hit
                const int k = tmax[0] <= tmax[1] ? (tmax[0] <= tmax[2] ? 0 : 2) : (tmax[1] <= tmax[2] ? 1 : 2);
                const double tn = tmax[k];
                if (tn > 1.0 || tn > (double)best.t) break;
                c[k] += step[k];
                tmax[k] += tdelta[k];
                entered = k;
            }
        }
        b3gRayHit& out = a.hits[r];
        out.hitFraction = 1.f;
        if (best.b != INT_MAX) {
            const float t = best.t, s = 1.f - t;
            const v3 hp = mk3(s * from.x + t * to.x, s * from.y + t * to.y, s * from.z + t * to.z);
            const v3 n = best.normal * (1.0f / sqrtf(dot3(best.normal, best.normal)));
            out.hitFraction = t;
            out.hitBody = best.b;
            out.hitPoint = b3gFloat4{hp.x, hp.y, hp.z, 0.f};
            out.hitNormal = b3gFloat4{n.x, n.y, n.z, 0.f};
        }
    }
}

__global__ void k_set_int(int* p, int v) { *p = v; }
void launch_set_int(int* p, int v, cudaStream_t s) { k_set_int<<<1, 1, 0, s>>>(p, v); }

// Morton code of the grid cell of each ray's origin (10 bits per axis), for the ray order
__device__ __forceinline__ uint32_t ray_spread3(uint32_t x) {
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}
__global__ void k_ray_keys(const float4* __restrict__ rays, int n, float inv_cell, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const float4 f = rays[2 * r];
        const uint32_t cx = (uint32_t)(int)floorf(f.x * inv_cell) & 1023u;
        const uint32_t cy = (uint32_t)(int)floorf(f.y * inv_cell) & 1023u;
        const uint32_t cz = (uint32_t)(int)floorf(f.z * inv_cell) & 1023u;
        keys[r] = (ray_spread3(cx) << 2) | (ray_spread3(cy) << 1) | ray_spread3(cz);
        vals[r] = (uint32_t)r;
    }
}

int launch_cast_rays(DeviceState& d, const float4* rays, b3gRayHit* hits, int n, cudaStream_t s) {
    int launches = launch_aabbs(d, s);  // the grid of the current poses
    launches += launch_cells(d, s);
    if (n <= 0) return launches;
    // neighbouring rays in neighbouring lanes: they walk the same cells and test the same bodies
    const int kgrid = std::max(1, std::min((n + 255) / 256, d.num_sms * 8));
    uint32_t* rk = d.ray_order;
    k_ray_keys<<<kgrid, 256, 0, s>>>(rays, n, d.inv_cell, rk, rk + 2 * (size_t)d.ray_cap);
    long long ll = 0;
    d.prim.sort_blocks = d.num_sms * d.tune.sort_blocks_per_sm;
    const int w = radix_sort_u32(d.prim, rk, rk + d.ray_cap, rk + 2 * (size_t)d.ray_cap, rk + 3 * (size_t)d.ray_cap,
                                 d.ray_n, 30, d.sort_scratch, s, &ll);
    launches += 1 + (int)ll;
    RayArgs a;
    a.rays = rays;
    a.hits = hits;
    a.order = rk + (w ? 3 : 2) * (size_t)d.ray_cap;
    a.aabbs = d.aabbs;
    a.n = n;
    a.bodies = d.bodies;
    a.cols = d.collidables;
    a.hulls = d.hulls;
    a.faces = d.faces;
    a.keys = d.cell_sorted_keys;
    a.vals = d.cell_sorted_bodies;
    a.cell_start = d.cell_start;
    a.n_dyn = d.num_dynamic;
    a.inv_cell = d.inv_cell;
    a.bits = d.grid_bits;
    a.body_scene = d.num_scenes > 1 ? d.body_scene : nullptr;
    a.num_scenes = d.num_scenes;
    a.large_list = d.large_list;
    a.large_off = d.num_scenes > 1 ? d.large_off : nullptr;
    a.num_large = d.num_large;
    a.sap_list = d.sap_list;
    a.sap_off = d.sap_off;
    const int grid = std::max(1, std::min((n + 127) / 128, d.num_sms * 16));
    k_cast_rays<<<grid, 128, 0, s>>>(a);
    return launches + 1;
}

}  // namespace b3g
