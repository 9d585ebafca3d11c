// World AABBs and the uniform-grid broadphase.
//
// Reference path:
//   initializeGpuAabbsFull (src/Bullet3OpenCL/RigidBody/kernels/updateAabbsKernel.cl:38)
//     -> b3ComputeWorldAabb / b3TransformAabb2 (Bullet3Collision/BroadPhaseCollision/shared/b3Aabb.h:24-43), margin 0
//   b3GpuGridBroadphase::calculateOverlappingPairs (src/Bullet3OpenCL/BroadphaseCollision/b3GpuGridBroadphase.cpp:117-259):
//     kCalcHashAABB (gridBroadphase.cl:25) cell of the AABB centre, floor(c * invCell) & (dim-1)
//     radix sort of (hash, body), kFindCellStart (:60), kFindOverlappingPairs (:169) 27-cell scan with
//     the inclusive overlap test testAABBOverlap (:89-94), one pair per (lower, higher) body index,
//     large (static, mass 0) proxies against every small proxy (computePairsKernelTwoArrays, sap.cl:66).
//
// GB300 design: one fused AABB+hash kernel; stable 8-bit LSD radix sort; run starts written
// into a dense hash table that is never cleared (entries are validated against the sorted keys);
// the pair kernel works in sorted (spatially coherent) order, buffers pairs per thread and
// reserves output with one warp-aggregated atomic; pairs are then radix-sorted on a packed
// (a, b) key so the pair list is canonical and deterministic (a < b, ascending).
#include <algorithm>
#include <cstddef>

#include "common.cuh"
#include "world_internal.h"

namespace b3g {

static constexpr int BP_THREADS = 256;


__device__ __forceinline__ int cell_coord(float c, float inv_cell, int mask) {
    return ((int)floorf(c * inv_cell)) & mask;
}

__global__ void __launch_bounds__(BP_THREADS) k_aabb_hash(const b3gBody* __restrict__ bodies,
                                                          const b3gCollidable* __restrict__ cols,
                                                          const b3gAabb* __restrict__ local_aabbs,
                                                          const int* __restrict__ dyn_slot,
                                                          const int* __restrict__ body_scene, int n,
                                                          b3gAabb* __restrict__ aabbs, uint32_t* __restrict__ keys,
                                                          uint32_t* __restrict__ vals, float inv_cell, int bits) {
    const int mask = (1 << bits) - 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const b3gBody& b = bodies[i];
        float4 p = ldg4(&b.pos);
        float4 qq = ldg4(&b.quat);
        int col = b.collidableIdx;
        float inv_mass = b.invMass;
        b3gAabb la = local_aabbs[col];
        v3 mn, mx;
        transform_aabb(la, mk3(p.x, p.y, p.z), quat{qq.x, qq.y, qq.z, qq.w}, 0.f, mn, mx);
        b3gAabb w;
        w.minv[0] = mn.x; w.minv[1] = mn.y; w.minv[2] = mn.z; w.minw = i;
        w.maxv[0] = mx.x; w.maxv[1] = mx.y; w.maxv[2] = mx.z; w.maxw = inv_mass == 0.f ? 0 : 1;
        aabbs[i] = w;
        int slot = dyn_slot[i];
        if (slot >= 0) {
            float cx = (mn.x + mx.x) * 0.5f, cy = (mn.y + mx.y) * 0.5f, cz = (mn.z + mx.z) * 0.5f;
            int gx = cell_coord(cx, inv_cell, mask), gy = cell_coord(cy, inv_cell, mask),
                gz = cell_coord(cz, inv_cell, mask);
            if (body_scene) {
                CellShift sh = scene_shift(body_scene[i], bits);
                gx += sh.x; gy += sh.y; gz += sh.z;
            }
            keys[slot] = cell_hash(gx, gy, gz, bits, mask);
            vals[slot] = (uint32_t)i;
        }
    }
}

__global__ void __launch_bounds__(BP_THREADS) k_cell_start(const uint32_t* __restrict__ keys, int n,
                                                           uint32_t* __restrict__ cell_start) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint32_t h = keys[p];
        if (p == 0 || keys[p - 1] != h) cell_start[h] = (uint32_t)p;
    }
}

// inclusive overlap test (testAABBOverlap, gridBroadphase.cl:89-94)
__device__ __forceinline__ bool overlap(const float4& amin, const float4& amax, const float4& bmin, const float4& bmax) {
    return (amin.x <= bmax.x) && (bmin.x <= amax.x) && (amin.y <= bmax.y) && (bmin.y <= amax.y) &&
           (amin.z <= bmax.z) && (bmin.z <= amax.z);
}

static constexpr int PAIR_BUF = 16;

struct PairEmitter {
    uint64_t buf[PAIR_BUF];
    int cnt;
    __device__ void flush_self(uint64_t* out, int* counter, int cap, unsigned int* status) {
        if (cnt == 0) return;
        int base = atomicAdd(counter, cnt);
        for (int k = 0; k < cnt; k++) {
            if (base + k < cap)
                out[base + k] = buf[k];
            else
                atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
        }
        cnt = 0;
    }
    __device__ void push(uint64_t key, uint64_t* out, int* counter, int cap, unsigned int* status) {
        if (cnt == PAIR_BUF) flush_self(out, counter, cap, status);
        buf[cnt++] = key;
    }
};

// 1-axis sweep and prune over the finite static proxies: per scene, the proxies sorted by their
// AABB min along one axis, and the largest AABB extent along it (rounded up).  A proxy L can
// overlap a body B only if L.min lies in [B.min - extent, B.max] on that axis, so each body scans
// that window (two binary searches) instead of the whole list.
struct SapView {
    const int* sorted;   // body indices, per scene sorted by AABB min along `axis`
    const float* mins;   // those mins
    const int* off;      // per scene: first entry (num_scenes + 1)
    const float* ext;    // per scene: largest extent along the axis (+inf: unsorted, scan all)
    int axis;
    int n;               // 0: no finite static proxies
};

__device__ __forceinline__ float axis_of(const float4& v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }

// One block per scene: bitonic sort of the scene's finite static proxies (<= B3G_SAP_MAX_PER_SCENE)
// by AABB min along the axis, in shared memory; larger scenes are copied unsorted with extent +inf.
__global__ void __launch_bounds__(512) k_sap_sort(const b3gAabb* __restrict__ aabbs, const int* __restrict__ list,
                                                  const int* __restrict__ off, int axis, int* __restrict__ sorted,
                                                  float* __restrict__ mins, float* __restrict__ ext) {
    __shared__ float s_key[B3G_SAP_MAX_PER_SCENE];
    __shared__ int s_idx[B3G_SAP_MAX_PER_SCENE];
    __shared__ float s_ext[512 / 32];
    const int sc = blockIdx.x;
    const int lo = off[sc], n = off[sc + 1] - lo;
    if (n <= 0) return;
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    float e = 0.f;
    if (n > B3G_SAP_MAX_PER_SCENE) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int b = list[lo + i];
            sorted[lo + i] = b;
            mins[lo + i] = axis_of(A[2 * b], axis);
        }
        if (threadIdx.x == 0) ext[sc] = __int_as_float(0x7f800000);
        return;
    }
    int P = 2;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < n) {
            const int b = list[lo + i];
            const float mn = axis_of(A[2 * b], axis), mx = axis_of(A[2 * b + 1], axis);
            s_key[i] = mn;
            s_idx[i] = b;
            e = fmaxf(e, __fsub_ru(mx, mn));
        } else {
            s_key[i] = __int_as_float(0x7f800000);
            s_idx[i] = -1;
        }
    }
    for (int o = 16; o; o >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) s_ext[threadIdx.x >> 5] = e;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l <= i) continue;
                const bool up = (i & k) == 0;
                const float a = s_key[i], b = s_key[l];
                if ((a > b) == up) {
                    s_key[i] = b;
                    s_key[l] = a;
                    const int t = s_idx[i];
                    s_idx[i] = s_idx[l];
                    s_idx[l] = t;
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sorted[lo + i] = s_idx[i];
        mins[lo + i] = s_key[i];
    }
    if (threadIdx.x == 0) {
        float m = 0.f;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) m = fmaxf(m, s_ext[w]);
        ext[sc] = m;
    }
}

// first index in [lo, hi) with v[index] >= x (lower) or > x (upper)
__device__ __forceinline__ int bound_search(const float* v, int lo, int hi, float x, bool upper) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float y = __ldg(&v[mid]);
        if (upper ? (y <= x) : (y < x))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Pairs of dynamic body i with the static proxies of its scene: the unbounded ones [l0, l1) of
// large_list brute force, the finite ones through the sweep-and-prune window.
__device__ __forceinline__ void static_pairs(const float4* __restrict__ A, uint32_t i, const float4& amin,
                                             const float4& amax, const int* __restrict__ large_list, int l0, int l1,
                                             const SapView& sap, int si, int body_bits, PairEmitter& em,
                                             uint64_t* __restrict__ out, int* __restrict__ counter, int cap,
                                             unsigned int* __restrict__ status) {
    for (int l = l0; l < l1; l++) {
        uint32_t j = (uint32_t)__ldg(&large_list[l]);
        float4 bmin = __ldg(&A[2 * j]), bmax = __ldg(&A[2 * j + 1]);
        if (overlap(amin, amax, bmin, bmax)) {
            uint32_t a = i < j ? i : j, b = i < j ? j : i;
            em.push(((uint64_t)a << body_bits) | b, out, counter, cap, status);
        }
    }
    if (sap.n > 0) {
        int q0 = __ldg(&sap.off[si]), q1 = __ldg(&sap.off[si + 1]);
        const float e = __ldg(&sap.ext[si]);
        if (q0 < q1 && e <= 3.4e38f) {
            // window of mins in [min - extent, max]; the lower end rounded down so that no
            // proxy reaching this body is left out
            q0 = bound_search(sap.mins, q0, q1, __fsub_rd(axis_of(amin, sap.axis), e), false);
            q1 = bound_search(sap.mins, q0, q1, axis_of(amax, sap.axis), true);
        }
        for (int q = q0; q < q1; q++) {
            uint32_t j = (uint32_t)__ldg(&sap.sorted[q]);
            float4 bmin = __ldg(&A[2 * j]), bmax = __ldg(&A[2 * j + 1]);
            if (overlap(amin, amax, bmin, bmax)) {
                uint32_t a = i < j ? i : j, b = i < j ? j : i;
                em.push(((uint64_t)a << body_bits) | b, out, counter, cap, status);
            }
        }
    }
}

// SCENES: bodies carry a scene index (b3g_set_scene_offsets); cells are shifted per scene, pairs
// need equal scenes and each body tests only its own scene's range of the large list.
template <bool SCENES>
__device__ __forceinline__ void find_pairs_body(const b3gAabb* __restrict__ aabbs, const uint32_t* __restrict__ keys,
                                                const uint32_t* __restrict__ vals,
                                                const uint32_t* __restrict__ cell_start, int n_dyn,
                                                const int* __restrict__ large_list, int n_large,
                                                const int* __restrict__ body_scene,
                                                const int* __restrict__ large_off, const SapView sap, float inv_cell,
                                                int bits, int body_bits, uint64_t* __restrict__ out,
                                                int* __restrict__ counter, int cap, unsigned int* __restrict__ status) {
    const int mask = (1 << bits) - 1;
    const int lane = threadIdx.x & 31;
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    // every lane of a warp runs the same number of outer iterations so the final
    // warp-aggregated flush is convergent
    const int stride = gridDim.x * blockDim.x;
    const int start = blockIdx.x * blockDim.x + threadIdx.x;
    const int iters = (n_dyn + stride - 1) / stride;
    PairEmitter em;
    em.cnt = 0;
    for (int it = 0; it < iters; it++) {
        int p = start + it * stride;
        if (p < n_dyn) {
            uint32_t i = vals[p];
            float4 amin = __ldg(&A[2 * i]), amax = __ldg(&A[2 * i + 1]);
            float cx = (amin.x + amax.x) * 0.5f, cy = (amin.y + amax.y) * 0.5f, cz = (amin.z + amax.z) * 0.5f;
            int gx = (int)floorf(cx * inv_cell), gy = (int)floorf(cy * inv_cell), gz = (int)floorf(cz * inv_cell);
            int si = 0, l0 = 0, l1 = n_large;
            if (SCENES) {
                si = __ldg(&body_scene[i]);
                CellShift sh = scene_shift(si, bits);
                gx += sh.x; gy += sh.y; gz += sh.z;
                l0 = __ldg(&large_off[si]);
                l1 = __ldg(&large_off[si + 1]);
            }
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        uint32_t h = cell_hash(gx + dx, gy + dy, gz + dz, bits, mask);
                        uint32_t s = __ldg(&cell_start[h]);
                        if (s >= (uint32_t)n_dyn) continue;
                        if (__ldg(&keys[s]) != h) continue;
                        if (s > 0 && __ldg(&keys[s - 1]) == h) continue;
                        for (uint32_t q = s; q < (uint32_t)n_dyn; q++) {
                            if (__ldg(&keys[q]) != h) break;
                            uint32_t j = __ldg(&vals[q]);
                            if (j <= i) continue;
                            if (SCENES && __ldg(&body_scene[j]) != si) continue;
                            float4 bmin = __ldg(&A[2 * j]), bmax = __ldg(&A[2 * j + 1]);
                            if (overlap(amin, amax, bmin, bmax))
                                em.push(((uint64_t)i << body_bits) | j, out, counter, cap, status);
                        }
                    }
            static_pairs(A, i, amin, amax, large_list, l0, l1, sap, si, body_bits, em, out, counter, cap, status);
        }
    }
    // warp-aggregated reservation of the remaining buffered pairs
    int c = em.cnt;
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    int my = base + incl - c;
    for (int k = 0; k < c; k++) {
        if (my + k < cap)
            out[my + k] = em.buf[k];
        else
            atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
    }
}

__global__ void __launch_bounds__(BP_THREADS) k_find_pairs(const b3gAabb* __restrict__ aabbs,
                                                           const uint32_t* __restrict__ keys,
                                                           const uint32_t* __restrict__ vals,
                                                           const uint32_t* __restrict__ cell_start, int n_dyn,
                                                           const int* __restrict__ large_list, int n_large,
                                                           float inv_cell, int bits, int body_bits,
                                                           uint64_t* __restrict__ out, int* __restrict__ counter,
                                                           int cap, unsigned int* __restrict__ status) {
    find_pairs_body<false>(aabbs, keys, vals, cell_start, n_dyn, large_list, n_large, nullptr, nullptr,
                           SapView{nullptr, nullptr, nullptr, nullptr, 0, 0}, inv_cell, bits, body_bits, out, counter,
                           cap, status);
}

// Warp-cooperative form of the same search.  A warp takes 32 consecutive dynamic bodies in cell
// order, which mostly share a cell and so the same 27 neighbour cells.  For each neighbour offset
// the lanes are grouped by target cell; the warp streams each distinct cell's members through
// shared memory 32 at a time (coalesced float4 AABB loads, once per group instead of once per
// lane), and every lane of the group tests its own body against the staged members.  The pair
// set is the thread-per-body one: same candidates, same inclusive test, j > i.
static constexpr int BP_WARPS = BP_THREADS / 32;
static constexpr int BP_COOP_MAX_CELLS = 2;  // distinct own cells in a warp for the cooperative scan

template <bool SCENES>
__device__ __forceinline__ void find_pairs_warp(const b3gAabb* __restrict__ aabbs, const uint32_t* __restrict__ keys,
                                                const uint32_t* __restrict__ vals,
                                                const uint32_t* __restrict__ cell_start, int n_dyn,
                                                const int* __restrict__ large_list, int n_large,
                                                const int* __restrict__ body_scene,
                                                const int* __restrict__ large_off, const SapView sap, float inv_cell,
                                                int bits, int body_bits, uint64_t* __restrict__ out,
                                                int* __restrict__ counter, int cap, unsigned int* __restrict__ status) {
    __shared__ float4 s_min[BP_WARPS][32], s_max[BP_WARPS][32];
    __shared__ uint32_t s_j[BP_WARPS][32];
    __shared__ int s_sc[BP_WARPS][32];
    const int mask = (1 << bits) - 1;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    const int nwarps = gridDim.x * BP_WARPS;
    PairEmitter em;
    em.cnt = 0;
    for (int base = (blockIdx.x * BP_WARPS + w) * 32; base < n_dyn; base += nwarps * 32) {
        const int p = base + lane;
        const bool live = p < n_dyn;
        uint32_t i = 0;
        float4 amin = make_float4(0, 0, 0, 0), amax = amin;
        int gx = 0, gy = 0, gz = 0, si = 0, l0 = 0, l1 = n_large;
        if (live) {
            i = vals[p];
            amin = __ldg(&A[2 * i]);
            amax = __ldg(&A[2 * i + 1]);
            const float cx = (amin.x + amax.x) * 0.5f, cy = (amin.y + amax.y) * 0.5f, cz = (amin.z + amax.z) * 0.5f;
            gx = (int)floorf(cx * inv_cell);
            gy = (int)floorf(cy * inv_cell);
            gz = (int)floorf(cz * inv_cell);
            if (SCENES) {
                si = __ldg(&body_scene[i]);
                CellShift sh = scene_shift(si, bits);
                gx += sh.x; gy += sh.y; gz += sh.z;
                l0 = __ldg(&large_off[si]);
                l1 = __ldg(&large_off[si + 1]);
            }
        }
        // cooperative streaming pays off where the warp's bodies crowd into few cells; a warp
        // spread over many sparse cells scans per lane instead (same candidates either way)
        const uint32_t h_own = live ? cell_hash(gx, gy, gz, bits, mask) : 0xffffffffu;
        const unsigned own_peers = __match_any_sync(0xffffffffu, h_own);
        const int distinct = __popc(__ballot_sync(0xffffffffu, live && lane == __ffs(own_peers) - 1));
        // Half stencil: a body scans its own cell (partners of higher index) and the 13 neighbour
        // cells after it in (z, y, x) order (every partner); two overlapping bodies' cells are
        // neighbours (cell >= every extent), so exactly one of them scans the other's cell, and
        // with at least 4 cells an axis no two of the 14 cells share a hash.  Keys are (lower,
        // higher) whichever body found the pair.
        if (distinct > BP_COOP_MAX_CELLS) {
            if (live)
                for (int off = 13; off < 27; off++) {
                            const int dx = off % 3 - 1, dy = (off / 3) % 3 - 1, dz = off / 9 - 1;
                            const uint32_t hh = cell_hash(gx + dx, gy + dy, gz + dz, bits, mask);
                            const uint32_t s0 = __ldg(&cell_start[hh]);
                            if (s0 >= (uint32_t)n_dyn) continue;
                            if (__ldg(&keys[s0]) != hh) continue;
                            if (s0 > 0 && __ldg(&keys[s0 - 1]) == hh) continue;
                            for (uint32_t q = s0; q < (uint32_t)n_dyn; q++) {
                                if (__ldg(&keys[q]) != hh) break;
                                const uint32_t j = __ldg(&vals[q]);
                                if (off == 13 ? j <= i : j == i) continue;
                                if (SCENES && __ldg(&body_scene[j]) != si) continue;
                                if (overlap(amin, amax, __ldg(&A[2 * j]), __ldg(&A[2 * j + 1])))
                                    em.push(i < j ? ((uint64_t)i << body_bits) | j : ((uint64_t)j << body_bits) | i, out,
                                            counter, cap, status);
                            }
                }
        } else
        for (int off = 13; off < 27; off++) {
            const int dx = off % 3 - 1, dy = (off / 3) % 3 - 1, dz = off / 9 - 1;
            // this lane's target cell and its run start (validated against the sorted keys)
            uint32_t h = 0xffffffffu, st = 0;
            if (live) {
                const uint32_t hh = cell_hash(gx + dx, gy + dy, gz + dz, bits, mask);
                const uint32_t s0 = __ldg(&cell_start[hh]);
                if (s0 < (uint32_t)n_dyn && __ldg(&keys[s0]) == hh && !(s0 > 0 && __ldg(&keys[s0 - 1]) == hh)) {
                    h = hh;
                    st = s0;
                }
            }
            unsigned pending = __ballot_sync(0xffffffffu, h != 0xffffffffu);
            while (pending) {
                const int leader = __ffs(pending) - 1;
                const uint32_t H = __shfl_sync(0xffffffffu, h, leader);
                const uint32_t S = __shfl_sync(0xffffffffu, st, leader);
                const bool mine = h == H;
                pending &= ~__ballot_sync(0xffffffffu, mine);
                // stream the cell's members through shared memory, 32 at a time
                for (uint32_t q0 = S;; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    const bool in = q < (uint32_t)n_dyn && __ldg(&keys[q]) == H;
                    const unsigned inmask = __ballot_sync(0xffffffffu, in);
                    // members are contiguous from S: the run ends at the first lane outside it
                    const int cnt = __ffs(~inmask) ? __ffs(~inmask) - 1 : 32;
                    if (lane < cnt) {
                        const uint32_t j = __ldg(&vals[q]);
                        s_j[w][lane] = j;
                        s_min[w][lane] = __ldg(&A[2 * j]);
                        s_max[w][lane] = __ldg(&A[2 * j + 1]);
                        if (SCENES) s_sc[w][lane] = __ldg(&body_scene[j]);
                    }
                    __syncwarp();
                    if (mine) {
                        for (int c = 0; c < cnt; c++) {
                            const uint32_t j = s_j[w][c];
                            if (off == 13 ? j <= i : j == i) continue;
                            if (SCENES && s_sc[w][c] != si) continue;
                            if (overlap(amin, amax, s_min[w][c], s_max[w][c]))
                                em.push(i < j ? ((uint64_t)i << body_bits) | j : ((uint64_t)j << body_bits) | i, out,
                                        counter, cap, status);
                        }
                    }
                    __syncwarp();
                    if (cnt < 32) break;
                }
            }
        }
        if (live) static_pairs(A, i, amin, amax, large_list, l0, l1, sap, si, body_bits, em, out, counter, cap, status);
    }
    // warp-aggregated reservation of the remaining buffered pairs
    int c = em.cnt;
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    int total = __shfl_sync(0xffffffffu, incl, 31);
    int wbase = 0;
    if (lane == 31 && total > 0) wbase = atomicAdd(counter, total);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    int my = wbase + incl - c;
    for (int k = 0; k < c; k++) {
        if (my + k < cap)
            out[my + k] = em.buf[k];
        else
            atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
    }
}

// the world's pair kernel: large (unbounded) list, sweep and prune over finite statics, scenes
template <bool SCENES>
__global__ void __launch_bounds__(BP_THREADS, 8) k_find_pairs_world(
    const b3gAabb* __restrict__ aabbs, const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
    const uint32_t* __restrict__ cell_start, int n_dyn, const int* __restrict__ large_list, int n_large,
    const int* __restrict__ body_scene, const int* __restrict__ large_off, const SapView sap, float inv_cell, int bits,
    int body_bits, uint64_t* __restrict__ out, int* __restrict__ counter, int cap, unsigned int* __restrict__ status) {
    find_pairs_warp<SCENES>(aabbs, keys, vals, cell_start, n_dyn, large_list, n_large, body_scene, large_off, sap,
                            inv_cell, bits, body_bits, out, counter, cap, status);
}

// ---------------------------------------------------------------------------------------- LBVH
// The alternative broadphase for the dynamic bodies, after b3GpuParallelLinearBvhBroadphase
// (b3GpuParallelLinearBvh.cpp:108-359, kernels/parallelLinearBvh.cl): the bounds of all AABB
// centres, a 30-bit Morton code per centre in that box (10 bits per axis,
// assignMortonCodesAndAabbIndicies :116-165), a sort, a binary radix tree over the sorted codes
// (Karras 2012, as constructBinaryRadixTree builds it), node AABBs bottom up, then one traversal
// per leaf that only visits leaves after it in sorted order, so every pair is found once
// (plbvhCalculateOverlappingPairs :176-300).  Here the scene index sits above the Morton code, so
// each scene is a contiguous run of leaves and a traversal never leaves its scene's run; the
// refit is one bottom-up pass with an arrival counter per node instead of one launch per tree
// level; the pairs go through the same canonical (lower, higher) key list as the grid's.

// float -> unsigned with the same order (so atomicMin/atomicMax order floats)
__device__ __forceinline__ unsigned int ord_enc(float f) {
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_dec(unsigned int e) {
    return __uint_as_float((e & 0x80000000u) ? (e & 0x7fffffffu) : ~e);
}

// bounds[0..2] = encoded min of the centres, bounds[3..5] = ~encoded max (both start all ones)
__global__ void __launch_bounds__(BP_THREADS) k_lbvh_bounds(const b3gAabb* __restrict__ aabbs,
                                                            const uint32_t* __restrict__ dyn, int n,
                                                            unsigned int* __restrict__ bounds) {
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(&dyn[p]);
        const float4 a = __ldg(&A[2 * i]), b = __ldg(&A[2 * i + 1]);
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        for (int k = 0; k < 3; k++) {
            mn[k] = fminf(mn[k], c[k]);
            mx[k] = fmaxf(mx[k], c[k]);
        }
    }
    for (int k = 0; k < 3; k++)
        for (int o = 16; o; o >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    // then across the block's warps, so that each block adds 6 atomics on the 6 shared words
    __shared__ float s_b[6][BP_THREADS / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; k++) {
            s_b[k][w] = mn[k];
            s_b[3 + k][w] = mx[k];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        float v = s_b[k][0];
        for (int j = 1; j < BP_THREADS / 32; j++) v = k < 3 ? fminf(v, s_b[k][j]) : fmaxf(v, s_b[k][j]);
        atomicMin(&bounds[k], k < 3 ? ord_enc(v) : ~ord_enc(v));
    }
}

// 10 bits -> every third bit of 30
__device__ __forceinline__ uint32_t spread3(uint32_t x) {
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__global__ void __launch_bounds__(BP_THREADS) k_lbvh_keys(const b3gAabb* __restrict__ aabbs,
                                                          const uint32_t* __restrict__ dyn, int n,
                                                          const unsigned int* __restrict__ bounds,
                                                          const int* __restrict__ body_scene,
                                                          uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    float lo[3], scale[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = ord_dec(bounds[k]);
        const float ext = ord_dec(~bounds[3 + k]) - lo[k];
        scale[k] = ext > 0.f ? 1024.f / ext : 0.f;
    }
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(&dyn[p]);
        const float4 a = __ldg(&A[2 * i]), b = __ldg(&A[2 * i + 1]);
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        uint32_t q[3];
        for (int k = 0; k < 3; k++) q[k] = (uint32_t)fminf(fmaxf((c[k] - lo[k]) * scale[k], 0.f), 1023.f);
        const uint32_t morton = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
        const uint64_t sc = body_scene ? (uint64_t)__ldg(&body_scene[i]) : 0ull;
        keys[p] = (sc << 30) | morton;
        vals[p] = i;
    }
}

// length of the common prefix of sorted keys i and j (-1 outside [0, n)); equal keys are told
// apart by their indices
__device__ __forceinline__ int lbvh_delta(const uint64_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = __ldg(&k[i]), b = __ldg(&k[j]);
    if (a == b) return 64 + __clz((unsigned int)(i ^ j));
    return __clzll((long long)(a ^ b));
}

// The tree's depth is at most the key bits plus the index bits that break ties between equal keys.
static constexpr int LBVH_MAX_DEPTH = 64 + 32;

// internal node i of the binary radix tree over n sorted keys: its leaf range, split and
// children (leaf l stored as ~l); node 0 is the root
__global__ void __launch_bounds__(BP_THREADS) k_lbvh_build(const uint64_t* __restrict__ keys, int n,
                                                           int2* __restrict__ child, int2* __restrict__ range,
                                                           int* __restrict__ parent, int* __restrict__ flag) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int d = lbvh_delta(keys, n, i, i + 1) - lbvh_delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
        const int dmin = lbvh_delta(keys, n, i, i - d);
        int lmax = 2;
        while (lbvh_delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (lbvh_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = lbvh_delta(keys, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (lbvh_delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int gamma = i + s * d + (d < 0 ? -1 : 0);
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        const int left = lo == gamma ? ~gamma : gamma;
        const int right = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
        child[i] = make_int2(left, right);
        range[i] = make_int2(lo, hi);
        parent[left < 0 ? ~left : n + left] = i;
        parent[right < 0 ? ~right : n + right] = i;
        flag[i] = 0;
        if (i == 0) parent[n] = -1;
    }
}

// node AABBs bottom up: every leaf walks towards the root; the first child to arrive at a node
// stops there, the second (which sees both children finished) merges them and goes on
__global__ void __launch_bounds__(BP_THREADS) k_lbvh_refit(const b3gAabb* __restrict__ aabbs,
                                                           const uint32_t* __restrict__ vals, int n,
                                                           const int2* __restrict__ child,
                                                           const int* __restrict__ parent, int* __restrict__ flag,
                                                           float4* __restrict__ box, unsigned int* __restrict__ status) {
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int node = parent[p];
        for (int level = 0; node >= 0; ++level) {
            if (level > LBVH_MAX_DEPTH) {  // deeper than any radix tree over these keys: report, stop
                atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
                break;
            }
            __threadfence();
            if (atomicAdd(&flag[node], 1) == 0) break;
            const int2 c = child[node];
            float4 mn[2], mx[2];
            const int cc[2] = {c.x, c.y};
            for (int k = 0; k < 2; k++) {
                if (cc[k] < 0) {
                    const uint32_t b = __ldg(&vals[~cc[k]]);
                    mn[k] = __ldg(&A[2 * b]);
                    mx[k] = __ldg(&A[2 * b + 1]);
                } else {
                    mn[k] = __ldcg(&box[2 * cc[k]]);
                    mx[k] = __ldcg(&box[2 * cc[k] + 1]);
                }
            }
            __stcg(&box[2 * node], make_float4(fminf(mn[0].x, mn[1].x), fminf(mn[0].y, mn[1].y),
                                               fminf(mn[0].z, mn[1].z), 0.f));
            __stcg(&box[2 * node + 1], make_float4(fmaxf(mx[0].x, mx[1].x), fmaxf(mx[0].y, mx[1].y),
                                                   fmaxf(mx[0].z, mx[1].z), 0.f));
            node = parent[n + node];
        }
    }
}

// Depth-first stack of a traversal: one pending sibling per level at most.
static constexpr int LBVH_STACK = LBVH_MAX_DEPTH + 2;

// One sorted leaf q per thread: the leaves after q in its scene's run whose AABBs overlap its
// body's, then the static proxies (same path as the grid's pair kernel).
template <bool SCENES>
__global__ void __launch_bounds__(BP_THREADS) k_lbvh_pairs(
    const b3gAabb* __restrict__ aabbs, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, int n,
    const int2* __restrict__ child, const int2* __restrict__ range, const float4* __restrict__ box,
    const int* __restrict__ large_list, int n_large, const int* __restrict__ body_scene,
    const int* __restrict__ large_off, const SapView sap, int body_bits, uint64_t* __restrict__ out,
    int* __restrict__ counter, int cap, unsigned int* __restrict__ status) {
    const float4* A = reinterpret_cast<const float4*>(aabbs);
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const int start = blockIdx.x * blockDim.x + threadIdx.x;
    const int iters = (n + stride - 1) / stride;  // equal for every lane: the final flush is convergent
    PairEmitter em;
    em.cnt = 0;
    int stack[LBVH_STACK];
    for (int it = 0; it < iters; it++) {
        const int q = start + it * stride;
        if (q >= n) continue;
        const uint32_t i = __ldg(&vals[q]);
        const float4 amin = __ldg(&A[2 * i]), amax = __ldg(&A[2 * i + 1]);
        int si = 0, l0 = 0, l1 = n_large, s_hi = n;
        if (SCENES) {
            si = __ldg(&body_scene[i]);
            l0 = __ldg(&large_off[si]);
            l1 = __ldg(&large_off[si + 1]);
            // end of the scene's run: the first sorted key of a later scene
            const uint64_t lim = (uint64_t)(si + 1) << 30;
            int lo = q + 1, hi = n;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (__ldg(&keys[mid]) < lim)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            s_hi = lo;
        }
        if (n > 1 && q + 1 < s_hi) {
            int sp = 0;
            stack[sp++] = 0;
            while (sp > 0) {
                const int node = stack[--sp];
                if (node < 0) {
                    const int l = ~node;
                    if (l <= q || l >= s_hi) continue;
                    const uint32_t j = __ldg(&vals[l]);
                    const float4 bmin = __ldg(&A[2 * j]), bmax = __ldg(&A[2 * j + 1]);
                    if (overlap(amin, amax, bmin, bmax)) {
                        const uint32_t a = i < j ? i : j, b = i < j ? j : i;
                        em.push(((uint64_t)a << body_bits) | b, out, counter, cap, status);
                    }
                    continue;
                }
                const int2 r = __ldg(&range[node]);
                if (r.y <= q || r.x >= s_hi) continue;
                if (!overlap(amin, amax, __ldg(&box[2 * node]), __ldg(&box[2 * node + 1]))) continue;
                const int2 c = __ldg(&child[node]);
                if (sp + 2 > LBVH_STACK) {  // cannot happen (see LBVH_STACK); reported, never silent
                    atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
                    continue;
                }
                stack[sp++] = c.y;
                stack[sp++] = c.x;
            }
        }
        static_pairs(A, i, amin, amax, large_list, l0, l1, sap, si, body_bits, em, out, counter, cap, status);
    }
    // warp-aggregated reservation of the remaining buffered pairs
    const int c = em.cnt;
    int incl = c;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int wbase = 0;
    if (lane == 31 && total > 0) wbase = atomicAdd(counter, total);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    const int my = wbase + incl - c;
    for (int k = 0; k < c; k++) {
        if (my + k < cap)
            out[my + k] = em.buf[k];
        else
            atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
    }
}

__global__ void k_clamp_count(int* counter, int cap, int* clamped) {
    int n = *counter;
    *clamped = n < cap ? n : cap;
}

__device__ __forceinline__ int pair_type(int ta, int tb) {
    if (ta == B3G_SHAPE_CONVEX_HULL && tb == B3G_SHAPE_CONVEX_HULL) return PT_HULL_HULL;
    if ((ta == B3G_SHAPE_PLANE && tb == B3G_SHAPE_CONVEX_HULL) || (tb == B3G_SHAPE_PLANE && ta == B3G_SHAPE_CONVEX_HULL))
        return PT_PLANE_HULL;
    if ((ta == B3G_SHAPE_SPHERE && tb == B3G_SHAPE_CONVEX_HULL) || (tb == B3G_SHAPE_SPHERE && ta == B3G_SHAPE_CONVEX_HULL))
        return PT_SPHERE_HULL;
    if (ta == B3G_SHAPE_SPHERE && tb == B3G_SHAPE_SPHERE) return PT_SPHERE_SPHERE;
    if ((ta == B3G_SHAPE_PLANE && tb == B3G_SHAPE_SPHERE) || (tb == B3G_SHAPE_PLANE && ta == B3G_SHAPE_SPHERE))
        return PT_PLANE_SPHERE;
    return -1;
}

// Unpack sorted keys into b3Int4 pairs, reset the per-pair contact flag, and bucket pairs
// by shape-type combination for the narrowphase kernels.
__global__ void __launch_bounds__(BP_THREADS) k_unpack_pairs(const uint64_t* __restrict__ keys,
                                                             const int* __restrict__ d_np, int body_bits,
                                                             const b3gBody* __restrict__ bodies,
                                                             const b3gCollidable* __restrict__ cols,
                                                             const int* __restrict__ col_small,
                                                             b3gPair* __restrict__ pairs, int* __restrict__ flags,
                                                             int* __restrict__ type_lists, int max_pairs,
                                                             int* __restrict__ type_count) {
    const int np = *d_np;
    const uint64_t bmask = (1ull << body_bits) - 1ull;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const int iters = (np + stride - 1) / stride;
    for (int it = 0; it < iters; it++) {
        int p = blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        int t = -1;
        if (p < np) {
            uint64_t k = keys[p];
            int a = (int)(k >> body_bits), b = (int)(k & bmask);
            b3gPair pr;
            pr.x = a; pr.y = b; pr.z = -1; pr.w = -1;
            pairs[p] = pr;
            flags[p] = 0;
            int ca = bodies[a].collidableIdx, cb = bodies[b].collidableIdx;
            int ta = cols[ca].shapeType;
            int tb = cols[cb].shapeType;
            t = pair_type(ta, tb);
            if (t == PT_HULL_HULL) {
                const int sa = col_small[ca], sb = col_small[cb];
                if (sa && sb) {
                    const int axes = ((sa >> 1) & 0x7fff) + ((sb >> 1) & 0x7fff) + (sa >> 16) * (sb >> 16);
                    if (axes <= B3G_SMALL_PAIR_AXES) t = PT_HULL_HULL_SMALL;
                }
            }
        }
        unsigned peers = __match_any_sync(0xffffffffu, t);
        int leader = __ffs(peers) - 1;
        int rank = __popc(peers & ((1u << lane) - 1u));
        int base = 0;
        if (t >= 0 && lane == leader) base = atomicAdd(&type_count[t], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        if (t >= 0) type_lists[t * max_pairs + base + rank] = p;
    }
}

int launch_aabbs(DeviceState& d, cudaStream_t s) {
    // one body per thread in a single wave (latency-bound: body -> collidable -> local AABB chain)
    const int grid = std::max(1, std::min((d.num_bodies + BP_THREADS - 1) / BP_THREADS, d.num_sms * 32));
    k_aabb_hash<<<grid, BP_THREADS, 0, s>>>(d.bodies, d.collidables, d.local_aabbs, d.dyn_slot,
                                            d.num_scenes > 1 ? d.body_scene : nullptr, d.num_bodies, d.aabbs,
                                            d.cell_keys[0], d.cell_vals[0], d.inv_cell, d.grid_bits);
    return 1;
}

// The grid of the current AABBs: (cell hash, body) sorted, run starts in the dense table.
int launch_cells(DeviceState& d, cudaStream_t s) {
    long long ll = 0;
    d.prim.sort_blocks = d.num_sms * d.tune.sort_blocks_per_sm;
    int which = radix_sort_u32(d.prim, d.cell_keys[0], d.cell_keys[1], d.cell_vals[0], d.cell_vals[1],
                               d.d_num_dynamic, 3 * d.grid_bits, d.sort_scratch, s, &ll);
    d.cell_sorted_keys = d.cell_keys[which];
    d.cell_sorted_bodies = d.cell_vals[which];  // dynamic bodies in cell order: the solver partitions this list
    k_cell_start<<<d.num_sms * 4, BP_THREADS, 0, s>>>(d.cell_sorted_keys, d.num_dynamic, d.cell_start);
    return 1 + (int)ll;
}

// The LBVH of the current AABBs: centre bounds, keys, sort, tree, node AABBs.  The dynamic bodies
// in (scene, Morton) order also serve the solver's partitions, as the cell order does for the grid.
static int launch_lbvh(DeviceState& d, cudaStream_t s) {
    const int n = d.num_dynamic;
    if (n == 0) return 0;
    long long ll = 0;
    const int grid = std::max(1, std::min((n + BP_THREADS - 1) / BP_THREADS, d.num_sms * 8));
    cudaMemsetAsync(d.lbvh_bounds, 0xff, 6 * sizeof(unsigned int), s);
    // the dynamic bodies, in slot order, are the values launch_aabbs wrote next to the cell keys
    k_lbvh_bounds<<<grid, BP_THREADS, 0, s>>>(d.aabbs, d.cell_vals[0], n, d.lbvh_bounds);
    k_lbvh_keys<<<grid, BP_THREADS, 0, s>>>(d.aabbs, d.cell_vals[0], n, d.lbvh_bounds,
                                            d.num_scenes > 1 ? d.body_scene : nullptr, d.lbvh_keys[0],
                                            d.lbvh_vals[0]);
    d.prim.sort_blocks = d.num_sms * d.tune.sort_blocks_per_sm;
    const int w = radix_sort_u64(d.prim, d.lbvh_keys[0], d.lbvh_keys[1], d.lbvh_vals[0], d.lbvh_vals[1],
                                 d.d_num_dynamic, 30 + d.scene_bits, d.sort_scratch, s, &ll);
    d.lbvh_sorted_keys = d.lbvh_keys[w];
    d.lbvh_sorted_vals = d.lbvh_vals[w];
    d.cell_sorted_bodies = d.lbvh_sorted_vals;
    d.cell_sorted_keys = nullptr;
    int launches = 3 + (int)ll;
    if (n > 1) {
        k_lbvh_build<<<grid, BP_THREADS, 0, s>>>(d.lbvh_sorted_keys, n, d.lbvh_child, d.lbvh_range, d.lbvh_parent,
                                                 d.lbvh_flag);
        k_lbvh_refit<<<grid, BP_THREADS, 0, s>>>(d.aabbs, d.lbvh_sorted_vals, n, d.lbvh_child, d.lbvh_parent,
                                                 d.lbvh_flag, d.lbvh_box, &d.counters->status);
        launches += 2;
    }
    return launches;
}

int launch_pairs(DeviceState& d, cudaStream_t s) {
    int launches = 0;
    long long ll = 0;
    const bool lbvh = d.broadphase == B3G_BROADPHASE_LBVH && d.lbvh_cap > 0;
    // 1-2. sort (cell hash, body) -- keys written by launch_aabbs -- and run starts; or the LBVH
    if (lbvh)
        launches += launch_lbvh(d, s);
    else
        launches += launch_cells(d, s);
    uint32_t* keys = const_cast<uint32_t*>(d.cell_sorted_keys);
    uint32_t* vals = const_cast<uint32_t*>(d.cell_sorted_bodies);
    // 3. pairs
    // per-step counters restart at zero; the status word accumulates until the host clears it
    cudaMemsetAsync(d.counters, 0, offsetof(DevCounters, status), s);
    cudaMemsetAsync(reinterpret_cast<char*>(d.counters) + offsetof(DevCounters, status) + sizeof(unsigned int), 0,
                    sizeof(DevCounters) - offsetof(DevCounters, status) - sizeof(unsigned int), s);
    const int pgrid = d.num_sms * d.tune.pairs_blocks_per_sm;
    const SapView sap{d.sap_sorted, d.sap_min, d.sap_off, d.sap_ext, d.sap_axis, d.num_sap};
    if (d.num_sap > 0) {
        k_sap_sort<<<d.num_scenes, 512, 0, s>>>(d.aabbs, d.sap_list, d.sap_off, d.sap_axis, d.sap_sorted, d.sap_min,
                                                d.sap_ext);
        launches++;
    }
    if (lbvh && d.num_scenes > 1)
        k_lbvh_pairs<true><<<pgrid, BP_THREADS, 0, s>>>(
            d.aabbs, d.lbvh_sorted_keys, d.lbvh_sorted_vals, d.num_dynamic, d.lbvh_child, d.lbvh_range, d.lbvh_box,
            d.large_list, d.num_large, d.body_scene, d.large_off, sap, d.body_bits, d.pair_keys[0],
            &d.counters->num_pairs, d.max_pairs, &d.counters->status);
    else if (lbvh)
        k_lbvh_pairs<false><<<pgrid, BP_THREADS, 0, s>>>(
            d.aabbs, d.lbvh_sorted_keys, d.lbvh_sorted_vals, d.num_dynamic, d.lbvh_child, d.lbvh_range, d.lbvh_box,
            d.large_list, d.num_large, nullptr, nullptr, sap, d.body_bits, d.pair_keys[0], &d.counters->num_pairs,
            d.max_pairs, &d.counters->status);
    else if (d.num_scenes > 1)
        k_find_pairs_world<true><<<pgrid, BP_THREADS, 0, s>>>(
            d.aabbs, keys, vals, d.cell_start, d.num_dynamic, d.large_list, d.num_large, d.body_scene, d.large_off,
            sap, d.inv_cell, d.grid_bits, d.body_bits, d.pair_keys[0], &d.counters->num_pairs, d.max_pairs,
            &d.counters->status);
    else
        k_find_pairs_world<false><<<pgrid, BP_THREADS, 0, s>>>(
            d.aabbs, keys, vals, d.cell_start, d.num_dynamic, d.large_list, d.num_large, nullptr, nullptr, sap,
            d.inv_cell, d.grid_bits, d.body_bits, d.pair_keys[0], &d.counters->num_pairs, d.max_pairs,
            &d.counters->status);
    launches++;
    // clamp the count to capacity for the consumers (the raw count stays in num_pairs)
    int* d_np = &d.counters->pad[0];
    k_clamp_count<<<1, 1, 0, s>>>(&d.counters->num_pairs, d.max_pairs, d_np);
    launches++;
    // 4. canonical order: sort packed (a, b) keys
    int w2 = radix_sort_u64(d.prim, d.pair_keys[0], d.pair_keys[1], nullptr, nullptr, d_np, 2 * d.body_bits,
                            d.sort_scratch, s, &ll);
    // 5. unpack + classify
    k_unpack_pairs<<<d.num_sms * 4, BP_THREADS, 0, s>>>(d.pair_keys[w2], d_np, d.body_bits, d.bodies, d.collidables,
                                                        d.col_small, d.pairs, d.contact_flag, d.type_lists, d.max_pairs,
                                                        d.counters->type_count);
    launches++;
    return launches + (int)ll;
}

// Caller-supplied pairs (computeContacts(pairs, ...)): packed (min, max) keys of the valid ones;
// an invalid pair becomes the all-ones key, which the sort moves behind the valid ones, and leaves
// the count.
__global__ void k_user_pair_keys(const b3gPair* __restrict__ pairs, int n, int num_bodies, int body_bits,
                                 uint64_t* __restrict__ keys, int* __restrict__ count, int cap,
                                 unsigned int* __restrict__ status) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n && i < cap; i += gridDim.x * blockDim.x) {
        const b3gPair p = pairs[i];
        const int a = min(p.x, p.y), b = max(p.x, p.y);
        if (a < 0 || b >= num_bodies || a == b) {
            keys[i] = ~0ull;
            atomicSub(count, 1);
            atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
            continue;
        }
        keys[i] = ((uint64_t)a << body_bits) | (uint64_t)b;
    }
    if (n > cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, B3G_FLAG_PAIR_OVERFLOW);
}

int launch_pairs_external(DeviceState& d, const b3gPair* pairs, int n, cudaStream_t s) {
    long long ll = 0;
    cudaMemsetAsync(d.counters, 0, offsetof(DevCounters, status), s);
    cudaMemsetAsync(reinterpret_cast<char*>(d.counters) + offsetof(DevCounters, status) + sizeof(unsigned int), 0,
                    sizeof(DevCounters) - offsetof(DevCounters, status) - sizeof(unsigned int), s);
    int* d_np = &d.counters->pad[0];       // valid pairs (the consumers' count)
    int* d_written = &d.counters->pad[2];  // keys written: the sort covers the invalid ones too
    const int m = std::min(n, d.max_pairs);
    launch_set_int(d_np, m, s);
    launch_set_int(d_written, m, s);
    k_user_pair_keys<<<d.num_sms * 4, BP_THREADS, 0, s>>>(pairs, n, d.num_bodies, d.body_bits, d.pair_keys[0], d_np,
                                                          d.max_pairs, &d.counters->status);
    const int w = radix_sort_u64(d.prim, d.pair_keys[0], d.pair_keys[1], nullptr, nullptr, d_written,
                                 2 * d.body_bits, d.sort_scratch, s, &ll);
    k_clamp_count<<<1, 1, 0, s>>>(d_np, d.max_pairs, &d.counters->num_pairs);
    k_unpack_pairs<<<d.num_sms * 4, BP_THREADS, 0, s>>>(d.pair_keys[w], d_np, d.body_bits, d.bodies, d.collidables,
                                                        d.col_small, d.pairs, d.contact_flag, d.type_lists,
                                                        d.max_pairs, d.counters->type_count);
    return 6 + (int)ll;
}

}  // namespace b3g
