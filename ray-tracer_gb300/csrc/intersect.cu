// Intersection of traversal candidates: any-hit (shadow) and closest-hit (reflection / primary).
//
// Reference: CalculateShadowRayIntersections (RayTracer.cu:1498-1614: per (leaf node, triangle) record
// test its <= 8 rays with a non-watertight Moller-Trumbore using __fdividef; occluded iff
// eps < t < |o - p| - 2 eps -> flag = UINT_MAX) and CalculateReflectionRayIntersections (:1711-1774:
// atomicMin of ((uint)(t*10 + 1) << 20) + triID, i.e. t quantised to 0.1 in 12 bits).
//
// Here: P threads per candidate (one per ray of the packet); a ray first tests the cluster's bounding
// sphere, then the cluster's triangles with the watertight test. Any-hit stores RSH_OCCLUDED and stops (and skips rays
// already known occluded); closest-hit keeps its best (float bits of t << 32 | original triangle id)
// and issues one 64-bit atomicMin. A persistent grid-stride loop reads the candidate count on the
// device, so no host readback sits between traversal and intersection.
#include "common.cuh"
#include "kernels.h"
#include "tests.cuh"

namespace rsh {

template <bool ANY>
__global__ void __launch_bounds__(256) k_intersect(IsectArgs a) {
    const uint32_t P = a.packet;
    const unsigned long long cc = *a.cand_count;
    const unsigned long long count = cc < a.capacity ? cc : a.capacity;
    const uint32_t n = dev_count(a.d_count, a.max_rays);
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane_in = gtid % P;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x / P;
    unsigned long long tests = 0;
    for (unsigned long long c = gtid / P; c < count; c += stride) {
        const unsigned long long cand = __ldg(a.cand + c);
        const uint32_t packet = (uint32_t)(cand >> 32), cluster = (uint32_t)cand;
        const uint32_t k = packet * P + lane_in;
        if (k >= n) continue;
        const uint32_t id = a.sorted_ids ? __ldg(a.sorted_ids + k) : k;
        if (id >= a.max_rays) continue;
        float4 o, d;
        load_ray(a.rays, id, o, d);
        if (!(d.w > o.w)) continue;
        if (ANY && *(volatile uint32_t*)(a.flags + id) == RSH_OCCLUDED) continue;
        if (!ray_hits_sphere(o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, __ldg(a.spheres + cluster))) continue;
        const RayWT r = wt_setup(o, d);
        uint32_t t0, t1;
        cluster_tris(a.kids, cluster, t0, t1);
        unsigned long long best = RSH_HIT_NONE;
        for (uint32_t t = t0; t < t1; ++t) {
            const float4 v0 = __ldg(a.tris + 3ull * t);
            const float4 v1 = __ldg(a.tris + 3ull * t + 1);
            const float4 v2 = __ldg(a.tris + 3ull * t + 2);
            float th;
            ++tests;
            if (wt_hit(r, v0, v1, v2, th)) {
                if (ANY) {
                    a.flags[id] = RSH_OCCLUDED;
                    break;
                }
                const unsigned long long key = hit_key(th, __float_as_uint(v0.w));
                best = key < best ? key : best;
            }
        }
        if (!ANY && best != RSH_HIT_NONE) {
            if (best < *(volatile unsigned long long*)(a.hits + id)) atomicMin(a.hits + id, best);
        }
    }
#pragma unroll
    for (int dd = 16; dd > 0; dd >>= 1) tests += __shfl_xor_sync(0xffffffffu, tests, dd);
    if ((threadIdx.x & 31u) == 0 && a.tri_tests) atomicAdd(a.tri_tests, tests);
}

// Per-ray candidates: one thread per (ray, cluster). A closest-hit ray skips a cluster whose sphere lies
// beyond its current best hit.
template <bool ANY>
__global__ void __launch_bounds__(256) k_intersect_rays(IsectArgs a) {
    const unsigned long long cc = *a.cand_count;
    const unsigned long long count = cc < a.capacity ? cc : a.capacity;
    const uint32_t n = dev_count(a.d_count, a.max_rays);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long tests = 0;
    for (unsigned long long c = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; c < count; c += stride) {
        const unsigned long long cand = __ldg(a.cand + c);
        const uint32_t k = (uint32_t)(cand >> 32), cluster = (uint32_t)cand & 0x7FFFFFFFu;
        if (k >= n) continue;
        const uint32_t id = a.sorted_ids ? __ldg(a.sorted_ids + k) : k;
        if (id >= a.max_rays) continue;
        float4 o, d;
        load_ray(a.rays, id, o, d);
        if (!(d.w > o.w)) continue;
        if (ANY && *(volatile uint32_t*)(a.flags + id) == RSH_OCCLUDED) continue;
        if (!ANY) {
            const unsigned long long cur = *(volatile unsigned long long*)(a.hits + id);
            if (cur != RSH_HIT_NONE) {
                const float tb = __uint_as_float((uint32_t)(cur >> 32));
                if (!ray_hits_sphere(o.x, o.y, o.z, d.x, d.y, d.z, o.w, fminf(d.w, tb), __ldg(a.spheres + cluster)))
                    continue;
            }
        }
        const RayWT r = wt_setup(o, d);
        uint32_t t0, t1;
        cluster_tris(a.kids, cluster, t0, t1);
        unsigned long long best = RSH_HIT_NONE;
        for (uint32_t t = t0; t < t1; ++t) {
            const float4 v0 = __ldg(a.tris + 3ull * t);
            const float4 v1 = __ldg(a.tris + 3ull * t + 1);
            const float4 v2 = __ldg(a.tris + 3ull * t + 2);
            float th;
            ++tests;
            if (wt_hit(r, v0, v1, v2, th)) {
                if (ANY) {
                    a.flags[id] = RSH_OCCLUDED;
                    break;
                }
                const unsigned long long key = hit_key(th, __float_as_uint(v0.w));
                best = key < best ? key : best;
            }
        }
        if (!ANY && best != RSH_HIT_NONE) {
            if (best < *(volatile unsigned long long*)(a.hits + id)) atomicMin(a.hits + id, best);
        }
    }
#pragma unroll
    for (int dd = 16; dd > 0; dd >>= 1) tests += __shfl_xor_sync(0xffffffffu, tests, dd);
    if ((threadIdx.x & 31u) == 0 && a.tri_tests) atomicAdd(a.tri_tests, tests);
}

cudaError_t launch_intersect(const IsectArgs& a, bool any_hit, cudaStream_t s) {
    int sms = 152, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t grid = (uint32_t)sms * 8u;
    if (a.per_ray) {
        if (any_hit) k_intersect_rays<true><<<grid, 256, 0, s>>>(a);
        else k_intersect_rays<false><<<grid, 256, 0, s>>>(a);
    } else {
        if (any_hit) k_intersect<true><<<grid, 256, 0, s>>>(a);
        else k_intersect<false><<<grid, 256, 0, s>>>(a);
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
