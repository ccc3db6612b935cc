// Object bounding-sphere hierarchy over the scene's triangles.
//
// Reference: one minimal enclosing sphere per mesh from the GPL Miniball (BoundingSphere.cpp:9-63),
// packed as {centre, radius, firstTri, lastTri} (main.cpp:2445-2470) and culled against the top ray
// nodes (CalculateBoundingSpheresIntersections, RayTracer.cu:1152-1280); triangles then get a bounding
// sphere each (CreateTriangleBoundingSphere, :301-376) inside the descent. Here the object spheres
// become a full sphere tree built on the GPU:
//   1. Morton code (10 bits per axis) of every triangle centroid over the cube around the scene box;
//   2. stable onesweep sort of (code, triangle id) -> cluster order;
//   3. gather triangles into cluster order (original id kept in the first vertex's w);
//   4. level 0: one sphere per cluster of `cluster` consecutive triangles: centre = midpoint of the
//      vertex box, radius = max vertex distance (x (1 + 2^-20));
//   5. levels 1..: fan-out 8 over consecutive nodes (until a level has at most 8 nodes); each node's
//      sphere from all vertices of its subtree by the same formula as the clusters.
// Every sphere encloses every vertex below it, so the hierarchy never culls a real hit.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr float kRadSlack = 1.0f + 1.0f / 1048576.0f;
}

__global__ void k_morton(const float4* __restrict__ pos, uint32_t n, v3 lo, v3 sc, uint32_t* codes) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = __ldg(pos + 3ull * i), b = __ldg(pos + 3ull * i + 1), c = __ldg(pos + 3ull * i + 2);
    const float cx = ((a.x + b.x) + c.x) / 3.0f;
    const float cy = ((a.y + b.y) + c.y) / 3.0f;
    const float cz = ((a.z + b.z) + c.z) / 3.0f;
    float fx = fminf(fmaxf((cx - lo.x) * sc.x, 0.f), 1023.f);
    float fy = fminf(fmaxf((cy - lo.y) * sc.y, 0.f), 1023.f);
    float fz = fminf(fmaxf((cz - lo.z) * sc.z, 0.f), 1023.f);
    codes[i] = (spread3((uint32_t)fx) << 2) | (spread3((uint32_t)fy) << 1) | spread3((uint32_t)fz);
}

__global__ void k_gather_tris(const float4* __restrict__ pos, const uint32_t* __restrict__ perm,
                              uint32_t n, float4* __restrict__ tris, uint32_t* __restrict__ order) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t t = __ldg(perm + k);
    float4 a = __ldg(pos + 3ull * t);
    a.w = __uint_as_float(t);
    tris[3ull * k] = a;
    tris[3ull * k + 1] = __ldg(pos + 3ull * t + 1);
    tris[3ull * k + 2] = __ldg(pos + 3ull * t + 2);
    order[k] = t;
}

__global__ void k_leaf_spheres(const float4* __restrict__ tris, uint32_t n, uint32_t cluster,
                               uint32_t nleaves, float4* __restrict__ sph) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nleaves) return;
    const uint32_t t0 = j * cluster, t1 = (t0 + cluster < n) ? t0 + cluster : n;
    const float inf = __int_as_float(0x7f800000);
    float mnx = inf, mny = inf, mnz = inf, mxx = -inf, mxy = -inf, mxz = -inf;
    for (uint32_t t = t0; t < t1; ++t)
        for (int v = 0; v < 3; ++v) {
            const float4 p = __ldg(tris + 3ull * t + v);
            mnx = fminf(mnx, p.x);
            mny = fminf(mny, p.y);
            mnz = fminf(mnz, p.z);
            mxx = fmaxf(mxx, p.x);
            mxy = fmaxf(mxy, p.y);
            mxz = fmaxf(mxz, p.z);
        }
    const v3 c = v3{(mnx + mxx) * 0.5f, (mny + mxy) * 0.5f, (mnz + mxz) * 0.5f};
    float r2 = 0.f;
    for (uint32_t t = t0; t < t1; ++t)
        for (int v = 0; v < 3; ++v) {
            const float4 p = __ldg(tris + 3ull * t + v);
            const v3 d = v3{p.x - c.x, p.y - c.y, p.z - c.z};
            r2 = fmaxf(r2, dot3(d, d));
        }
    sph[j] = make_float4(c.x, c.y, c.z, sqrtf(r2) * kRadSlack);
}

// Level >= 1: the same formula over every vertex of the node's subtree (one warp per node); tighter than
// enclosing the children's spheres. Min/max and max reductions are exact in any order.
__global__ void k_level_spheres(const float4* __restrict__ tris, uint32_t n, uint64_t span, uint32_t nnodes,
                                float4* __restrict__ sph) {
    const uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (j >= nnodes) return;
    const uint64_t t0 = (uint64_t)j * span;
    const uint64_t t1 = (t0 + span < n) ? t0 + span : n;
    const uint64_t v0 = 3 * t0, v1 = 3 * t1;
    const float inf = __int_as_float(0x7f800000);
    float mnx = inf, mny = inf, mnz = inf, mxx = -inf, mxy = -inf, mxz = -inf;
    for (uint64_t v = v0 + lane; v < v1; v += 32) {
        const float4 p = __ldg(tris + v);
        mnx = fminf(mnx, p.x);
        mny = fminf(mny, p.y);
        mnz = fminf(mnz, p.z);
        mxx = fmaxf(mxx, p.x);
        mxy = fmaxf(mxy, p.y);
        mxz = fmaxf(mxz, p.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
        mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
    }
    const v3 c = v3{(mnx + mxx) * 0.5f, (mny + mxy) * 0.5f, (mnz + mxz) * 0.5f};
    float r2 = 0.f;
    for (uint64_t v = v0 + lane; v < v1; v += 32) {
        const float4 p = __ldg(tris + v);
        const v3 d = v3{p.x - c.x, p.y - c.y, p.z - c.z};
        r2 = fmaxf(r2, dot3(d, d));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, o));
    if (lane == 0) sph[j] = make_float4(c.x, c.y, c.z, sqrtf(r2) * kRadSlack);
}

size_t objh_scratch_bytes(uint32_t tri_count) {
    return 4ull * tri_count * 2 + sort_scratch_bytes(tri_count, 30) + 4096;
}

cudaError_t build_object_hierarchy(const float4* positions_dev, uint32_t n, uint32_t cluster,
                                   const float lo[3], const float hi[3], ObjHierarchy& h,
                                   void* scratch, size_t scratch_bytes, uint32_t* err, cudaStream_t s) {
    (void)scratch_bytes;
    h.tri_count = n;
    h.cluster = cluster;
    if (n == 0) {
        h.levels = 0;
        return cudaSuccess;
    }
    // level sizes
    uint32_t sizes[16];
    uint32_t levels = 0;
    uint32_t cur = (n + cluster - 1) / cluster;
    sizes[levels++] = cur;
    while (cur > 8 && levels < 16) {
        cur = (cur + 7) / 8;
        sizes[levels++] = cur;
    }
    uint32_t total = 0;
    for (uint32_t l = 0; l < levels; ++l) {
        h.level_off[l] = total;
        h.level_size[l] = sizes[l];
        total += sizes[l];
    }
    h.levels = levels;
    cudaError_t e;
    if ((e = cudaMalloc(&h.spheres, sizeof(float4) * total)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.tris, sizeof(float4) * 3ull * n)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.order, sizeof(uint32_t) * n)) != cudaSuccess) return e;

    char* b = static_cast<char*>(scratch);
    uint32_t* codes = reinterpret_cast<uint32_t*>(b);
    uint32_t* sorted_codes = codes + n;
    uint32_t* perm = reinterpret_cast<uint32_t*>(h.order);  // sorted values land in order[] first
    void* sort_scratch = b + ((8ull * n + 255) & ~255ull);
    v3 vlo = v3{lo[0], lo[1], lo[2]};
    v3 vsc;
    // one scale for all axes (the cube over the largest extent): Morton bits follow physical size, so a
    // flat scene does not spend its high-order splits on its thin axis
    float ext = hi[0] - lo[0];
    if (hi[1] - lo[1] > ext) ext = hi[1] - lo[1];
    if (hi[2] - lo[2] > ext) ext = hi[2] - lo[2];
    const float sc1 = (ext > 0.0f) ? 1024.0f / ext : 0.0f;
    vsc.x = sc1;
    vsc.y = sc1;
    vsc.z = sc1;
    k_morton<<<(n + 255) / 256, 256, 0, s>>>(positions_dev, n, vlo, vsc, codes);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    uint32_t* perm_tmp = nullptr;
    if ((e = cudaMalloc(&perm_tmp, sizeof(uint32_t) * n)) != cudaSuccess) return e;
    e = launch_sort_pairs(codes, nullptr, sorted_codes, perm_tmp, n, nullptr, 30, sort_scratch, err, s);
    if (e != cudaSuccess) {
        cudaFree(perm_tmp);
        return e;
    }
    k_gather_tris<<<(n + 255) / 256, 256, 0, s>>>(positions_dev, perm_tmp, n, h.tris, perm);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) {
        cudaFree(perm_tmp);
        return e;
    }
    k_leaf_spheres<<<(sizes[0] + 127) / 128, 128, 0, s>>>(h.tris, n, cluster, sizes[0], h.spheres);
    note_launch();
    uint64_t span = cluster;
    for (uint32_t l = 1; l < levels; ++l) {
        span *= 8;
        k_level_spheres<<<(sizes[l] * 32 + 127) / 128, 128, 0, s>>>(h.tris, n, span, sizes[l],
                                                                   h.spheres + h.level_off[l]);
        note_launch();
    }
    e = cudaGetLastError();
    cudaStreamSynchronize(s);
    cudaFree(perm_tmp);
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace rsh
