// Object bounding-sphere hierarchy over the scene's triangles.
//
// Reference: one minimal enclosing sphere per mesh from the GPL Miniball (BoundingSphere.cpp:9-63),
// packed as {centre, radius, firstTri, lastTri} (main.cpp:2445-2470) and culled against the top ray
// nodes (CalculateBoundingSpheresIntersections, RayTracer.cu:1152-1280); triangles then get a bounding
// sphere each (CreateTriangleBoundingSphere, :301-376) inside the descent. Here the object spheres
// become a full sphere tree built on the GPU, level by level, every level a list of nodes whose children
// are consecutive nodes of the level below:
//   1. Morton code (10 bits per axis) of every triangle centroid over the cube around the scene box;
//   2. stable onesweep sort of (code, triangle id) -> cluster order; gather the triangles (original id
//      kept in the first vertex's w);
//   3. boundary strength before sorted triangle k: the highest differing bit of the 64-bit keys
//      (code << 32 | k) of triangles k-1 and k (the splits of a binary radix tree over the keys);
//   4. level 0 groups triangles into clusters of at most `cluster`, every level above groups the level
//      below into nodes of at most 8: the items are cut exactly where the recursive split at the
//      strongest boundary would stop, i.e. boundary j is a cut iff the range it splits (bounded by the
//      nearest stronger boundaries on either side) holds more than G items -- decided from a window of
//      G items on each side; the cut positions are compacted with the compress kernel. A level whose
//      groups would reduce too little (< 2x for clusters, < 4x above) is cut into fixed groups of G;
//   5. every node's sphere from all vertices of its triangle range: centre = midpoint of the vertex
//      box, radius = max vertex distance (x (1 + 2^-20));
//   6. up to the first level with at most 8 nodes (the children of the virtual root).
// Every sphere encloses every vertex below it, so the hierarchy never culls a real hit. Child ranges are
// stored per level as size + 1 starts: node j of level l covers [kids[l][j], kids[l][j + 1]) of level l-1
// (of the triangles, for level 0).
#include <algorithm>

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

// boundary strength before sorted triangle k (k = 0 and k = T: 64, stronger than any)
__global__ void k_delta_tri(const uint32_t* __restrict__ scode, uint32_t T, uint32_t* __restrict__ dtri) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > T) return;
    uint32_t d = 64u;
    if (k > 0 && k < T) {
        const uint32_t a = __ldg(scode + k - 1), b = __ldg(scode + k);
        d = (a != b) ? 32u + (31u - (uint32_t)__clz(a ^ b)) : 31u - (uint32_t)__clz((k - 1) ^ k);
    }
    dtri[k] = d;
}

// Cut flags of one level: key 0 (kept by the compaction) where a group starts, RSH_KEY_NONE elsewhere.
// start == nullptr: the items are the triangles themselves.
__global__ void k_level_cuts(const uint32_t* __restrict__ dtri, const uint32_t* __restrict__ start, uint32_t n,
                             uint32_t G, uint32_t* __restrict__ cutkey) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    auto delta = [&](uint32_t q) -> uint32_t {
        return (q == 0 || q >= n) ? 64u : __ldg(dtri + (start ? __ldg(start + q) : q));
    };
    bool cut = (j == 0);
    if (!cut) {
        const uint32_t d = delta(j);
        int64_t lo = -1, hi = -1;
        for (int64_t q = (int64_t)j - 1; q >= 0 && q >= (int64_t)j - (int64_t)G; --q)
            if (delta((uint32_t)q) > d) {
                lo = q;
                break;
            }
        for (uint64_t q = (uint64_t)j + 1; q <= n && q <= (uint64_t)j + G; ++q)
            if (delta((uint32_t)q) > d) {
                hi = (int64_t)q;
                break;
            }
        cut = lo < 0 || hi < 0 || (hi - lo) > (int64_t)G;
    }
    cutkey[j] = cut ? 0u : RSH_KEY_NONE;
}

__global__ void k_fixed_firsts(uint32_t* __restrict__ firsts, uint32_t nn, uint32_t G) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < nn) firsts[g] = g * G;
}

// Node g of the new level: children [firsts[g], firsts[g+1]) of the items, triangles
// [start(firsts[g]), start(firsts[g+1])); writes the level's child-range starts (triangle starts at level 0)
// and the new items' triangle starts (both nn + 1 entries).
__global__ void k_level_nodes(const uint32_t* __restrict__ firsts, uint32_t nn, uint32_t n,
                              const uint32_t* __restrict__ start, uint32_t T, bool level0,
                              uint32_t* __restrict__ kids, uint32_t* __restrict__ new_start) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > nn) return;
    const uint32_t f = (g < nn) ? __ldg(firsts + g) : n;
    const uint32_t ts = (f >= n) ? T : (start ? __ldg(start + f) : f);
    kids[g] = level0 ? ts : f;
    new_start[g] = ts;
}

// One warp per node: the sphere over every vertex of the node's triangle range. Min/max and max
// reductions are exact in any order.
// Also the node's box, widened by `pad` on every side, whose spare w words hold the node's child link as
// raw u32 bits. A cluster (level 0): lo.w = its first triangle, hi.w = its triangle count. A node of level
// l >= 1: lo.w = its whole single-ray job-stack entry, l << 27 | (children - 1) << 24 | absolute node index
// of its first child (`child_off` + the level's child-range start), hi.w = its child count. A single ray
// that tests a node's box pushes that word as it is and, when it pops it, loads the children's boxes
// directly, with no child-range lookup in between. Traversals rely on every node above level 0 having 1
// to 8 children; a node outside that range raises RSH_DEVERR_OVERFLOW (its entry then lists 1 or 8).
__global__ void k_level_spheres(const float4* __restrict__ tris, const uint32_t* __restrict__ tstart, uint32_t nnodes,
                                const uint32_t* __restrict__ kids, uint32_t child_off, uint32_t level,
                                float4* __restrict__ sph, float4* __restrict__ box, float pad, uint32_t* err) {
    const uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (j >= nnodes) return;
    const uint64_t v0 = 3ull * __ldg(tstart + j), v1 = 3ull * __ldg(tstart + j + 1);
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
    if (lane == 0) {
        const uint32_t k0 = __ldg(kids + j), k1 = __ldg(kids + j + 1);
        uint32_t link = k0;  // level 0: the first triangle
        if (level > 0u) {
            uint32_t n = k1 - k0;
            if (k1 <= k0 || n > 8u) {
                raise_device_error(err, RSH_DEVERR_OVERFLOW);
                n = k1 <= k0 ? 1u : 8u;
            }
            link = (level << 27) | ((n - 1u) << 24) | ((child_off + k0) & 0xFFFFFFu);
        }
        box[2 * j] = make_float4(mnx - pad, mny - pad, mnz - pad, __uint_as_float(link));
        box[2 * j + 1] = make_float4(mxx + pad, mxy + pad, mxz + pad, __uint_as_float(k1 - k0));
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
    const size_t T = tri_count;
    // codes + sorted codes, sort scratch, then dtri, two start arrays, cut keys, firsts, compress outputs
    const size_t a = 8 * T + 256;
    const size_t b = std::max(sort_scratch_bytes(tri_count, 30), compress_scratch_bytes(tri_count)) + 256;
    return a + b + 4 * (T + 1) * 7 + 4096;
}

cudaError_t build_object_hierarchy(const float4* positions_dev, uint32_t n, uint32_t cluster,
                                   const float lo[3], const float hi[3], ObjHierarchy& h,
                                   void* scratch, size_t scratch_bytes, uint32_t* err, cudaStream_t s) {
    (void)scratch_bytes;
    h.tri_count = n;
    h.cluster = cluster;
    h.levels = 0;
    if (n == 0) return cudaSuccess;
    cudaError_t e;
    // node capacity: level 0 holds at most n nodes, every level above at most (size + 3) / 4
    const size_t node_cap = (size_t)n + (n + 2) / 3 + 64;
    if ((e = cudaMalloc(&h.spheres, sizeof(float4) * node_cap)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.kids, sizeof(uint32_t) * (node_cap + 16))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.tris, sizeof(float4) * 3ull * n)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.order, sizeof(uint32_t) * n)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&h.boxes, 2 * sizeof(float4) * node_cap)) != cudaSuccess) return e;

    char* b = static_cast<char*>(scratch);
    uint32_t* codes = reinterpret_cast<uint32_t*>(b);
    uint32_t* sorted_codes = codes + n;
    uint32_t* perm = reinterpret_cast<uint32_t*>(h.order);  // sorted values land in order[] first
    char* work = b + ((8ull * n + 255) & ~255ull);
    void* sort_scratch = work;
    char* rest = work + ((std::max(sort_scratch_bytes(n, 30), compress_scratch_bytes(n)) + 255) & ~255ull);
    uint32_t* dtri = reinterpret_cast<uint32_t*>(rest);
    uint32_t* startA = dtri + (n + 1);
    uint32_t* startB = startA + (n + 1);
    uint32_t* cutkey = startB + (n + 1);
    uint32_t* firsts = cutkey + (n + 1);
    uint32_t* cko = firsts + (n + 1);
    uint32_t* cbo = cko + (n + 1);
    uint32_t* counts = cbo + (n + 1);
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
    k_delta_tri<<<(n + 256) / 256, 256, 0, s>>>(sorted_codes, n, dtri);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) {
        cudaFree(perm_tmp);
        return e;
    }
    // cluster boxes are widened by 1e-5 of the scene's largest coordinate magnitude: far more than the
    // rounding of a float slab test over the scene, so the box cull never drops a hit of the watertight test
    float smax = 0.0f;
    for (int a = 0; a < 3; ++a) smax = fmaxf(smax, fmaxf(fabsf(lo[a]), fabsf(hi[a])));
    const float box_pad = 1e-5f * smax + 1e-30f;
    // levels, bottom up; each level's size is read back (a scene build, not a per-frame step)
    uint32_t items = n, total = 0;
    const uint32_t* start = nullptr;  // items of level 0 are the triangles
    uint32_t* nstart = startA;
    while (true) {
        const uint32_t l = h.levels;
        const uint32_t G = (l == 0) ? cluster : 8u;
        k_level_cuts<<<(items + 255) / 256, 256, 0, s>>>(dtri, start, items, G, cutkey);
        note_launch();
        if ((e = launch_compress(cutkey, items, firsts, cko, cbo, counts, work, err, s)) != cudaSuccess) break;
        uint32_t nn = 0;
        if ((e = cudaMemcpyAsync(&nn, counts, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        // fixed groups of G when the Morton groups reduce too little
        if ((l == 0 && 2ull * nn > (uint64_t)items + 1) || (l > 0 && 4ull * nn > (uint64_t)items + 3) || nn == 0) {
            nn = (items + G - 1) / G;
            k_fixed_firsts<<<(nn + 255) / 256, 256, 0, s>>>(firsts, nn, G);
            note_launch();
        }
        if ((size_t)total + nn > node_cap) {
            e = cudaErrorInvalidValue;
            break;
        }
        h.level_off[l] = total;
        h.level_size[l] = nn;
        k_level_nodes<<<(nn + 256) / 256, 256, 0, s>>>(firsts, nn, items, start, n, l == 0,
                                                       h.kids + total + l, nstart);
        note_launch();
        k_level_spheres<<<(nn * 32 + 127) / 128, 128, 0, s>>>(h.tris, nstart, nn, h.kids + total + l,
                                                              l == 0 ? 0u : h.level_off[l - 1], l,
                                                              h.spheres + total, h.boxes + 2ull * total, box_pad,
                                                              err);
        note_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        total += nn;
        h.levels = l + 1;
        start = nstart;
        nstart = (nstart == startA) ? startB : startA;
        items = nn;
        if (items <= 8 || h.levels >= 16) break;
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(perm_tmp);
    if (e != cudaSuccess) return e;
    if (e2 != cudaSuccess || (e2 = cudaGetLastError()) != cudaSuccess) return e2;
    // the single-ray box tree over the same Morton-ordered triangles, with the same padding
    return build_box_tree(h, box_pad, s);
}

}  // namespace rsh
