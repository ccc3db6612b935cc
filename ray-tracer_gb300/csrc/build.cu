// Bottom-up build of the ray-space hierarchy (cone + sphere nodes).
//
// Reference: HierarchyCreationWrapper (RayTracer.cu:2469-2535) with CreateHierarchyLevel0 (:1061-1108,
// 8 consecutive sorted rays -> sphere of origins + cone of directions via CreateHierarchySphere
// :427-446 / CreateHierarchyCone0 :379-406) and CreateHierarchyLevelN (:1110-1150, 8 children via
// CreateHierarchyConeN :408-425). Those merges use acos/cos/sin and are not conservative (a cone can
// miss a ray), so the nodes are redefined to be conservative by construction:
//   leaf (P rays, one lane each, shuffles within the P-lane group):
//     centre = midpoint of the origins' bounding box, radius = max |o - centre|,
//     axis = normalize(sum of directions), cos_spread = min dot(axis, d) - 4e-6 (<= 0: full cone),
//     reach = max(|o - centre| + tmax)  (how far any ray of the node can get from the centre);
//   level L (8 children): box of child spheres -> centre, radius = max(|c_i - c| + r_i),
//     axis = normalize(sum count_i * axis_i), cos_spread = min cos(angle(axis, axis_i) + spread_i),
//     reach = max(|c_i - c| + reach_i).
// Sums are pairwise trees in index order (xor-butterfly 1, 2, 4, ...), reproducible on the host.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr float kRadSlack = 1.0f + 1.0f / 1048576.0f;  // 1 + 2^-20
constexpr float kCosMargin = 4e-6f;
}

uint32_t hierarchy_capacity(uint32_t max_rays, uint32_t packet, uint32_t offsets[4]) {
    const uint32_t n0 = (max_rays + packet - 1) / packet;
    const uint32_t n1 = (n0 + 7) / 8;
    const uint32_t n2 = (n1 + 7) / 8;
    offsets[0] = 0;
    offsets[1] = n0;
    offsets[2] = n0 + n1;
    offsets[3] = n0 + n1 + n2;
    return offsets[3];
}

template <int P>
__global__ void k_build_leaves(const rsh_ray* __restrict__ rays, const uint32_t* __restrict__ sorted_ids,
                               uint32_t max_rays, const uint32_t* __restrict__ d_count,
                               rsh_node* __restrict__ leaves) {
    const uint32_t n = dev_count(d_count, max_rays);
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n_pad = ((n + P - 1) / P) * P;
    if ((k & ~31u) >= n_pad) return;  // whole warp beyond the last packet
    bool active = k < n;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = make_float4(0.f, 0.f, 0.f, -1.f);
    if (active) {
        const uint32_t id = sorted_ids ? __ldg(sorted_ids + k) : k;
        if (id != 0xFFFFFFFFu) {  // padding slot of the batched layout: no ray
            load_ray(rays, id, o, d);
            active = d.w > o.w;
        } else {
            active = false;
        }
    }
    const float inf = __int_as_float(0x7f800000);
    float mnx = active ? o.x : inf, mny = active ? o.y : inf, mnz = active ? o.z : inf;
    float mxx = active ? o.x : -inf, mxy = active ? o.y : -inf, mxz = active ? o.z : -inf;
    float sx = active ? d.x : 0.f, sy = active ? d.y : 0.f, sz = active ? d.z : 0.f;
#pragma unroll
    for (int off = 1; off < P; off <<= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, off));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, off));
        mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, off));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, off));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, off));
        mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, off));
        sx = sx + __shfl_xor_sync(0xffffffffu, sx, off);
        sy = sy + __shfl_xor_sync(0xffffffffu, sy, off);
        sz = sz + __shfl_xor_sync(0xffffffffu, sz, off);
    }
    const uint32_t lane = lane_id();
    const uint32_t gmask = (P == 32) ? 0xffffffffu : (((1u << P) - 1u) << (lane & ~(uint32_t)(P - 1)));
    const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, active) & gmask);
    const v3 c = v3{(mnx + mxx) * 0.5f, (mny + mxy) * 0.5f, (mnz + mxz) * 0.5f};
    const float sl = sqrtf((sx * sx + sy * sy) + sz * sz);
    bool full = !(sl > 1e-20f);
    const v3 a = full ? v3{0.f, 0.f, 1.f} : v3{sx / sl, sy / sl, sz / sl};
    // second phase: radius, cone spread, reach
    const v3 oc = v3{o.x - c.x, o.y - c.y, o.z - c.z};
    const float r2 = active ? dot3(oc, oc) : 0.f;
    float dt = active ? dot3(a, mk3(d)) : inf;
    float rc = active ? sqrtf(r2) + d.w : 0.f;
    float mr2 = r2;
#pragma unroll
    for (int off = 1; off < P; off <<= 1) {
        mr2 = fmaxf(mr2, __shfl_xor_sync(0xffffffffu, mr2, off));
        dt = fminf(dt, __shfl_xor_sync(0xffffffffu, dt, off));
        rc = fmaxf(rc, __shfl_xor_sync(0xffffffffu, rc, off));
    }
    if ((k & (P - 1)) != 0 || k >= n_pad) return;
    float cs = dt - kCosMargin;
    if (!(cs > 0.f)) full = true;
    rsh_node nd;
    nd.c[0] = c.x;
    nd.c[1] = c.y;
    nd.c[2] = c.z;
    nd.radius = sqrtf(mr2) * kRadSlack;
    nd.axis[0] = a.x;
    nd.axis[1] = a.y;
    nd.axis[2] = a.z;
    nd.cos_spread = full ? -1.f : cs;
    nd.sin_spread = full ? 0.f : sqrtf((1.f - cs) * (1.f + cs));
    nd.reach = rc * kRadSlack;
    nd.first = k;
    nd.count = cnt;
    leaves[k / P] = nd;
}

__global__ void k_build_level(rsh_node* __restrict__ nodes, uint32_t child_off, uint32_t parent_off,
                              uint32_t max_rays, const uint32_t* __restrict__ d_count, uint32_t packet,
                              uint32_t level) {
    const uint32_t n = dev_count(d_count, max_rays);
    uint32_t nc = (n + packet - 1) / packet;  // level-0 size
    for (uint32_t l = 1; l < level; ++l) nc = (nc + 7) / 8;
    const uint32_t np = (nc + 7) / 8;
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= np) return;
    const uint32_t c0 = 8 * j, c1 = (8 * j + 8 < nc) ? 8 * j + 8 : nc;
    const float inf = __int_as_float(0x7f800000);
    rsh_node ch[8];
    float mnx = inf, mny = inf, mnz = inf, mxx = -inf, mxy = -inf, mxz = -inf;
    uint32_t count = 0;
    bool full = false;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (uint32_t i = c0; i < c1; ++i) {
        const rsh_node q = nodes[child_off + i];
        ch[i - c0] = q;
        if (q.count == 0) continue;
        count += q.count;
        mnx = fminf(mnx, q.c[0] - q.radius);
        mny = fminf(mny, q.c[1] - q.radius);
        mnz = fminf(mnz, q.c[2] - q.radius);
        mxx = fmaxf(mxx, q.c[0] + q.radius);
        mxy = fmaxf(mxy, q.c[1] + q.radius);
        mxz = fmaxf(mxz, q.c[2] + q.radius);
        if (!(q.cos_spread > 0.f)) full = true;
        const float w = (float)q.count;
        sx = sx + q.axis[0] * w;
        sy = sy + q.axis[1] * w;
        sz = sz + q.axis[2] * w;
    }
    rsh_node nd;
    nd.first = ch[0].first;
    nd.count = count;
    const v3 c = v3{(mnx + mxx) * 0.5f, (mny + mxy) * 0.5f, (mnz + mxz) * 0.5f};
    const float sl = sqrtf((sx * sx + sy * sy) + sz * sz);
    if (!(sl > 1e-20f)) full = true;
    const v3 a = full ? v3{0.f, 0.f, 1.f} : v3{sx / sl, sy / sl, sz / sl};
    float rad = 0.f, reach = 0.f, cs = 1.f;
    for (uint32_t i = c0; i < c1; ++i) {
        const rsh_node& q = ch[i - c0];
        if (q.count == 0) continue;
        const v3 dc = v3{q.c[0] - c.x, q.c[1] - c.y, q.c[2] - c.z};
        const float dl = len3(dc);
        rad = fmaxf(rad, dl + q.radius);
        reach = fmaxf(reach, dl + q.reach);
        if (!full) {
            float ca = dot3(a, v3{q.axis[0], q.axis[1], q.axis[2]});
            ca = fminf(fmaxf(ca, -1.f), 1.f);
            const float sa = sqrtf((1.f - ca) * (1.f + ca));
            cs = fminf(cs, ca * q.cos_spread - sa * q.sin_spread);
        }
    }
    cs = cs - kCosMargin;
    if (!(cs > 0.f)) full = true;
    nd.c[0] = c.x;
    nd.c[1] = c.y;
    nd.c[2] = c.z;
    nd.radius = rad * kRadSlack;
    nd.axis[0] = a.x;
    nd.axis[1] = a.y;
    nd.axis[2] = a.z;
    nd.cos_spread = full ? -1.f : cs;
    nd.sin_spread = full ? 0.f : sqrtf((1.f - cs) * (1.f + cs));
    nd.reach = reach * kRadSlack;
    if (count == 0) {
        nd.c[0] = nd.c[1] = nd.c[2] = 0.f;
        nd.radius = 0.f;
        nd.reach = 0.f;
    }
    nodes[parent_off + j] = nd;
}

cudaError_t launch_build_rsh(const rsh_ray* rays, const uint32_t* sorted_ids, uint32_t max_rays,
                             const uint32_t* d_count, uint32_t packet, rsh_node* nodes,
                             cudaStream_t s) {
    if (max_rays == 0) return cudaSuccess;
    uint32_t off[4];
    hierarchy_capacity(max_rays, packet, off);
    const uint32_t threads = ((max_rays + packet - 1) / packet) * packet;
    const uint32_t grid = (threads + 255) / 256;
    switch (packet) {
        case 8: k_build_leaves<8><<<grid, 256, 0, s>>>(rays, sorted_ids, max_rays, d_count, nodes); break;
        case 16: k_build_leaves<16><<<grid, 256, 0, s>>>(rays, sorted_ids, max_rays, d_count, nodes); break;
        case 32: k_build_leaves<32><<<grid, 256, 0, s>>>(rays, sorted_ids, max_rays, d_count, nodes); break;
        default: return cudaErrorInvalidValue;
    }
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    for (uint32_t lvl = 1; lvl <= 2; ++lvl) {
        const uint32_t np = off[lvl + 1] - off[lvl];
        if (np == 0) break;
        k_build_level<<<(np + 127) / 128, 128, 0, s>>>(nodes, off[lvl - 1], off[lvl], max_rays, d_count,
                                                       packet, lvl);
        note_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace rsh
