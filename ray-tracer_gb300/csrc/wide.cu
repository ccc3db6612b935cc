// The single-ray box tree: an 8-wide bounding-volume tree over the scene's triangles that the batched form's
// rays-only kernel (fused.cu k_fused_rays) descends. It is built beside the object-sphere hierarchy (objh.cu),
// which the packet traversals and the exported level structure keep using.
//
// Build, from the triangles in the object hierarchy's Morton order:
//  1. A binary tree by PLOC (Meister & Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
//     Hierarchy Construction", IEEE TVCG 2018): every pass, each cluster finds the neighbour within R
//     positions of the Morton-ordered cluster list whose merged box has the smallest surface area (ties to
//     the nearer-indexed one), mutual nearest neighbours merge (the merged node takes the lower position),
//     and the list is compacted in order, until one cluster is left. A node's surface-area measure is
//     (x y + y z) + x z of its box extents, all in FP32, so the host restatement builds the same tree.
//  2. Triangles laid out in the binary tree's depth-first order (left first), so every subtree's triangles
//     are one contiguous range.
//  3. Collapse to 8-wide nodes by the surface-area cost of the single-ray traversal, chosen by dynamic
//     programming over the binary tree (children before parents, pass by pass): with A(x) the area
//     measure of subtree x, f(x, k) = the least cost of covering x's subtree with exactly k child slots
//     of its parent: f(x, 1) = min(A(x) (8 + triangles) if x has at most `cluster` triangles (a cluster),
//     min over 2 <= j <= 8 of A(x) (16 + j) + f(x, j) (a node with j children)), ties to the cluster and
//     to the smaller j; f(x, k >= 2) = min over 1 <= i < k of f(left, i) + f(right, k - i), ties to the
//     smaller i; a single triangle has only f(., 1). The weights (16 + children per node step, 8 +
//     triangles per cluster step) follow the traversal kernel, whose cost tracks its steps more than its
//     box tests. Every f is an FP32 sum in a fixed order, so the host restatement makes the same choices.
//     Then breadth first: a node's children are the slots of its decomposition (left parts first), in
//     consecutive slots allocated level after level in queue order.
// Slot layout (2 float4 per slot, padded box lo and hi): a cluster keeps its first triangle in lo.w and
// 0x80000000 | its triangle count in hi.w; a node keeps its single-ray stack entry in lo.w,
// 1 << 27 | (children - 1) << 24 | first child slot, and its child count in hi.w. Slot 0 is unused; the
// root's entry lists its children from slot 1.
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {

constexpr int PLOC_R = 8;  // PLOC search radius
constexpr uint32_t CLUSTER_BIT = 0x80000000u;

struct WNode {
    float4 lo;  // box min xyz, w = triangle count (u32 bits)
    float4 hi;  // box max xyz
};

RSH_DEV float box_area(float4 a, float4 b) {
    const float x = b.x - a.x, y = b.y - a.y, z = b.z - a.z;
    return (x * y + y * z) + x * z;
}
RSH_DEV float merged_area(const WNode& p, const WNode& q) {
    const float4 a = make_float4(fminf(p.lo.x, q.lo.x), fminf(p.lo.y, q.lo.y), fminf(p.lo.z, q.lo.z), 0.f);
    const float4 b = make_float4(fmaxf(p.hi.x, q.hi.x), fmaxf(p.hi.y, q.hi.y), fmaxf(p.hi.z, q.hi.z), 0.f);
    return box_area(a, b);
}

__global__ void k_wide_leaves(const float4* __restrict__ tris, uint32_t n, WNode* __restrict__ nodes,
                              int2* __restrict__ ch, int32_t* __restrict__ cur) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 a = __ldg(tris + 3ull * k), b = __ldg(tris + 3ull * k + 1), c = __ldg(tris + 3ull * k + 2);
    WNode w;
    w.lo = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z),
                       __uint_as_float(1u));
    w.hi = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z), 0.f);
    nodes[k] = w;
    ch[k] = make_int2(-(int32_t)k - 1, 0);
    cur[k] = (int32_t)k;
}

// nearest neighbour of every cluster within PLOC_R positions (ties: the lower position)
__global__ void k_ploc_nn(const int32_t* __restrict__ cur, uint32_t n, const WNode* __restrict__ nodes,
                          int32_t* __restrict__ nn) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const WNode me = nodes[cur[i]];
    const uint32_t j0 = i > (uint32_t)PLOC_R ? i - PLOC_R : 0u;
    const uint32_t j1 = min(n - 1u, i + (uint32_t)PLOC_R);
    float best = __int_as_float(0x7f800000);
    int32_t bj = -1;
    for (uint32_t j = j0; j <= j1; ++j) {
        if (j == i) continue;
        const float a = merged_area(me, nodes[cur[j]]);
        if (a < best) {
            best = a;
            bj = (int32_t)j;
        }
    }
    nn[i] = bj;
}

// keep[i]: position i stays in the list (a non-mutual cluster, or the lower position of a mutual pair);
// merge[i]: position i is the lower position of a mutual pair
__global__ void k_ploc_flags(const int32_t* __restrict__ nn, uint32_t n, uint32_t* __restrict__ keep,
                             uint32_t* __restrict__ merge) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t j = nn[i];
    const bool mutual = j >= 0 && nn[j] == (int32_t)i;
    keep[i] = (!mutual || (int32_t)i < j) ? 1u : 0u;
    merge[i] = (mutual && (int32_t)i < j) ? 1u : 0u;
}

__global__ void k_ploc_emit(const int32_t* __restrict__ cur, uint32_t n, const int32_t* __restrict__ nn,
                            const uint32_t* __restrict__ keep, const uint32_t* __restrict__ kpos,
                            const uint32_t* __restrict__ mpos, uint32_t node_base, WNode* __restrict__ nodes,
                            int2* __restrict__ ch, int32_t* __restrict__ nxt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    int32_t id = cur[i];
    const int32_t j = nn[i];
    if (j > (int32_t)i && nn[j] == (int32_t)i) {
        const int32_t a = cur[i], b = cur[j];
        const WNode p = nodes[a], q = nodes[b];
        WNode m;
        m.lo = make_float4(fminf(p.lo.x, q.lo.x), fminf(p.lo.y, q.lo.y), fminf(p.lo.z, q.lo.z),
                           __uint_as_float(__float_as_uint(p.lo.w) + __float_as_uint(q.lo.w)));
        m.hi = make_float4(fmaxf(p.hi.x, q.hi.x), fmaxf(p.hi.y, q.hi.y), fmaxf(p.hi.z, q.hi.z), 0.f);
        id = (int32_t)(node_base + mpos[i]);
        nodes[id] = m;
        ch[id] = make_int2(a, b);
    }
    nxt[kpos[i]] = id;
}

// depth-first position of the first triangle of each child of the nodes [b, e) (whose own is known)
__global__ void k_wide_first(const int2* __restrict__ ch, const WNode* __restrict__ nodes, uint32_t b, uint32_t e,
                             uint32_t* __restrict__ first) {
    const uint32_t x = b + blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= e) return;
    const int2 c = ch[x];
    const uint32_t f = first[x];
    first[c.x] = f;
    first[c.y] = f + __float_as_uint(nodes[c.x].lo.w);
}

__global__ void k_wide_tris(const float4* __restrict__ tris, uint32_t n, const uint32_t* __restrict__ first,
                            float4* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint64_t d = 3ull * first[k];
    out[d] = __ldg(tris + 3ull * k);
    out[d + 1] = __ldg(tris + 3ull * k + 1);
    out[d + 2] = __ldg(tris + 3ull * k + 2);
}

// per node of the binary tree: f(x, 1..8) and its choices packed in one word -- bits 3 (k - 2) .. for the
// split i of f(x, k), k = 2..8; bits 21-23: j - 2 of the node choice; bit 24: x is a cluster
constexpr float COST_NODE = 16.0f, COST_CLUSTER = 8.0f;
constexpr uint32_t CH_CLUSTER = 1u << 24;

RSH_DEV void collapse_costs(const WNode& w, uint32_t cluster, float* f, uint32_t& choice) {
    const float A = box_area(w.lo, w.hi);
    const uint32_t cnt = __float_as_uint(w.lo.w);
    float best = __int_as_float(0x7f800000);
    uint32_t bj = 0;
    for (uint32_t j = 2; j <= 8; ++j) {
        const float c = A * (COST_NODE + (float)j) + f[j - 1];
        if (c < best) {
            best = c;
            bj = j;
        }
    }
    const float ccl = cnt <= cluster ? A * (COST_CLUSTER + (float)cnt) : __int_as_float(0x7f800000);
    if (ccl <= best) {
        f[0] = ccl;
        choice |= CH_CLUSTER;
    } else {
        f[0] = best;
        choice |= (bj - 2u) << 21;
    }
}

__global__ void k_collapse_leaves(const WNode* __restrict__ nodes, uint32_t n, uint32_t cluster, float* __restrict__ fc,
                                  uint32_t* __restrict__ choice) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    float f[8];
    for (int k = 0; k < 8; ++k) f[k] = __int_as_float(0x7f800000);
    uint32_t ch = 0;
    collapse_costs(nodes[x], cluster, f, ch);
    for (int k = 0; k < 8; ++k) fc[8ull * x + k] = f[k];
    choice[x] = ch;
}

// the nodes [b, e) of one PLOC pass (their children come from earlier passes)
__global__ void k_collapse_pass(const WNode* __restrict__ nodes, const int2* __restrict__ chb, uint32_t b, uint32_t e,
                                uint32_t cluster, float* __restrict__ fc, uint32_t* __restrict__ choice) {
    const uint32_t x = b + blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= e) return;
    const int2 lr = chb[x];
    float fl[8], fr[8], f[8];
    for (int k = 0; k < 8; ++k) {
        fl[k] = fc[8ull * lr.x + k];
        fr[k] = fc[8ull * lr.y + k];
    }
    uint32_t ch = 0;
    f[0] = __int_as_float(0x7f800000);
    for (uint32_t k = 2; k <= 8; ++k) {
        float best = __int_as_float(0x7f800000);
        uint32_t bi = 1;
        for (uint32_t i = 1; i < k; ++i) {
            const float c = fl[i - 1] + fr[k - i - 1];
            if (c < best) {
                best = c;
                bi = i;
            }
        }
        f[k - 1] = best;
        ch |= bi << (3u * (k - 2u));
    }
    collapse_costs(nodes[x], cluster, f, ch);
    for (int k = 0; k < 8; ++k) fc[8ull * x + k] = f[k];
    choice[x] = ch;
}

// one BFS level of the collapse: the children of every item that is a node (its decomposition into the
// j slots its choice says, left parts first), and their count; a cluster has none. At the root (which has
// no slot of its own) a cluster is its own single child.
__global__ void k_wide_expand(const int32_t* __restrict__ items, uint32_t n, const int2* __restrict__ chb,
                              const uint32_t* __restrict__ choice, bool root, int32_t* __restrict__ kids,
                              uint32_t* __restrict__ nkids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t x = items[i];
    const uint32_t cx = choice[x];
    uint32_t m = 0;
    if (cx & CH_CLUSTER) {
        if (root) kids[8ull * i + m++] = x;
    } else {
        int32_t sy[8];
        uint32_t sk[8], top = 0;
        sy[0] = x;
        sk[0] = ((cx >> 21) & 7u) + 2u;
        top = 1;
        while (top > 0) {
            --top;
            const int32_t y = sy[top];
            const uint32_t k = sk[top];
            if (k == 1u) {
                kids[8ull * i + m++] = y;
                continue;
            }
            const uint32_t si = (choice[y] >> (3u * (k - 2u))) & 7u;
            const int2 lr = chb[y];
            sy[top] = lr.y;  // the right part after the left one
            sk[top] = k - si;
            sy[top + 1] = lr.x;
            sk[top + 1] = si;
            top += 2;
        }
    }
    nkids[i] = m;
}

// writes every item's slot (cluster: triangle range; node: its stack entry) and the next level's items
__global__ void k_wide_write(const int32_t* __restrict__ items, const uint32_t* __restrict__ slots, uint32_t n,
                             const WNode* __restrict__ nodes, const uint32_t* __restrict__ first,
                             const int32_t* __restrict__ kids, const uint32_t* __restrict__ nkids,
                             const uint32_t* __restrict__ kpos, uint32_t slot_base, float pad,
                             float4* __restrict__ boxes, int32_t* __restrict__ next_items,
                             uint32_t* __restrict__ next_slots) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t x = items[i];
    const WNode w = nodes[x];
    const uint32_t m = nkids[i];
    const uint32_t f = slot_base + kpos[i];
    uint32_t lw, hw;
    if (m == 0) {  // a cluster
        lw = first[x];
        hw = CLUSTER_BIT | __float_as_uint(w.lo.w);
    } else {
        lw = (1u << 27) | ((m - 1u) << 24) | (f & 0xFFFFFFu);
        hw = m;
        for (uint32_t q = 0; q < m; ++q) {
            next_items[kpos[i] + q] = kids[8ull * i + q];
            next_slots[kpos[i] + q] = f + q;
        }
    }
    const uint32_t s = slots[i];
    if (s == 0u) return;  // the root has no slot of its own
    boxes[2ull * s] = make_float4(w.lo.x - pad, w.lo.y - pad, w.lo.z - pad, __uint_as_float(lw));
    boxes[2ull * s + 1] = make_float4(w.hi.x + pad, w.hi.y + pad, w.hi.z + pad, __uint_as_float(hw));
}

// Traversal records: the slot tree laid out again for the rays-only kernel, one record per node (per
// block of consecutive child slots), REC_F4 float4 each: the eight children's padded boxes plane by plane
// (lo x, hi x, lo y, hi y, lo z, hi z: 8 floats each) and their eight stack entries. A ray picks the near
// and the far plane of each axis once per record from the sign of its direction, so a child's entry and
// exit distances need no min / max per axis. An unused child has the empty box (lo = +inf, hi = -inf,
// which every ray misses) and entry 0. A child's entry: a cluster's first triangle | (triangles - 1) << 23
// (bit 31 clear; fewer than 2^23 triangles, at most 64 per cluster), or a node's REC_NODE | (children - 1)
// << 28 | record index (kernels.h).

// start[f] = 1 and cnt[f] = children for the first child slot f of every node (the root's at slot 1)
__global__ void k_rec_mark(const float4* __restrict__ boxes, uint32_t nslots, uint32_t root_children,
                           uint32_t* __restrict__ start, uint32_t* __restrict__ cnt) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nslots) return;
    if (t == 0u) {
        start[1] = 1u;
        cnt[1] = root_children;
        return;
    }
    if (__float_as_uint(boxes[2ull * t + 1].w) & CLUSTER_BIT) return;
    const uint32_t e = __float_as_uint(boxes[2ull * t].w);
    const uint32_t f = e & 0xFFFFFFu;
    start[f] = 1u;
    cnt[f] = ((e >> 24) & 7u) + 1u;
}

__global__ void k_rec_write(const float4* __restrict__ boxes, uint32_t nslots, const uint32_t* __restrict__ start,
                            const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ rid,
                            float4* __restrict__ recs) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nslots || !start[f]) return;
    const uint32_t n = cnt[f];
    float* r = reinterpret_cast<float*>(recs + REC_F4 * (size_t)rid[f]);
    uint32_t* re = reinterpret_cast<uint32_t*>(r + 48);
    const float inf = __int_as_float(0x7f800000);
    for (uint32_t c = 0; c < 8u; ++c) {
        if (c < n) {
            const uint32_t t = f + c;
            const float4 b0 = boxes[2ull * t], b1 = boxes[2ull * t + 1];
            r[c] = b0.x;
            r[8 + c] = b1.x;
            r[16 + c] = b0.y;
            r[24 + c] = b1.y;
            r[32 + c] = b0.z;
            r[40 + c] = b1.z;
            const uint32_t lw = __float_as_uint(b0.w);
            const uint32_t hw = __float_as_uint(b1.w);
            re[c] = (hw & CLUSTER_BIT) ? lw | ((hw - CLUSTER_BIT - 1u) << 23)
                                       : REC_NODE | (((lw >> 24) & 7u) << 28) | rid[lw & 0xFFFFFFu];
        } else {
            r[c] = r[16 + c] = r[32 + c] = inf;
            r[8 + c] = r[24 + c] = r[40 + c] = -inf;
            re[c] = 0u;
        }
    }
}

// exclusive scan of n u32 with the total at out[n]: per-block scans, a one-block scan of the block sums,
// then the block offsets added (three launches; the build runs once per scene)
constexpr uint32_t SCAN_B = 1024;
__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ out,
                              uint32_t* __restrict__ sums) {
    __shared__ uint32_t ws[32];
    const uint32_t i = blockIdx.x * SCAN_B + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31u) >= (uint32_t)o) x += y;
    }
    if ((threadIdx.x & 31u) == 31u) ws[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t s = ws[threadIdx.x];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (threadIdx.x >= (uint32_t)o) s += y;
        }
        ws[threadIdx.x] = s;
    }
    __syncthreads();
    const uint32_t warp_off = (threadIdx.x >= 32) ? ws[(threadIdx.x >> 5) - 1] : 0u;
    if (i < n) out[i] = warp_off + x - v;
    if (threadIdx.x == SCAN_B - 1) sums[blockIdx.x] = ws[31];
}
__global__ void k_scan_sums(uint32_t* __restrict__ sums, uint32_t nb, uint32_t* __restrict__ total) {
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nb; base += 32) {
        if (threadIdx.x < 32) {
            const uint32_t j = base + threadIdx.x;
            const uint32_t v = j < nb ? sums[j] : 0u;
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (threadIdx.x >= (uint32_t)o) x += y;
            }
            const uint32_t c = carry;
            if (j < nb) sums[j] = c + x - v;
            __syncwarp();
            if (threadIdx.x == 31) carry = c + x;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}
__global__ void k_scan_add(uint32_t* __restrict__ out, uint32_t n, const uint32_t* __restrict__ sums) {
    const uint32_t i = blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
}
cudaError_t scan_u32(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* sums, cudaStream_t s) {
    const uint32_t nb = (n + SCAN_B - 1) / SCAN_B;
    if (n > 0) {
        k_scan_blocks<<<nb, SCAN_B, 0, s>>>(in, n, out, sums);
        note_launch();
    }
    k_scan_sums<<<1, 32, 0, s>>>(sums, nb, out + n);
    note_launch();
    if (n > 0) {
        k_scan_add<<<nb, SCAN_B, 0, s>>>(out, n, sums);
        note_launch();
    }
    return cudaGetLastError();
}

template <class T>
cudaError_t alloc(T*& p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * (count ? count : 1));
}

// The traversal records of a finished slot tree (slot 0 starts no block, so the root's children are
// record 0).
cudaError_t build_records(ObjHierarchy& h, uint32_t root_children, cudaStream_t s) {
    const uint32_t ns = h.wslots;
    uint32_t *start = nullptr, *cnt = nullptr, *rid = nullptr, *sums = nullptr;
    uint32_t recs = 0;
    cudaError_t e = cudaSuccess;
    if (!(e = alloc(start, ns + 1)) && !(e = alloc(cnt, ns + 1)) && !(e = alloc(rid, ns + 1)) &&
        !(e = alloc(sums, (ns + SCAN_B - 1) / SCAN_B + 1)) && !(e = cudaMemsetAsync(start, 0, 4ull * (ns + 1), s))) {
        k_rec_mark<<<(ns + 255) / 256, 256, 0, s>>>(h.wboxes, ns, root_children, start, cnt);
        note_launch();
        if (!(e = scan_u32(start, ns, rid, sums, s)) &&
            !(e = cudaMemcpyAsync(&recs, rid + ns, 4, cudaMemcpyDeviceToHost, s)) &&
            !(e = cudaStreamSynchronize(s)) && !(e = alloc(h.wnodes, (size_t)REC_F4 * recs))) {
            k_rec_write<<<(ns + 255) / 256, 256, 0, s>>>(h.wboxes, ns, start, cnt, rid, h.wnodes);
            note_launch();
            e = cudaGetLastError();
            h.wnode_count = recs;
            h.wnroot = REC_NODE | ((root_children - 1u) << 28);
        }
    }
    const cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(start);
    cudaFree(cnt);
    cudaFree(rid);
    cudaFree(sums);
    return e != cudaSuccess ? e : e2;
}

}  // namespace

cudaError_t build_box_tree(ObjHierarchy& h, float pad, cudaStream_t s) {
    const uint32_t n = h.tri_count;
    h.wslots = 0;
    h.wroot = 0;
    if (n == 0) return cudaSuccess;
    if ((uint64_t)2 * n + 8 > (1ull << 24)) return cudaErrorInvalidValue;  // slots are 24-bit indices
    const uint32_t cluster = h.cluster;
    const uint32_t cap_nodes = 2 * n;
    WNode* nodes = nullptr;
    int2* chb = nullptr;
    int32_t *cur = nullptr, *nxt = nullptr, *nn = nullptr, *kids = nullptr;
    uint32_t *keep = nullptr, *merge = nullptr, *kpos = nullptr, *mpos = nullptr, *sums = nullptr, *first = nullptr;
    uint32_t *slots = nullptr, *nslots = nullptr, *nk = nullptr, *choice = nullptr;
    float* fc = nullptr;
    cudaError_t e = cudaSuccess;
    const uint32_t nb = (n + SCAN_B - 1) / SCAN_B + 1;
    if ((e = alloc(nodes, cap_nodes)) || (e = alloc(chb, cap_nodes)) || (e = alloc(cur, n)) || (e = alloc(nxt, n)) ||
        (e = alloc(nn, n)) || (e = alloc(keep, n)) || (e = alloc(merge, n)) || (e = alloc(kpos, n + 1)) ||
        (e = alloc(mpos, n + 1)) || (e = alloc(sums, nb)) || (e = alloc(first, cap_nodes)) ||
        (e = alloc(kids, 8ull * n)) || (e = alloc(nk, n)) || (e = alloc(slots, 2ull * n + 8)) ||
        (e = alloc(nslots, 2ull * n + 8)) || (e = alloc(h.wboxes, 2ull * (2ull * n + 8))) ||
        (e = alloc(h.wtris, 3ull * n)) || (e = alloc(fc, 8ull * cap_nodes)) || (e = alloc(choice, cap_nodes))) {
        cudaFree(fc);
        cudaFree(choice);
        cudaFree(nodes);
        cudaFree(chb);
        cudaFree(cur);
        cudaFree(nxt);
        cudaFree(nn);
        cudaFree(keep);
        cudaFree(merge);
        cudaFree(kpos);
        cudaFree(mpos);
        cudaFree(sums);
        cudaFree(first);
        cudaFree(kids);
        cudaFree(nk);
        cudaFree(slots);
        cudaFree(nslots);
        return e;
    }
    auto blocks = [](uint32_t m) { return (m + 255) / 256; };
    // 1. PLOC passes; the nodes created by pass p occupy ids [pass_begin[p], pass_begin[p + 1])
    std::vector<uint32_t> pass_begin{n};
    k_wide_leaves<<<blocks(n), 256, 0, s>>>(h.tris, n, nodes, chb, cur);
    note_launch();
    uint32_t m = n, node_count = n;
    while (m > 1 && e == cudaSuccess) {
        k_ploc_nn<<<blocks(m), 256, 0, s>>>(cur, m, nodes, nn);
        k_ploc_flags<<<blocks(m), 256, 0, s>>>(nn, m, keep, merge);
        note_launch(2);
        if ((e = scan_u32(keep, m, kpos, sums, s)) != cudaSuccess) break;
        if ((e = scan_u32(merge, m, mpos, sums, s)) != cudaSuccess) break;
        k_ploc_emit<<<blocks(m), 256, 0, s>>>(cur, m, nn, keep, kpos, mpos, node_count, nodes, chb, nxt);
        note_launch();
        uint32_t merges = 0;
        if ((e = cudaMemcpyAsync(&merges, mpos + m, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        if (merges == 0) {  // cannot happen (the closest pair is mutual); never loop forever
            e = cudaErrorUnknown;
            break;
        }
        node_count += merges;
        pass_begin.push_back(node_count);
        m -= merges;
        std::swap(cur, nxt);
    }
    int32_t root = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&root, cur, 4, cudaMemcpyDeviceToHost, s);
    // 2. depth-first triangle order: passes from the last (the root's) to the first
    if (e == cudaSuccess) e = cudaMemsetAsync(first + root, 0, 4, s);
    for (size_t p = pass_begin.size() - 1; p > 0 && e == cudaSuccess; --p) {
        const uint32_t b = pass_begin[p - 1], en = pass_begin[p];
        k_wide_first<<<blocks(en - b), 256, 0, s>>>(chb, nodes, b, en, first);
        note_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_wide_tris<<<blocks(n), 256, 0, s>>>(h.tris, n, first, h.wtris);
        note_launch();
        e = cudaGetLastError();
    }
    // 3. collapse costs, children before parents (leaves, then the passes in order), then breadth first:
    // level items (binary node, slot); the root's slot is 0 (none)
    if (e == cudaSuccess) {
        k_collapse_leaves<<<blocks(n), 256, 0, s>>>(nodes, n, cluster, fc, choice);
        note_launch();
        e = cudaGetLastError();
    }
    for (size_t p = 1; p < pass_begin.size() && e == cudaSuccess; ++p) {
        const uint32_t b = pass_begin[p - 1], en = pass_begin[p];
        k_collapse_pass<<<blocks(en - b), 256, 0, s>>>(nodes, chb, b, en, cluster, fc, choice);
        note_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(h.wboxes, 0, 2 * sizeof(float4), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cur, &root, 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(slots, 0, 4, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    uint32_t items = 1, slot_base = 1, root_children = 0;
    bool at_root = true;
    while (items > 0 && e == cudaSuccess) {
        k_wide_expand<<<blocks(items), 256, 0, s>>>(cur, items, chb, choice, at_root, kids, nk);
        note_launch();
        if ((e = scan_u32(nk, items, kpos, sums, s)) != cudaSuccess) break;
        k_wide_write<<<blocks(items), 256, 0, s>>>(cur, slots, items, nodes, first, kids, nk, kpos, slot_base, pad,
                                                   h.wboxes, nxt, nslots);
        note_launch();
        uint32_t total = 0;
        if ((e = cudaMemcpyAsync(&total, kpos + items, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        if (at_root) {
            root_children = total;
            at_root = false;
        }
        slot_base += total;
        items = total;
        std::swap(cur, nxt);
        std::swap(slots, nslots);
    }
    if (e == cudaSuccess) {
        if (root_children == 0) {
            e = cudaErrorUnknown;  // a tree over at least one triangle always has children at its root
        } else {
            h.wroot = (1u << 27) | ((root_children - 1u) << 24) | 1u;
            h.wslots = slot_base;
        }
    }
    // 4. the traversal records
    if (e == cudaSuccess) e = build_records(h, root_children, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(fc);
    cudaFree(choice);
    cudaFree(nodes);
    cudaFree(chb);
    cudaFree(cur);
    cudaFree(nxt);
    cudaFree(nn);
    cudaFree(keep);
    cudaFree(merge);
    cudaFree(kpos);
    cudaFree(mpos);
    cudaFree(sums);
    cudaFree(first);
    cudaFree(kids);
    cudaFree(nk);
    cudaFree(slots);
    cudaFree(nslots);
    if (e != cudaSuccess) return e;
    return e2;
}

}  // namespace rsh
