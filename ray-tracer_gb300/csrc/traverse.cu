// Hierarchy-vs-hierarchy traversal emitting (packet, triangle-cluster) candidates.
//
// Reference: HierarchyTraversalWarmUpWrapper (RayTracer.cu:2537-2739: top ray nodes x object spheres
// -> interval flags -> scan -> (node, tri) records -> per-triangle-sphere test -> scan-compact ->
// blocking D2H of the count) and HierarchyTraversalWrapper (:2741-2852: per level, expand each record
// x8, test, scan, compact, D2H), inside a host loop over 5000-triangle batches (main.cpp:685-755).
//
// GB300 form: one persistent launch, one warp per level-1 ray node (8 packets) taken from an atomic
// work counter. The warp walks the object-sphere tree depth-first with a shared-memory stack of
// (object node, packet mask): at every node the 32 lanes test its <= 8 children against the <= 8
// still-active packets (8 children x 8 packets = 64 tests, two per lane), and ballots give each
// child's surviving packet mask. Children that are clusters emit one candidate per surviving packet,
// compacted with a warp scan and one atomicAdd per warp; inner children are pushed. No dense
// node x triangle matrix, no per-level host sync. If the candidate buffer fills, the warp records the
// first unfinished work unit (atomicMin) and stops; the host drains the buffer and resumes there.
// With ray_level >= 1, rays leave their packet at and below that object-tree level (and at once when the
// packet's cone is wider than a half-space) and emit per-ray (ray, cluster) candidates instead.
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"
#include "tests.cuh"

namespace cg = cooperative_groups;

namespace rsh {

namespace {
constexpr int TV_WARPS = 4;
constexpr int TV_STACK = 96;
}

// Appends one candidate with one atomic per group of lanes that reach this point together.
RSH_DEV bool emit_candidate(const TravArgs& a, unsigned long long val) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(a.cand_count, (unsigned long long)g.size());
    base = g.shfl(base, 0);
    const unsigned long long pos = base + g.thread_rank();
    if (pos >= a.capacity) return false;
    a.cand[pos] = val;
    return true;
}

// A ray leaves its packet and descends the subtree of (L0, idx0) alone, testing every child sphere
// against itself, and emits one candidate per cluster whose sphere it pierces. False: buffer full.
RSH_DEV bool ray_emit(const TravArgs& a, uint32_t k, float4 o, float4 d, uint32_t L0, uint32_t idx0,
                      unsigned long long& tests) {
    uint32_t stk[72];
    int sp = 0;
    stk[sp++] = (L0 << 24) | idx0;
    bool ok = true;
    while (sp > 0) {
        const uint32_t e = stk[--sp];
        const uint32_t L = e >> 24, idx = e & 0xFFFFFFu;
        const uint32_t cl = L - 1u;
        uint32_t first, cnt;
        node_children(a.kids, a.lvl_off, a.lvl_size, a.levels, L, idx, first, cnt);
        const float4* sb = a.spheres + a.lvl_off[cl] + first;
        for (uint32_t c = 0; c < cnt; ++c) {
            ++tests;
            if (!ray_hits_sphere(o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, __ldg(sb + c))) continue;
            if (cl == 0) {
                ok = emit_candidate(a, ((unsigned long long)k << 32) | 0x80000000ull | (first + c)) && ok;
            } else if (sp < 72) {
                stk[sp++] = (cl << 24) | (first + c);
            }
        }
    }
    return ok;
}

__global__ void __launch_bounds__(TV_WARPS * 32) k_traverse(TravArgs a) {
    __shared__ uint32_t s_stack[TV_WARPS][TV_STACK];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t n = dev_count(a.d_count, a.max_rays);
    const uint32_t P = a.packet;
    const uint32_t n0 = (n + P - 1) / P;
    const uint32_t n1 = (n0 + 7) / 8;
    const uint32_t ch = lane & 7u, q = lane >> 3;
    const uint32_t levels = a.levels;
    unsigned long long tests = 0;
    uint32_t* stack = s_stack[warp];

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(&a.work[0], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= n1 || u >= a.unit_end) break;
        if (*(volatile uint32_t*)&a.work[1] != 0xFFFFFFFFu) break;  // an overflow happened: stop
        // this lane's two packets: 2q and 2q+1 of the unit
        const uint32_t p0 = 8u * u + 2u * q, p1 = p0 + 1u;
        NodeR P0, P1;
        bool v0 = false, v1 = false;
        if (p0 < n0) {
            P0 = load_node(a.nodes, a.node_off[0] + p0);
            v0 = P0.count > 0;
        }
        if (p1 < n0) {
            P1 = load_node(a.nodes, a.node_off[0] + p1);
            v1 = P1.count > 0;
        }
        const uint32_t b0 = __ballot_sync(0xffffffffu, v0), b1 = __ballot_sync(0xffffffffu, v1);
        uint32_t mask = 0;
#pragma unroll
        for (uint32_t g = 0; g < 4; ++g)
            mask |= (((b0 >> (8u * g)) & 1u) << (2u * g)) | (((b1 >> (8u * g)) & 1u) << (2u * g + 1u));
        if (mask == 0) continue;
        const uint32_t f0 = __ballot_sync(0xffffffffu, v0 && !(P0.cs > 0.0f));
        const uint32_t f1 = __ballot_sync(0xffffffffu, v1 && !(P1.cs > 0.0f));
        uint32_t fullmask = 0;
#pragma unroll
        for (uint32_t g = 0; g < 4; ++g)
            fullmask |= (((f0 >> (8u * g)) & 1u) << (2u * g)) | (((f1 >> (8u * g)) & 1u) << (2u * g + 1u));
        int sp = 0;
        if (lane == 0) stack[0] = (levels << 28) | mask;  // virtual root above the top level
        sp = 1;
        __syncwarp();
        bool failed = false;
        while (sp > 0) {
            const uint32_t e = stack[sp - 1];
            __syncwarp();
            --sp;
            const uint32_t L = e >> 28, idx = (e >> 8) & 0xFFFFFu;
            uint32_t m = e & 0xFFu;
            if (a.ray_level > 0) {
                // rays leave their packet below the switch level (at once for full cones) and emit
                // per-ray candidates
                const uint32_t m_ray = (L <= a.ray_level) ? m : (m & fullmask);
                if (m_ray) {
                    const uint32_t nr = __popc(m_ray) * P;
                    bool ok = true;
                    for (uint32_t ir = lane; ir < nr; ir += 32) {
                        uint32_t pmm = m_ray;
                        for (uint32_t s2 = 0; s2 < ir / P; ++s2) pmm &= pmm - 1u;
                        const uint32_t k = 8u * u * P + (__ffs(pmm) - 1u) * P + (ir % P);
                        if (k >= n) continue;
                        const uint32_t id = a.sorted_ids ? __ldg(a.sorted_ids + k) : k;
                        if (id >= a.max_rays) continue;
                        float4 o, d;
                        load_ray(a.rays, id, o, d);
                        if (!(d.w > o.w)) continue;
                        ok = ray_emit(a, k, o, d, L, idx, tests) && ok;
                    }
                    __syncwarp();
                    if (__any_sync(0xffffffffu, !ok)) {
                        failed = true;
                        if (lane == 0) atomicMin(&a.work[1], u);
                        break;
                    }
                    m &= ~m_ray;
                    if (m == 0) continue;
                }
            }
            const uint32_t cl = L - 1u;
            uint32_t first, cnt;
            node_children(a.kids, a.lvl_off, a.lvl_size, levels, L, idx, first, cnt);
            const bool has = ch < cnt;
            float4 S = make_float4(0.f, 0.f, 0.f, 0.f);
            if (has) S = __ldg(a.spheres + a.lvl_off[cl] + first + ch);
            const bool t0 = has && ((m >> (2u * q)) & 1u);
            const bool t1 = has && ((m >> (2u * q + 1u)) & 1u);
            const bool r0 = t0 && node_hits_sphere(P0, S);
            const bool r1 = t1 && node_hits_sphere(P1, S);
            tests += (t0 ? 1u : 0u) + (t1 ? 1u : 0u);
            const uint32_t h0 = __ballot_sync(0xffffffffu, r0), h1 = __ballot_sync(0xffffffffu, r1);
            uint32_t cm = 0;
#pragma unroll
            for (uint32_t g = 0; g < 4; ++g)
                cm |= (((h0 >> (ch + 8u * g)) & 1u) << (2u * g)) | (((h1 >> (ch + 8u * g)) & 1u) << (2u * g + 1u));
            if (lane >= 8u) cm = 0;
            if (cl == 0) {
                // emit (packet, cluster) candidates for lanes 0..7 (= children)
                const uint32_t c = __popc(cm);
                uint32_t inc = c;
#pragma unroll
                for (int d = 1; d < 8; d <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, d);
                    if (lane >= (uint32_t)d) inc += y;
                }
                const uint32_t total = __shfl_sync(0xffffffffu, inc, 7);
                if (total) {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(a.cand_count, (unsigned long long)total);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (base + total > a.capacity) {
                        failed = true;
                        if (lane == 0) atomicMin(&a.work[1], u);
                    }
                    unsigned long long pos = base + inc - c;
                    uint32_t bits = cm;
                    while (bits) {
                        const uint32_t p = __ffs(bits) - 1u;
                        bits &= bits - 1u;
                        if (pos < a.capacity)
                            a.cand[pos] = ((unsigned long long)(8u * u + p) << 32) | (first + ch);
                        ++pos;
                    }
                }
                if (failed) break;
            } else {
                const uint32_t pb = __ballot_sync(0xffffffffu, cm != 0u);
                if (sp + __popc(pb) > TV_STACK) {
                    raise_device_error(a.err, RSH_DEVERR_OVERFLOW);
                    failed = true;
                    if (lane == 0) atomicMin(&a.work[1], u);
                    break;
                }
                if (cm) stack[sp + __popc(pb & lanemask_lt())] = (cl << 28) | ((first + ch) << 8) | cm;
                sp += __popc(pb);
                __syncwarp();
            }
        }
        if (failed) break;
    }
    // node-test counter
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) tests += __shfl_xor_sync(0xffffffffu, tests, d);
    if (lane == 0 && a.node_tests) atomicAdd(a.node_tests, tests);
}

cudaError_t launch_traverse(const TravArgs& a, cudaStream_t s) {
    int sms = 152;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_traverse, TV_WARPS * 32, 0);
    if (per_sm < 1) per_sm = 1;
    const uint32_t units = (((a.max_rays + a.packet - 1) / a.packet) + 7) / 8;
    uint32_t grid = (uint32_t)(sms * per_sm);
    const uint32_t need = (units + TV_WARPS - 1) / TV_WARPS;
    if (need < grid) grid = need > 0 ? need : 1;
    k_traverse<<<grid, TV_WARPS * 32, 0, s>>>(a);
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
