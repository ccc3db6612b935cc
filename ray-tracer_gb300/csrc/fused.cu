// Fused persistent traversal + intersection (the batched form's single launch). Two kernels:
//   k_fused_rays (switch level at or above every segment's tree depth, the default): each lane traces one
//     ray at a time from the root, refilled from the warp's current unit of 64 sorted rays; no packet
//     phase and no ray hierarchy; the launch's last units go out as half units, and (instance SHARE) a
//     drained warp's last rays are shared among its idle lanes;
//   k_fused (a lower switch level): packets of the ray hierarchy walk the upper object tree, rays leave
//     them at the switch level, as described next.
//
// Reference: the per-frame loop of HierarchyTraversalWarmUpWrapper -> HierarchyTraversalWrapper ->
// Shadow/ReflectionRayIntersectionWrapper (main.cpp:685-755, RayTracer.cu:2537-3031), which materialises
// (node, triangle) records and resolves hits with atomics. Here one persistent kernel takes work units
// (level-1 ray nodes = 8 packets, never straddling a batch segment) from an atomic counter; each warp
// keeps the unit's rays in shared memory (watertight setup precomputed), walks the segment's
// object-sphere tree depth-first with (node, packet-mask) stack entries, children pushed farthest-first
// so that the nearest subtree is visited first, and at every triangle cluster immediately tests the
// surviving packets' rays against the cluster's triangles staged in shared memory. At and below a
// configurable object-tree level (and at once for packets whose cone is wider than a half-space) rays
// leave their packet and descend the subtree one by one (the ray level of the ray hierarchy).
//   closest hit: per-ray best (t bits << 32 | triangle id) kept in shared memory; after each cluster a
//     packet's `reach` shrinks to max(|o - c| + best t), so later subtrees beyond every current hit are
//     culled by the node test (early termination without changing any result);
//   any hit: a packet leaves the traversal once all its rays are occluded.
// Each ray belongs to exactly one work unit, so results are written with plain stores (no atomics).
#include "common.cuh"
#include "kernels.h"
#include "tests.cuh"

namespace rsh {

namespace {
constexpr int FW = 4;            // warps per block
constexpr int F_STACK = 96;
constexpr int F_MAXK = 32;       // max cluster size staged in shared memory
constexpr uint32_t INVALID_ID = 0xFFFFFFFFu;
constexpr int J_STACK = 96;                // per-lane node stack of a job
constexpr uint32_t J_CAP = 512;            // job queue entries per warp
#ifndef RSH_J_DRAIN
#define RSH_J_DRAIN 256
#endif
constexpr uint32_t J_DRAIN = RSH_J_DRAIN;  // queue length at which the packet walk stops to run the jobs
}

template <int P>
struct FusedSmem {
    float4 ro[8 * P];             // origin xyz, tmin
    float4 rs[8 * P];             // shear sx, sy, sz, tmax (original)
    float4 rd[8 * P];             // direction (for the per-ray cluster-sphere filter)
    uint16_t list[8 * P];         // rays of the current cluster that pass the sphere filter
    uint32_t meta[8 * P];         // kx | ky << 2 | kz << 4 | active << 6 | occluded << 7
    uint32_t slot[8 * P];
    float roc[8 * P];             // |o - packet centre|
    unsigned long long best[8 * P];
    float4 tri[F_MAXK * 3];
    uint32_t stack[F_STACK];
    uint32_t jobs[J_CAP];
    uint32_t qn;                  // jobs queued
};

RSH_DEV uint32_t find_segment(const FusedSeg* segs, uint32_t nseg, uint32_t u) {
    uint32_t lo = 0, hi = nseg;  // last s with unit_begin <= u
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&segs[mid].unit_begin) <= u) lo = mid; else hi = mid;
    }
    return lo;
}

// Per-ray jobs. A job is one ray and one object-tree node whose subtree the ray walks alone, nearest
// child first (job word: ray index | level << 8 | node index << 12). The warp keeps a queue of jobs in
// shared memory and runs it with all 32 lanes: a lane without a job takes the next one from the queue,
// and every iteration the busy lanes make ONE bounded step of one kind (the kind more of them want) --
// pop a node and test its (up to 8) children's boxes, pushing the hits farthest first, or pop a triangle
// cluster and test its box, then its triangles. Lanes never wait for another lane's whole ray. Every object-tree node
// carries a bounding sphere (the packet phase tests packet cones against it) and a padded box: a single
// ray descends by the boxes, which bound the thin triangles of tessellated surfaces far more tightly than
// spheres do (on the architecture scene: 6x fewer triangle tests, 1.7x faster).
//   closest hit: a hit updates the ray's shared best (atomicMin) at once, and every step re-reads it, so
//     jobs of the same ray running on other lanes cull with it too; triangle tests keep the ray's
//     original interval and the key comparison, so ties still resolve to the smaller triangle id;
//   any hit: an occluding hit sets the ray's occluded bit, which ends its other jobs at their next step.

RSH_DEV uint32_t job_word(uint32_t i, uint32_t L, uint32_t idx) { return i | (L << 8) | (idx << 12); }

// A job's stack entry. Triangle cluster c: c itself (level bits 0). Node of level L >= 1: L << 27 |
// (children - 1) << 24 | absolute node index of its first child -- the word its box carries in lo.w
// (written by the object-tree build), so a popped node's children are loaded straight away. Fits 32 bits:
// L <= 16, at most 8 children, fewer than 2^24 nodes (the batched form takes at most 2^20 nodes at
// level 1).
constexpr uint32_t E_LSHIFT = 27;
RSH_DEV uint32_t child_entry(float lo_w) { return __float_as_uint(lo_w); }
// The entry of a job's start node (L, idx); L == levels is the virtual root over the top level.
RSH_DEV uint32_t job_entry(const FusedSeg& sg, const float4* boxes, uint32_t L, uint32_t idx, uint32_t* err) {
    if (L == 0u) return idx;
    if (L == sg.levels) {
        uint32_t cnt = sg.lvl_size[L - 1u];
        if (cnt == 0u || cnt > 8u) {
            raise_device_error(err, RSH_DEVERR_OVERFLOW);
            cnt = cnt == 0u ? 1u : 8u;
        }
        return (L << 27) | ((cnt - 1u) << 24) | sg.lvl_off[L - 1u];
    }
    return child_entry(__ldg(&boxes[2ull * (sg.lvl_off[L] + idx)].w));
}

// Ray vs a padded node box over [tmin, tmax]: slab test, NaN-free for zero direction components (fminf /
// fmaxf drop a NaN operand); tn = entry distance (the nearest-first order key). The padding (1e-5 of the
// scene's largest coordinate) is far above the rounding of these products, so the cull is conservative.
RSH_DEV bool box_hit(float4 b0, float4 b1, float ox, float oy, float oz, float ix, float iy, float iz, float tmin,
                     float tmax, float& tn) {
    const float ax = (b0.x - ox) * ix, bx = (b1.x - ox) * ix;
    const float ay = (b0.y - oy) * iy, by = (b1.y - oy) * iy;
    const float az = (b0.z - oz) * iz, bz = (b1.z - oz) * iz;
    tn = fmaxf(fmaxf(tmin, fminf(ax, bx)), fmaxf(fminf(ay, by), fminf(az, bz)));
    const float tf = fminf(fminf(tmax, fmaxf(ax, bx)), fminf(fmaxf(ay, by), fmaxf(az, bz)));
    return tn <= tf;
}

template <int P, class SM>
RSH_DEV void run_jobs(SM& S, const FusedSeg& sg, bool any, uint32_t lane, unsigned long long& ntests,
                      unsigned long long& ttests, uint32_t* err) {
    const float4* __restrict__ boxes = sg.boxes;
    const float4* __restrict__ tris = sg.tris;
    const uint32_t qn = S.qn;
    uint32_t qh = 0;
    bool has = false;
    uint32_t i = 0;
    int sp = 0;
    uint32_t stk[J_STACK];
    float ox = 0.f, oy = 0.f, oz = 0.f, tmin = 0.f, tcur = 0.f;
    float ix = 0.f, iy = 0.f, iz = 0.f;  // 1 / direction (infinite for a zero component) for the box cull
    RayWT w;
    unsigned long long best = RSH_HIT_NONE;
    for (;;) {
        // lanes without a job take the next ones in queue order
        const uint32_t need = __ballot_sync(0xffffffffu, !has);
        if (need) {
            const uint32_t my = qh + __popc(need & lanemask_lt());
            qh += __popc(need);
            if (!has && my < qn) {
                const uint32_t job = S.jobs[my];
                i = job & 255u;
                const uint32_t mt = S.meta[i];
                if (!(any && (mt & 128u))) {
                    const float4 o = S.ro[i], d = S.rd[i], sh = S.rs[i];
                    ox = o.x;
                    oy = o.y;
                    oz = o.z;
                    tmin = o.w;
                    ix = __frcp_rn(d.x);
                    iy = __frcp_rn(d.y);
                    iz = __frcp_rn(d.z);
                    w.ox = o.x;
                    w.oy = o.y;
                    w.oz = o.z;
                    w.tmin = o.w;
                    w.sx = sh.x;
                    w.sy = sh.y;
                    w.sz = sh.z;
                    w.tmax = sh.w;
                    w.kx = mt & 3u;
                    w.ky = (mt >> 2) & 3u;
                    w.kz = (mt >> 4) & 3u;
                    tcur = sh.w;
                    best = RSH_HIT_NONE;
                    stk[0] = job_entry(sg, boxes, (job >> 8) & 15u, job >> 12, err);
                    sp = 1;
                    has = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, has)) {
            // every lane is idle: the queue is done only once it is exhausted (a job whose ray was occluded
            // after it was queued is skipped at fetch and takes no lane, so a whole round can come up empty)
            if (qh >= qn) break;
            continue;
        }
        // one kind of step per iteration, the kind more lanes want: node steps and cluster steps of one
        // warp would otherwise run one after the other, each with part of the lanes (+2% on the
        // architecture frame; with sphere descent it had cost 25%)
        bool do_nodes;
        {
            const bool want = has && sp > 0, node = want && (stk[sp - 1] >> E_LSHIFT) != 0u;
            const uint32_t nn = __popc(__ballot_sync(0xffffffffu, node));
            const uint32_t nc = __popc(__ballot_sync(0xffffffffu, want && !node));
            do_nodes = nn >= nc;
        }
        if (!has) continue;
        // what other jobs of this ray found so far
        if (any) {
            if (*(volatile uint32_t*)&S.meta[i] & 128u) sp = 0;
        } else {
            const unsigned long long b = *(volatile unsigned long long*)&S.best[i];
            if (b < best) {
                best = b;
                tcur = fminf(tcur, __uint_as_float((uint32_t)(b >> 32)));
            }
        }
        if (sp > 0 && ((stk[sp - 1] >> E_LSHIFT) != 0u) == do_nodes) {
            const uint32_t e = stk[--sp];
            const uint32_t L = e >> E_LSHIFT, idx = e & 0xFFFFFFu;
            if (L == 0u) {
                // the cluster's padded box against [tmin, current best]: slab test, NaN-free for zero
                // direction components (fminf/fmaxf drop a NaN operand); a miss skips the triangles
                const float4 b0 = __ldg(boxes + 2ull * idx), b1 = __ldg(boxes + 2ull * idx + 1);
                const uint32_t t0 = __float_as_uint(b0.w);  // the cluster's triangles: its box's link
                uint32_t t1 = t0 + __float_as_uint(b1.w);
                float tnb;
                if (!box_hit(b0, b1, ox, oy, oz, ix, iy, iz, tmin, tcur, tnb)) t1 = t0;
                for (uint32_t tt = t0; tt < t1; ++tt) {
                    const float4 v0 = __ldg(tris + 3ull * tt), v1 = __ldg(tris + 3ull * tt + 1),
                                 v2 = __ldg(tris + 3ull * tt + 2);
                    float th;
                    ++ttests;
                    if (wt_hit(w, v0, v1, v2, th)) {
                        if (any) {
                            atomicOr(&S.meta[i], 128u);
                            sp = 0;
                            break;
                        }
                        const unsigned long long key = hit_key(th, __float_as_uint(v0.w));
                        if (key < best) {
                            best = key;
                            tcur = fminf(tcur, th);
                            atomicMin(&S.best[i], key);
                        }
                    }
                }
            } else {
                const uint32_t cl = L - 1u;
                // the entry holds the children's link: up to 8 boxes from absolute node `idx` on
                const uint32_t cnt = ((e >> 24) & 7u) + 1u;
                const float4* bb = boxes + 2ull * idx;
                ntests += cnt;
                // children (at most 8, an invariant of the object tree): their boxes tested into registers,
                // hits pushed farthest first by selection, so the nearest pops first
                float tcs[8];
                uint32_t hm = 0;
#pragma unroll
                for (uint32_t c = 0; c < 8; ++c) {
                    tcs[c] = 0.0f;
                    if (c < cnt) {
                        float tc;
                        const float4 b0 = __ldg(bb + 2 * c), b1 = __ldg(bb + 2 * c + 1);
                        if (box_hit(b0, b1, ox, oy, oz, ix, iy, iz, tmin, tcur, tc)) {
                            hm |= 1u << c;
                            tcs[c] = tc;
                        }
                    }
                }
                if (sp + __popc(hm) > J_STACK) {
                    raise_device_error(err, RSH_DEVERR_OVERFLOW);
                    hm = 0;
                }
                while (hm) {
                    uint32_t bc = 0;
                    float bt = -INFINITY;
                    if (!any) {
#pragma unroll
                        for (uint32_t c = 0; c < 8; ++c)
                            if (((hm >> c) & 1u) && tcs[c] >= bt) {
                                bt = tcs[c];
                                bc = c;
                            }
                    } else {
                        bc = __ffs(hm) - 1u;
                    }
                    hm &= ~(1u << bc);
                    // a child node's own link, from the box just tested (an L1 hit)
                    stk[sp++] = cl == 0u ? idx + bc : child_entry(__ldg(&bb[2 * bc].w));
                }
            }
        }
        if (sp == 0) has = false;
    }
    __syncwarp();
    if (lane == 0) S.qn = 0;
    __syncwarp();
}

// After rays were tested: retire fully occluded packets (any hit) or shrink each packet's reach to
// max(|o - c| + best t) (closest hit). Lanes of group q hold packets 2q and 2q+1.
template <int P>
RSH_DEV void refresh_packets(FusedSmem<P>& S, bool any, uint32_t q, uint32_t ch, uint32_t& alive, NodeR& P0,
                             NodeR& P1) {
    if (any) {
        bool all0 = true, all1 = true;
        for (uint32_t jj = 0; jj < P; ++jj) {
            const uint32_t m0 = S.meta[(2u * q) * P + jj], m1 = S.meta[(2u * q + 1u) * P + jj];
            if ((m0 & 64u) && !(m0 & 128u)) all0 = false;
            if ((m1 & 64u) && !(m1 & 128u)) all1 = false;
        }
        const uint32_t d0 = __ballot_sync(0xffffffffu, all0 && ch == 0);
        const uint32_t d1 = __ballot_sync(0xffffffffu, all1 && ch == 0);
        uint32_t dead = 0;
#pragma unroll
        for (uint32_t g = 0; g < 4; ++g)
            dead |= (((d0 >> (8u * g)) & 1u) << (2u * g)) | (((d1 >> (8u * g)) & 1u) << (2u * g + 1u));
        alive &= ~dead;
    } else {
        float r0m = 0.f, r1m = 0.f;
        for (uint32_t jj = 0; jj < P; ++jj) {
            const uint32_t i0 = (2u * q) * P + jj, i1 = (2u * q + 1u) * P + jj;
            if (S.meta[i0] & 64u) {
                const unsigned long long b = S.best[i0];
                const float tb = (b == RSH_HIT_NONE) ? S.rs[i0].w : __uint_as_float((uint32_t)(b >> 32));
                r0m = fmaxf(r0m, S.roc[i0] + tb);
            }
            if (S.meta[i1] & 64u) {
                const unsigned long long b = S.best[i1];
                const float tb = (b == RSH_HIT_NONE) ? S.rs[i1].w : __uint_as_float((uint32_t)(b >> 32));
                r1m = fmaxf(r1m, S.roc[i1] + tb);
            }
        }
        P0.reach = fminf(P0.reach, r0m * (1.0f + 1.0f / 1048576.0f));
        P1.reach = fminf(P1.reach, r1m * (1.0f + 1.0f / 1048576.0f));
    }
}

#ifndef RSH_FUSED_MIN_BLOCKS
#define RSH_FUSED_MIN_BLOCKS 5
#endif
template <int P>
__global__ void __launch_bounds__(FW * 32, RSH_FUSED_MIN_BLOCKS) k_fused(FusedArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FusedSmem<P>& S = reinterpret_cast<FusedSmem<P>*>(smem_raw)[threadIdx.x >> 5];
    const uint32_t lane = lane_id();
    const uint32_t ch = lane & 7u, q = lane >> 3;
    const uint32_t units = dev_count(a.d_units, a.units_max);
    unsigned long long ntests = 0, ttests = 0;
    constexpr uint32_t R = 8 * P;
    if (lane == 0) S.qn = 0;
    __syncwarp();

    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(&a.work[0], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= units) break;
        const uint32_t sidx = find_segment(a.segs, a.nseg, u);
        const FusedSeg& sg = a.segs[sidx];
        const bool any = sg.any_hit != 0;
        // ---- rays of the unit -> shared memory
        const NodeR U = load_node(a.nodes, a.node_off[1] + u);
        for (uint32_t i = lane; i < R; i += 32) {
            const uint32_t k = u * R + i;
            const uint32_t id = __ldg(a.sorted_ids + k);
            uint32_t meta = 0;
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = make_float4(0.f, 0.f, 1.f, -1.f);
            if (id != INVALID_ID) load_ray(a.rays, id, o, d);
            const bool active = (id != INVALID_ID) && (d.w > o.w);
            const RayWT w = wt_setup(o, d);
            meta = (uint32_t)w.kx | ((uint32_t)w.ky << 2) | ((uint32_t)w.kz << 4) | (active ? 64u : 0u);
            S.ro[i] = make_float4(o.x, o.y, o.z, o.w);
            S.rs[i] = make_float4(w.sx, w.sy, w.sz, d.w);
            S.rd[i] = d;
            S.meta[i] = meta;
            S.slot[i] = id;
            S.best[i] = RSH_HIT_NONE;
            S.roc[i] = 0.f;
        }
        // ---- the lane's two packets (2q, 2q+1) in registers
        const uint32_t p0 = 8u * u + 2u * q, p1 = p0 + 1u;
        NodeR P0 = load_node(a.nodes, a.node_off[0] + p0);
        NodeR P1 = load_node(a.nodes, a.node_off[0] + p1);
        const bool v0 = P0.count > 0, v1 = P1.count > 0;
        __syncwarp();
        // |o - packet centre| per ray (for the shrinking reach of closest-hit packets)
        {
            // lane ch of group q computes for packet 2q (rays [2q*P, 2q*P+P)) and 2q+1, spread over 8 lanes
            for (uint32_t j = ch; j < 2u * P; j += 8u) {
                const uint32_t pk = 2u * q + (j / P);
                const uint32_t i = pk * P + (j % P);
                const NodeR& Pk = (j / P) ? P1 : P0;
                const float4 o = S.ro[i];
                const v3 dd = v3{o.x - Pk.cx, o.y - Pk.cy, o.z - Pk.cz};
                S.roc[i] = len3(dd);
            }
        }
        const uint32_t b0 = __ballot_sync(0xffffffffu, v0), b1 = __ballot_sync(0xffffffffu, v1);
        uint32_t mask = 0;
#pragma unroll
        for (uint32_t g = 0; g < 4; ++g)
            mask |= (((b0 >> (8u * g)) & 1u) << (2u * g)) | (((b1 >> (8u * g)) & 1u) << (2u * g + 1u));
        uint32_t alive = mask;
        const uint32_t f0 = __ballot_sync(0xffffffffu, v0 && !(P0.cs > 0.0f));
        const uint32_t f1 = __ballot_sync(0xffffffffu, v1 && !(P1.cs > 0.0f));
        uint32_t fullmask = 0;
#pragma unroll
        for (uint32_t g = 0; g < 4; ++g)
            fullmask |= (((f0 >> (8u * g)) & 1u) << (2u * g)) | (((f1 >> (8u * g)) & 1u) << (2u * g + 1u));
        __syncwarp();
        if (mask != 0 && sg.levels > 0u) {  // a scene without triangles has no tree: every ray misses
            int sp = 1;
            if (lane == 0) S.stack[0] = (sg.levels << 28) | mask;
            __syncwarp();
            while (sp > 0) {
                const uint32_t e = S.stack[sp - 1];
                __syncwarp();
                --sp;
                const uint32_t L = e >> 28, idx = (e >> 8) & 0xFFFFFu;
                uint32_t m = (e & 0xFFu) & alive;
                if (m == 0) continue;
                // rays of these packets leave the packet and descend this subtree one by one: below the
                // switch level, and at once for packets whose cone is wider than a half-space
                const uint32_t m_ray = (L <= sg.ray_level) ? m : (m & fullmask);
                if (m_ray) {
                    // queue one job per live ray of these packets; run the queue once it is long enough
                    // to keep every lane busy (or would overflow)
                    const uint32_t nr = __popc(m_ray) * P;
                    if (S.qn + nr > J_CAP) {
                        run_jobs<P>(S, sg, any, lane, ntests, ttests, a.err);
                        refresh_packets<P>(S, any, q, ch, alive, P0, P1);
                    }
                    uint32_t qn = S.qn;
                    __syncwarp();
                    for (uint32_t base = 0; base < nr; base += 32) {
                        const uint32_t ir = base + lane;
                        bool push = false;
                        uint32_t i = 0;
                        if (ir < nr) {
                            uint32_t pmm = m_ray;
                            for (uint32_t s2 = 0; s2 < ir / P; ++s2) pmm &= pmm - 1u;
                            i = (__ffs(pmm) - 1u) * P + (ir % P);
                            const uint32_t mt = S.meta[i];
                            push = (mt & 64u) && !(any && (mt & 128u)) && ((alive >> (i / P)) & 1u);
                        }
                        const uint32_t bl = __ballot_sync(0xffffffffu, push);
                        if (push) S.jobs[qn + __popc(bl & lanemask_lt())] = job_word(i, L, idx);
                        qn += __popc(bl);
                    }
                    __syncwarp();
                    if (lane == 0) S.qn = qn;
                    __syncwarp();
                    if (qn >= J_DRAIN) {
                        run_jobs<P>(S, sg, any, lane, ntests, ttests, a.err);
                        refresh_packets<P>(S, any, q, ch, alive, P0, P1);
                    }
                    m &= ~m_ray & alive;
                    if (alive == 0) break;
                    if (m == 0) continue;
                }
                const uint32_t cl = L - 1u;
                uint32_t first, cnt;
                node_children(sg.kids, sg.lvl_off, sg.lvl_size, sg.levels, L, idx, first, cnt);
                const bool has = ch < cnt;
                float4 Sph = make_float4(0.f, 0.f, 0.f, 0.f);
                if (has) Sph = __ldg(sg.spheres + sg.lvl_off[cl] + first + ch);
                const bool t0 = has && ((m >> (2u * q)) & 1u);
                const bool t1 = has && ((m >> (2u * q + 1u)) & 1u);
                const bool r0 = t0 && node_hits_sphere(P0, Sph);
                const bool r1 = t1 && node_hits_sphere(P1, Sph);
                ntests += (t0 ? 1u : 0u) + (t1 ? 1u : 0u);
                const uint32_t h0 = __ballot_sync(0xffffffffu, r0), h1 = __ballot_sync(0xffffffffu, r1);
                uint32_t cm = 0;
#pragma unroll
                for (uint32_t g = 0; g < 4; ++g)
                    cm |= (((h0 >> (ch + 8u * g)) & 1u) << (2u * g)) | (((h1 >> (ch + 8u * g)) & 1u) << (2u * g + 1u));
                if (lane >= 8u) cm = 0;
                // distance of each surviving child from the unit centre -> order
                const bool live = cm != 0u;
                const float dist = live ? len3(v3{Sph.x - U.cx, Sph.y - U.cy, Sph.z - U.cz}) - Sph.w : 0.f;
                const uint32_t lb = __ballot_sync(0xffffffffu, live);
                if (lb == 0) continue;
                uint32_t farther = 0;  // children farther than this one (ties: larger index counts as farther)
#pragma unroll
                for (uint32_t o2 = 0; o2 < 8; ++o2) {
                    const float od = __shfl_sync(0xffffffffu, dist, o2);
                    if (live && ((lb >> o2) & 1u) && o2 != lane && (od > dist || (od == dist && o2 > lane))) ++farther;
                }
                const uint32_t nlive = __popc(lb);
                if (cl == 0) {
                    // visit clusters nearest first: rank r = nlive-1-farther
                    for (uint32_t rk = 0; rk < nlive; ++rk) {
                        const uint32_t sel = __ballot_sync(0xffffffffu, live && (nlive - 1u - farther) == rk);
                        const uint32_t c = __ffs(sel) - 1u;
                        const uint32_t pm = __shfl_sync(0xffffffffu, cm, c) & alive;
                        if (pm == 0) continue;
                        const uint32_t cluster = first + c;
                        uint32_t t0i, t1i;
                        cluster_tris(sg.kids, cluster, t0i, t1i);
                        const uint32_t K = t1i - t0i;
                        for (uint32_t j = lane; j < 3u * K; j += 32) S.tri[j] = __ldg(sg.tris + 3ull * t0i + j);
                        __syncwarp();
                        // per-ray filter against the cluster sphere, compacted into S.list
                        const float4 csph = make_float4(__shfl_sync(0xffffffffu, Sph.x, c), __shfl_sync(0xffffffffu, Sph.y, c),
                                                        __shfl_sync(0xffffffffu, Sph.z, c), __shfl_sync(0xffffffffu, Sph.w, c));
                        const uint32_t nr = __popc(pm) * P;
                        uint32_t nlist = 0;
                        for (uint32_t base = 0; base < nr; base += 32) {
                            const uint32_t ir = base + lane;
                            bool pass = false;
                            uint32_t i = 0;
                            if (ir < nr) {
                                uint32_t pmm = pm;
                                for (uint32_t s2 = 0; s2 < ir / P; ++s2) pmm &= pmm - 1u;
                                i = (__ffs(pmm) - 1u) * P + (ir % P);
                                const uint32_t mt = S.meta[i];
                                if ((mt & 64u) && !(any && (mt & 128u))) {
                                    const float4 o = S.ro[i], dd = S.rd[i];
                                    pass = ray_hits_sphere(o.x, o.y, o.z, dd.x, dd.y, dd.z, o.w, dd.w, csph);
                                }
                            }
                            const uint32_t bl = __ballot_sync(0xffffffffu, pass);
                            if (pass) S.list[nlist + __popc(bl & lanemask_lt())] = (uint16_t)i;
                            nlist += __popc(bl);
                        }
                        __syncwarp();
                        const uint32_t pairs = nlist * K;
                        for (uint32_t qq = lane; qq < pairs; qq += 32) {
                            const uint32_t ir = qq / K, j = qq - ir * K;
                            const uint32_t i = S.list[ir];
                            const uint32_t meta = S.meta[i];
                            if (any && (*(volatile uint32_t*)&S.meta[i] & 128u)) continue;
                            RayWT w;
                            const float4 o = S.ro[i], sh = S.rs[i];
                            w.ox = o.x;
                            w.oy = o.y;
                            w.oz = o.z;
                            w.tmin = o.w;
                            w.sx = sh.x;
                            w.sy = sh.y;
                            w.sz = sh.z;
                            w.tmax = sh.w;
                            w.kx = meta & 3u;
                            w.ky = (meta >> 2) & 3u;
                            w.kz = (meta >> 4) & 3u;
                            float th;
                            ++ttests;
                            if (wt_hit(w, S.tri[3 * j], S.tri[3 * j + 1], S.tri[3 * j + 2], th)) {
                                if (any) atomicOr(&S.meta[i], 128u);
                                else atomicMin(&S.best[i], hit_key(th, __float_as_uint(S.tri[3 * j].w)));
                            }
                        }
                        __syncwarp();
                        // refresh the packets' state: occlusion (any) or shrunken reach (closest)
                        refresh_packets<P>(S, any, q, ch, alive, P0, P1);
                        if (alive == 0) break;
                    }
                } else {
                    if (sp + nlive > F_STACK) {
                        raise_device_error(a.err, RSH_DEVERR_OVERFLOW);
                        break;
                    }
                    if (live) S.stack[sp + farther] = (cl << 28) | ((first + ch) << 8) | cm;
                    sp += nlive;
                    __syncwarp();
                }
                if (alive == 0) break;
            }
            if (S.qn) run_jobs<P>(S, sg, any, lane, ntests, ttests, a.err);
        }
        __syncwarp();
        // ---- results (each ray belongs to exactly one unit)
        for (uint32_t i = lane; i < R; i += 32) {
            const uint32_t meta = S.meta[i];
            if (!(meta & 64u)) continue;
            const uint32_t slot = S.slot[i] - sg.slot_base;
            if (any) sg.flags[slot] = (meta & 128u) ? RSH_OCCLUDED : 0u;
            else sg.hits[slot] = S.best[i];
        }
        __syncwarp();
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        ntests += __shfl_xor_sync(0xffffffffu, ntests, d);
        ttests += __shfl_xor_sync(0xffffffffu, ttests, d);
    }
    if (lane == 0) {
        if (a.node_tests) atomicAdd(a.node_tests, ntests);
        if (a.tri_tests) atomicAdd(a.tri_tests, ttests);
    }
}

// Rays-only form: every segment's switch level is at or above its tree's depth, so every ray is one job
// from the root, traced by one lane (until, in the SHARE instance, the launch's end). The rays descend the scene's single-ray box tree (wide.cu: an
// 8-wide tree of mixed depth built by PLOC clustering, tighter than the object-sphere hierarchy's level
// structure) in its traversal-record form: a stack entry is a node's REC_NODE | (children - 1) << 28 |
// record index, or a cluster's first triangle | (triangles - 1) << 23. A node step reads the
// record's near planes and far planes for the ray's octant (12 float4 loads, no per-axis min / max) and
// the entries of the children it pushes. The warp keeps no per-unit state: it takes work units
// (RSH_RAYS_UNIT sorted rays, never straddling a segment) by atomic ticket, and every lane whose ray has
// finished takes the next ray of the warp's current unit straight from global memory (its id from the
// sorted order, the ray itself from the segment's array), fetching the next unit when the current one runs
// out. So lanes are refilled continuously and no lane waits for the slowest ray of a unit; a lane writes its
// ray's result (shadow flag or hit record) itself when the ray ends. The launch's last units go out as
// pieces of RSH_RAYS_UNIT / RSH_TAIL_SPLIT rays. Single long rays (up to 20x the median ray's tests) still
// hold an SM after the others have finished; the SHARE instance (the default) lets a drained warp's idle
// lanes take their subtrees (described at its loop's top), at the price of about 4% on every step, which
// the instance without it (RSH_FLAG_SEQUENTIAL_RAYS) does not pay.
//
// Box test (box_hit_fma): t = b * (1 / d) - o * (1 / d) as one fused multiply-add per plane, with direction
// components below 1e-20 in magnitude replaced by +-1e-20 (finite reciprocals, no inf - inf), and the
// entry / exit distances reduced with three-input min / max. The change of rounding against (b - o) / d is
// about one ulp of the coordinates, far below the boxes' padding (1e-5 of the scene's largest coordinate),
// so the cull stays conservative; the triangle tests alone decide every hit.
RSH_DEV float fmax3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
RSH_DEV float fmin3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
RSH_DEV float safe_rcp(float d) {
    const float m = 1e-20f;
    return __frcp_rn(fabsf(d) < m ? copysignf(m, d) : d);
}
RSH_DEV bool box_hit_fma(float4 b0, float4 b1, float ix, float iy, float iz, float oix, float oiy, float oiz,
                         float tmin, float tmax, float& tn) {
    const float ax = __fmaf_rn(b0.x, ix, -oix), bx = __fmaf_rn(b1.x, ix, -oix);
    const float ay = __fmaf_rn(b0.y, iy, -oiy), by = __fmaf_rn(b1.y, iy, -oiy);
    const float az = __fmaf_rn(b0.z, iz, -oiz), bz = __fmaf_rn(b1.z, iz, -oiz);
    tn = fmaxf(fmax3f(tmin, fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
    const float tf = fminf(fmin3f(tmax, fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
    return tn <= tf;
}

// Two plane distances at once: the packed FP32 fused multiply-add (fma.rn.f32x2, sm_100 and later), each
// half rounded exactly like a scalar fma.rn.
RSH_DEV void fma2(float a0, float a1, float b, float c, float& r0, float& r1) {
    unsigned long long ra, rb, rc, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a0), "f"(a1));
    asm("mov.b64 %0, {%1, %1};" : "=l"(rb) : "f"(b));
    asm("mov.b64 %0, {%1, %1};" : "=l"(rc) : "f"(c));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r0), "=f"(r1) : "l"(rd));
}

// Entry (near) or exit (far) distances of four children of a traversal record from one plane of each axis:
// near: max(tmin, tx, ty, tz); far: min(tmax, tx, ty, tz), each t = plane * (1 / d) - o * (1 / d). With the
// plane chosen by the direction's sign (the lower plane is the near one for a positive component), tx equals
// the min (near) or the max (far) of the two planes' distances that box_hit_fma takes, so both tests decide
// every box alike.
RSH_DEV void slab4(float4 px, float4 py, float4 pz, float ix, float iy, float iz, float oix, float oiy, float oiz,
                   float lim, float* t, bool near) {
    float tx[4], ty[4], tz[4];
    fma2(px.x, px.y, ix, -oix, tx[0], tx[1]);
    fma2(px.z, px.w, ix, -oix, tx[2], tx[3]);
    fma2(py.x, py.y, iy, -oiy, ty[0], ty[1]);
    fma2(py.z, py.w, iy, -oiy, ty[2], ty[3]);
    fma2(pz.x, pz.y, iz, -oiz, tz[0], tz[1]);
    fma2(pz.z, pz.w, iz, -oiz, tz[2], tz[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        t[k] = near ? fmaxf(fmax3f(lim, tx[k], ty[k]), tz[k]) : fminf(fmin3f(lim, tx[k], ty[k]), tz[k]);
}

#ifndef RSH_RAYS_MIN_BLOCKS
#define RSH_RAYS_MIN_BLOCKS 7
#endif
#ifndef RSH_SHARE_BUSY
#define RSH_SHARE_BUSY 16  // busy lanes at or below which a drained warp shares its rays (SHARE)
#endif
#ifndef RSH_TAIL_PER_WARP
#define RSH_TAIL_PER_WARP 16
#endif
#ifndef RSH_TAIL_SPLIT
#define RSH_TAIL_SPLIT 2
#endif

template <int U, bool SHARE>
__global__ void __launch_bounds__(FW * 32, RSH_RAYS_MIN_BLOCKS) k_fused_rays(FusedArgs a) {
    // SHARE: a drained warp's rays shared among its idle lanes; the records of the rays being shared, one per
    // lane: the owner's best hit key (closest hit), occluded (any hit), helpers still on a subtree of it
    __shared__ unsigned long long sh_best[SHARE ? FW : 1][32];
    __shared__ uint32_t sh_occ[SHARE ? FW : 1][32], sh_pend[SHARE ? FW : 1][32];
    const uint32_t lane = lane_id();
    const uint32_t units = dev_count(a.d_units, a.units_max);
    const uint32_t tail = min(units, (uint32_t)RSH_TAIL_PER_WARP * gridDim.x * FW);
    const uint32_t head = units - tail, tickets = head + RSH_TAIL_SPLIT * tail;
    uint32_t ntests = 0, ttests = 0;  // the lane's counts, flushed to the launch's counters before 2^31
    // the warp's current unit: sorted rays [nk, nend) of segment cs
    uint32_t nk = 0, nend = 0, cs = 0;
    bool drained = false;
    // the lane's ray
    bool has = false, any = false;
    uint32_t seg = 0, slot = 0;
    const float4* __restrict__ nodes = nullptr;
    const float4* __restrict__ tris = nullptr;
    int sp = 0;
    uint32_t stk[J_STACK];
    float stt[J_STACK];  // closest hit: each entry's entry distance, from its parent's test
    float ox = 0.f, oy = 0.f, oz = 0.f, tmin = 0.f, tcur = 0.f;
    float ix = 0.f, iy = 0.f, iz = 0.f, oix = 0.f, oiy = 0.f, oiz = 0.f;
    uint32_t oct = 0;  // the direction's octant: bit a set when component a is negative
    RayWT w;
    unsigned long long best = RSH_HIT_NONE;
    bool sharing = false;  // warp-uniform (SHARE): the warp shares its last rays
    bool done = false;     // sharing: the lane's subtree is done, its result not yet merged
    uint32_t own = lane;   // sharing: the lane whose ray this lane works on
    // the ray is done: its result, written by its own lane (while sharing: merged at the loop's top)
    auto finish = [&]() {
        if (SHARE && sharing) {
            done = true;
            has = false;
            return;
        }
        const FusedSeg& sg = a.segs[seg];
        if (any) sg.flags[slot] = best == 0ull ? RSH_OCCLUDED : 0u;
        else sg.hits[slot] = best;
        has = false;
        // one ray adds fewer than 2^28 node tests (8 per slot) and 2^24 triangle tests
        if ((ntests | ttests) >> 31) {
            if (a.node_tests) atomicAdd(a.node_tests, (unsigned long long)ntests);
            if (a.tri_tests) atomicAdd(a.tri_tests, (unsigned long long)ttests);
            ntests = ttests = 0;
        }
    };
    for (;;) {
        // idle lanes take the next rays of the warp's unit, units are fetched as they run out
        for (;;) {
            const uint32_t need = __ballot_sync(0xffffffffu, !has);
            if (!need) break;
            if (nk >= nend) {
                if (drained) break;
                uint32_t t = 0;
                if (lane == 0) t = atomicAdd(&a.work[0], 1u);
                t = __shfl_sync(0xffffffffu, t, 0);
                if (t >= tickets) {
                    drained = true;
                    break;
                }
                uint32_t u = t, lo = 0, hi = U;
                if (t >= head) {
                    const uint32_t h = t - head;
                    u = head + h / RSH_TAIL_SPLIT;
                    lo = (h % RSH_TAIL_SPLIT) * (U / RSH_TAIL_SPLIT);
                    hi = lo + U / RSH_TAIL_SPLIT;
                }
                nk = u * U + lo;
                nend = u * U + hi;
                cs = find_segment(a.segs, a.nseg, u);
            }
            const uint32_t k = nk + __popc(need & lanemask_lt());
            if (!has && k < nend) {
                // no sorted order: the rays' own order, padded past ordered_n
                const uint32_t id = a.sorted_ids ? __ldg(a.sorted_ids + k) : (k < a.ordered_n ? k : INVALID_ID);
                if (id != INVALID_ID) {
                    const FusedSeg& sg = a.segs[cs];
                    float4 o, d;
                    load_ray(sg.rays, id - sg.slot_base, o, d);
                    if (d.w > o.w) {
                        if (sg.levels == 0u) {
                            // a scene without triangles has no tree: the ray misses
                            if (sg.any_hit) sg.flags[id - sg.slot_base] = 0u;
                            else sg.hits[id - sg.slot_base] = RSH_HIT_NONE;
                        } else {
                            seg = cs;
                            slot = id - sg.slot_base;
                            any = sg.any_hit != 0u;
                            nodes = sg.wnodes;
                            tris = sg.wtris;
                            ox = o.x;
                            oy = o.y;
                            oz = o.z;
                            tmin = o.w;
                            tcur = d.w;
                            ix = safe_rcp(d.x);
                            iy = safe_rcp(d.y);
                            iz = safe_rcp(d.z);
                            oix = ox * ix;
                            oiy = oy * iy;
                            oiz = oz * iz;
                            w = wt_setup(o, d);
                            best = RSH_HIT_NONE;
                            oct = (ix < 0.f ? 1u : 0u) | (iy < 0.f ? 2u : 0u) | (iz < 0.f ? 4u : 0u);
                            stk[0] = sg.wnroot;
                            stt[0] = -INFINITY;
                            sp = 1;
                            has = true;
                        }
                    }
                }
            }
            nk = min(nend, nk + __popc(need));
        }
        if (!__any_sync(0xffffffffu, has || (SHARE && done))) break;  // nothing in flight, nothing to fetch
        // SHARE: once no ray is left to take and at most RSH_SHARE_BUSY lanes still trace one, idle lanes take
        // stack entries (subtrees) of the warp's rays in flight, so that a long ray near the launch's end
        // runs on many lanes instead of one. A ray's lane (its owner) keeps its result; a helper merges its
        // own into the owner's record when its subtree is done (atomicMin of the hit key, or the occluded
        // flag), and the owner writes the result once its stack is empty and no helper is left. Everything
        // happens here, between steps: the steps themselves are the sequential ones.
        if (SHARE && drained && (sharing || __popc(__ballot_sync(0xffffffffu, has)) <= RSH_SHARE_BUSY)) {
            const uint32_t wp = threadIdx.x >> 5;
            if (!sharing) {
                sh_best[wp][lane] = has ? best : RSH_HIT_NONE;
                sh_occ[wp][lane] = 0u;
                sh_pend[wp][lane] = 0u;
                own = lane;
                sharing = true;
            }
            __syncwarp();
            if (has) {
                if (any) {
                    if (sh_occ[wp][own]) {
                        sp = 0;
                        done = true;
                        has = false;
                    }
                } else {
                    tcur = fminf(tcur, __uint_as_float((uint32_t)(sh_best[wp][own] >> 32)));
                }
            }
            if (done && own == lane && sh_pend[wp][lane] == 0u) {
                // the owner, with no helper left: the ray's merged result
                if (any) best = (best == 0ull || sh_occ[wp][lane]) ? 0ull : best;
                else best = min(best, sh_best[wp][lane]);
                const FusedSeg& sg = a.segs[seg];
                if (any) sg.flags[slot] = best == 0ull ? RSH_OCCLUDED : 0u;
                else sg.hits[slot] = best;
                done = false;
            } else if (done && own != lane) {
                // a helper's subtree is done: its result into the owner's record
                if (any) {
                    if (best == 0ull) sh_occ[wp][own] = 1u;
                } else {
                    atomicMin(&sh_best[wp][own], best);
                }
                atomicSub(&sh_pend[wp][own], 1u);
                done = false;
            }
            __syncwarp();
            const uint32_t idle = __ballot_sync(0xffffffffu, !has && !done);
            const uint32_t donors = __ballot_sync(0xffffffffu, has && sp >= 2);
            if (idle && donors) {
                const uint32_t r = __popc(idle & lanemask_lt());
                const bool recv = !has && !done && r < (uint32_t)__popc(donors);
                const uint32_t src = recv ? __fns(donors, 0u, (int)r + 1) : lane;
                const bool give = has && sp >= 2 && (uint32_t)__popc(donors & lanemask_lt()) < (uint32_t)__popc(idle);
                uint32_t ge = 0u;
                float gt = 0.0f;
                if (give) {
                    --sp;
                    ge = stk[sp];
                    gt = stt[sp];
                }
                ge = __shfl_sync(0xffffffffu, ge, src);
                gt = __shfl_sync(0xffffffffu, gt, src);
                const uint32_t go = __shfl_sync(0xffffffffu, own, src);
                any = __shfl_sync(0xffffffffu, any, src);
                seg = __shfl_sync(0xffffffffu, seg, src);
                slot = __shfl_sync(0xffffffffu, slot, src);
                nodes = reinterpret_cast<const float4*>(
                    __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(nodes), src));
                tris = reinterpret_cast<const float4*>(
                    __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(tris), src));
                tmin = __shfl_sync(0xffffffffu, tmin, src);
                tcur = __shfl_sync(0xffffffffu, tcur, src);
                ix = __shfl_sync(0xffffffffu, ix, src);
                iy = __shfl_sync(0xffffffffu, iy, src);
                iz = __shfl_sync(0xffffffffu, iz, src);
                oix = __shfl_sync(0xffffffffu, oix, src);
                oiy = __shfl_sync(0xffffffffu, oiy, src);
                oiz = __shfl_sync(0xffffffffu, oiz, src);
                oct = __shfl_sync(0xffffffffu, oct, src);
                w.ox = __shfl_sync(0xffffffffu, w.ox, src);
                w.oy = __shfl_sync(0xffffffffu, w.oy, src);
                w.oz = __shfl_sync(0xffffffffu, w.oz, src);
                w.sx = __shfl_sync(0xffffffffu, w.sx, src);
                w.sy = __shfl_sync(0xffffffffu, w.sy, src);
                w.sz = __shfl_sync(0xffffffffu, w.sz, src);
                w.kx = __shfl_sync(0xffffffffu, w.kx, src);
                w.ky = __shfl_sync(0xffffffffu, w.ky, src);
                w.kz = __shfl_sync(0xffffffffu, w.kz, src);
                w.tmin = __shfl_sync(0xffffffffu, w.tmin, src);
                w.tmax = __shfl_sync(0xffffffffu, w.tmax, src);
                if (recv) {
                    own = go;
                    stk[0] = ge;
                    stt[0] = gt;
                    sp = 1;
                    best = RSH_HIT_NONE;
                    has = true;
                    atomicAdd(&sh_pend[wp][own], 1u);
                }
            }
            __syncwarp();
        }
        // closest hit: entries that the ray enters beyond its current best are dropped unread (their
        // subtrees cannot hold a nearer hit: a child's box lies inside its parent's, so no child is entered
        // before its parent)
        if (has && !any) {
            while (sp > 0 && stt[sp - 1] > tcur) --sp;
            if (sp == 0) finish();
        }
        // one kind of step per iteration, the kind more lanes want
        bool do_nodes;
        {
            const bool node = has && (stk[sp - 1] >> 31) != 0u;
            const uint32_t nn = __popc(__ballot_sync(0xffffffffu, node));
            const uint32_t nc = __popc(__ballot_sync(0xffffffffu, has && !node));
            do_nodes = nn >= nc;
        }
        if (has && ((stk[sp - 1] >> 31) != 0u) == do_nodes) {
            const uint32_t e = stk[--sp];
            if (!(e >> 31)) {
                // a cluster: its triangles t0 .. t0 + count - 1 (its box was tested with the parent's
                // children; a closest-hit ray re-checks only its entry distance, above)
                const uint32_t t0 = e & 0x7FFFFFu, t1 = t0 + ((e >> 23) & 63u) + 1u;
                for (uint32_t tt = t0; tt < t1; ++tt) {
                    const float4 v0 = __ldg(tris + 3ull * tt), v1 = __ldg(tris + 3ull * tt + 1),
                                 v2 = __ldg(tris + 3ull * tt + 2);
                    float th;
                    ++ttests;
                    if (wt_hit(w, v0, v1, v2, th)) {
                        if (any) {
                            best = 0ull;  // occluded
                            sp = 0;
                            break;
                        }
                        const unsigned long long key = hit_key(th, __float_as_uint(v0.w));
                        if (key < best) {
                            best = key;
                            tcur = fminf(tcur, th);
                        }
                    }
                }
            } else {
                // a node record: the children's near planes and far planes, axis by axis, then their entries
                const uint32_t cnt = ((e >> 28) & 7u) + 1u;
                const float4* rec = nodes + REC_F4 * (size_t)(e & 0x0FFFFFFFu);
                ntests += cnt;
                if (sp + cnt > J_STACK) {
                    raise_device_error(a.err, RSH_DEVERR_OVERFLOW);
                } else {
                    const uint32_t nxo = (oct & 1u) << 1, nyo = 4u | (oct & 2u), nzo = 8u | ((oct >> 1) & 2u);
                    float tn[8];
                    uint32_t hm = 0;
#pragma unroll
                    for (uint32_t h = 0; h < 2; ++h) {
                        float n4[4], f4[4];
                        slab4(__ldg(rec + nxo + h), __ldg(rec + nyo + h), __ldg(rec + nzo + h), ix, iy, iz, oix,
                              oiy, oiz, tmin, n4, true);
                        slab4(__ldg(rec + (nxo ^ 2u) + h), __ldg(rec + (nyo ^ 2u) + h), __ldg(rec + (nzo ^ 2u) + h),
                              ix, iy, iz, oix, oiy, oiz, tcur, f4, false);
#pragma unroll
                        for (uint32_t k = 0; k < 4; ++k) {
                            tn[4 * h + k] = n4[k];
                            hm |= (n4[k] <= f4[k] ? 1u : 0u) << (4 * h + k);
                        }
                    }
                    const uint32_t* ent = reinterpret_cast<const uint32_t*>(rec + 12);
                    if (any) {
                        // any hit: every child whose box the ray crosses is pushed in child order (the last
                        // pops first)
#pragma unroll
                        for (uint32_t h = 0; h < 2; ++h) {
                            if ((hm >> (4 * h)) & 15u) {
                                const uint4 ee = __ldg(reinterpret_cast<const uint4*>(ent) + h);
                                const uint32_t ce[4] = {ee.x, ee.y, ee.z, ee.w};
#pragma unroll
                                for (uint32_t k = 0; k < 4; ++k)
                                    if ((hm >> (4 * h + k)) & 1u) stk[sp++] = ce[k];
                            }
                        }
                    } else {
                        // closest hit: the hits pushed farthest first, so that the nearest pops first (among
                        // equal entry distances the lower child)
                        while (hm) {
                            uint32_t bc = 0;
                            float bt = -INFINITY;
#pragma unroll
                            for (uint32_t c = 0; c < 8; ++c)
                                if (((hm >> c) & 1u) && tn[c] >= bt) {
                                    bt = tn[c];
                                    bc = c;
                                }
                            hm &= ~(1u << bc);
                            stk[sp] = __ldg(ent + bc);  // an L1 hit: the record was just read
                            stt[sp++] = bt;
                        }
                    }
                }
            }
            if (sp == 0) finish();
        }
    }
    unsigned long long nt = ntests, tt = ttests;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        nt += __shfl_xor_sync(0xffffffffu, nt, d);
        tt += __shfl_xor_sync(0xffffffffu, tt, d);
    }
    if (lane == 0) {
        if (a.node_tests) atomicAdd(a.node_tests, nt);
        if (a.tri_tests) atomicAdd(a.tri_tests, tt);
    }
}

template <int U, bool SHARE>
static cudaError_t launch_fused_rays_s(const FusedArgs& a, cudaStream_t s) {
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_rays<U, SHARE>, FW * 32, 0);
    if (per_sm < 1) per_sm = 1;
    if (a.blocks_per_sm && (int)a.blocks_per_sm < per_sm) per_sm = (int)a.blocks_per_sm;
    uint32_t grid = (uint32_t)(sms * per_sm);
    const uint32_t need = (a.units_max + FW - 1) / FW;
    if (need < grid) grid = need > 0 ? need : 1;
    k_fused_rays<U, SHARE><<<grid, FW * 32, 0, s>>>(a);
    note_launch();
    return cudaGetLastError();
}
template <int U>
static cudaError_t launch_fused_rays_u(const FusedArgs& a, cudaStream_t s) {
    return a.share_tail ? launch_fused_rays_s<U, true>(a, s) : launch_fused_rays_s<U, false>(a, s);
}

template <int P>
static cudaError_t launch_fused_p(const FusedArgs& a, cudaStream_t s) {
    if (a.rays_only) return launch_fused_rays_u<RSH_RAYS_UNIT>(a, s);  // units of RSH_RAYS_UNIT rays
    const size_t smem = sizeof(FusedSmem<P>) * FW;
    cudaError_t e = cudaFuncSetAttribute(k_fused<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused<P>, FW * 32, smem);
    if (per_sm < 1) per_sm = 1;
    if (a.blocks_per_sm && (int)a.blocks_per_sm < per_sm) per_sm = (int)a.blocks_per_sm;
    uint32_t grid = (uint32_t)(sms * per_sm);
    const uint32_t need = (a.units_max + FW - 1) / FW;
    if (need < grid) grid = need > 0 ? need : 1;
    k_fused<P><<<grid, FW * 32, smem, s>>>(a);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_fused(const FusedArgs& a, cudaStream_t s) {
    switch (a.packet) {
        case 8: return launch_fused_p<8>(a, s);
        case 16: return launch_fused_p<16>(a, s);
        case 32: return launch_fused_p<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace rsh
