// Batched form: many ray batches of uneven size over several resident scenes in one pass.
//
// The reference has no batched path: every batch is a host loop of wrappers with a blocking count
// readback after each stage (main.cpp:951-1054, RayTracer.cu:2316-2832). Here, for S segments:
//   k_batch_prep     one pass over all rays: key = segment << shift | hash (per-segment scene box),
//                    pre-fill each segment's output, count each segment's rays (shared-memory counters,
//                    one global atomic per segment per block); it gathers the rays into one array only for
//                    the packet kernel when the segments do not already lie back to back;
//   k_batch_bounds   from those counts (one block): each segment's range of the sorted order (the
//                    segment tag is the top key digit, so the sorted order is segment-major: a segmented
//                    sort for free) and of the padded layout, padded so that no level-1 ray node straddles
//                    two segments, laid out in schedule order -- closest-hit segments before any-hit
//                    ones, larger before smaller, so the work units handed out last (the launch's tail)
//                    are the cheap ones; the padding slots are marked empty;
//   compress / sort / decompress over all keys at once; decompress writes each ray straight to its
//                    padded position (RSH_FLAG_NO_COMPRESS: the slots are sorted as they are and
//                    k_batch_scatter writes them to the padded layout);
//   build            ray-space hierarchy over the padded order (packet kernel only);
//   fused            ONE persistent traversal + intersection launch over every segment's work units
//                    (the rays-only kernel reads each segment's rays in place).
// Nothing reads a count back to the host, so the whole sequence is captured in a CUDA graph.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "engine.h"
#include "hash.cuh"

namespace rsh {

namespace {
constexpr uint32_t INVALID_ID = 0xFFFFFFFFu;

struct PrepSeg {  // per-segment table of k_batch_prep
    const rsh_ray* rays;
    uint32_t start;
    uint32_t any_hit;
    uint32_t* flags;
    unsigned long long* hits;
    HashP hp;
};
}  // namespace

__global__ void k_batch_prep(const PrepSeg* __restrict__ segs, uint32_t nseg, uint32_t total, uint32_t tag_shift,
                             uint32_t hash_drop,
                             rsh_ray* __restrict__ rays_all, bool gather, uint32_t* __restrict__ keys,
                             uint32_t* __restrict__ seg_cnt) {
    __shared__ uint32_t s_cnt[1024];  // the block's rays per segment (nseg <= 1024)
    for (uint32_t j = threadIdx.x; j < nseg; j += blockDim.x) s_cnt[j] = 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = false;
    uint32_t lo = 0;
    if (i < total) {
        uint32_t hi = nseg;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(&segs[mid].start) <= i) lo = mid; else hi = mid;
        }
        const PrepSeg& sg = segs[lo];
        const uint32_t j = i - sg.start;
        float4 o, d;
        load_ray(sg.rays, j, o, d);
        if (gather) store_ray(rays_all, i, o, d);  // else the segments already lie back to back there
        uint32_t key = RSH_KEY_NONE;
        valid = d.w > o.w;
        if (valid) key = (lo << tag_shift) | (ray_hash(o.x, o.y, o.z, d.x, d.y, d.z, sg.hp, 0u) >> hash_drop);
        keys[i] = key;
        if (sg.any_hit) sg.flags[j] = 0u;
        else sg.hits[j] = RSH_HIT_NONE;
    }
    // rays per segment: one shared atomic per segment present in the warp, then one global atomic per
    // segment present in the block (a frame's two segments would otherwise see one per warp)
    const uint32_t peers = __match_any_sync(0xffffffffu, valid ? lo : 0xFFFFFFFFu);
    if (valid && (peers & lanemask_lt()) == 0u) atomicAdd(s_cnt + lo, (uint32_t)__popc(peers));
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < nseg; j += blockDim.x)
        if (s_cnt[j]) atomicAdd(seg_cnt + j, s_cnt[j]);
}

// Per-segment ranges in the sorted (segment-major) order and the padded layout, from the per-segment ray
// counts; one block. seg_delta[s] = padded position - sorted position for segment s's rays.
__global__ void k_batch_bounds(const uint32_t* __restrict__ seg_cnt, uint32_t nseg, uint32_t unit_rays,
                               uint32_t* __restrict__ seg_begin, uint32_t* __restrict__ pstart,
                               uint32_t* __restrict__ seg_delta, const uint32_t* __restrict__ sched,
                               FusedSeg* __restrict__ fsegs, uint32_t* __restrict__ totals,
                               uint32_t* __restrict__ padded, uint32_t max_padded) {
    __shared__ uint32_t s_pad_end[1025], s_pad_begin[1025];
    if (threadIdx.x == 0) {
        uint32_t acc = 0;  // sorted order: segment index order
        for (uint32_t s = 0; s < nseg; ++s) {
            seg_begin[s] = acc;
            acc += seg_cnt[s];
        }
        acc = 0;  // padded layout in schedule order: position k holds segment sched[k]
        for (uint32_t k = 0; k < nseg; ++k) {
            const uint32_t s = sched[k];
            pstart[k] = acc;
            fsegs[k].unit_begin = acc / unit_rays;
            seg_delta[s] = acc - seg_begin[s];
            s_pad_begin[k] = acc + seg_cnt[s];
            acc += ((seg_cnt[s] + unit_rays - 1) / unit_rays) * unit_rays;
            s_pad_end[k] = acc;
        }
        pstart[nseg] = acc;
        totals[0] = acc;              // padded ray count
        totals[1] = acc / unit_rays;  // work units
    }
    __syncthreads();
    // empty slots at the end of each segment's last work unit
    for (uint32_t k = 0; k < nseg; ++k)
        for (uint32_t q = s_pad_begin[k] + threadIdx.x; q < s_pad_end[k] && q < max_padded; q += blockDim.x)
            padded[q] = INVALID_ID;
}

// Without run compression: the sorted slots go straight to the padded layout (valid keys sort before
// every empty slot, whose key has the bit above the key's width set); also the stats words (rays,
// "chunks" = rays) from the per-segment counts.
__global__ void k_batch_scatter(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ svals,
                                uint32_t total, uint32_t tag_shift, const uint32_t* __restrict__ seg_delta,
                                uint32_t* __restrict__ padded, uint32_t max_padded,
                                const uint32_t* __restrict__ seg_cnt, uint32_t nseg, uint32_t* __restrict__ counts) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < total) {
        const uint32_t key = skeys[k];
        if (key != RSH_KEY_NONE) {
            const uint32_t q = k + __ldg(seg_delta + (key >> tag_shift));
            if (q < max_padded) padded[q] = svals[k];
        }
    }
    if (k == 0) {
        uint32_t n = 0;
        for (uint32_t s = 0; s < nseg; ++s) n += seg_cnt[s];
        counts[0] = n;
        counts[1] = n;
    }
}

}  // namespace rsh

using namespace rsh;

namespace {

struct BatchPlan {
    uint32_t nseg = 0, total = 0, tag_shift = 0, key_bits = 0, P = 8, unit_rays = 64, max_padded = 0, hash_drop = 0;
    uint32_t rays_only = 1;  // cleared by any segment whose rays use packets below the root
    bool contiguous = false; // the segments' rays lie back to back in one array: no gather
    bool gather = false;     // copy every segment's rays into one array (packet kernel, not contiguous)
    void *rays_all, *keys, *trimmed, *ckeys, *cbases, *counts, *skeys, *svals, *sorted_keys, *sorted_ids, *scr;
    void *padded, *nodes, *prep, *fsegs, *seg_begin, *seg_cnt, *pstart, *totals, *work, *sched, *seg_delta;
    std::vector<PrepSeg> h_prep;
    std::vector<FusedSeg> h_fsegs;  // in schedule order
    std::vector<uint32_t> h_sched;  // schedule position -> segment index
};

// The context's configuration with a scene's own tuning (rsh_scene_set_tuning) applied.
rsh_config tuned_config(const rsh_config& base, const rsh_scene* sc) {
    rsh_config c = base;
    if (!sc) return c;
    if (sc->tune.grid_bits != RSH_TUNE_DEFAULT) c.grid_bits = sc->tune.grid_bits;
    if (sc->tune.dir_log2 != RSH_TUNE_DEFAULT) c.dir_log2 = sc->tune.dir_log2;
    if (sc->tune.ray_level != RSH_TUNE_DEFAULT) c.ray_level = sc->tune.ray_level;
    return c;
}

rsh_status batch_prepare(rsh_ctx* ctx, const rsh_batch_segment* segs, uint32_t count, BatchPlan& pl) {
    if (!ctx || (!segs && count)) return RSH_ERR_INVALID;
    if (count > 1024) {
        set_error("at most 1024 batch segments");
        return RSH_ERR_INVALID;
    }
    pl.nseg = count;
    uint64_t total = 0;
    for (uint32_t s = 0; s < count; ++s) {
        const rsh_batch_segment& g = segs[s];
        if (!g.scene || (g.n && !g.rays) || (g.any_hit ? !g.flags : !g.hits)) return RSH_ERR_INVALID;
        total += g.n;
    }
    if (total >= (1ull << 31)) return RSH_ERR_INVALID;
    pl.total = (uint32_t)total;
    uint32_t tag_bits = 0;
    while ((1u << tag_bits) < count) ++tag_bits;
    // segment tag above the hash; when both do not fit in 31 bits, the hash's lowest bits are dropped (the
    // hash only orders rays for coherence, no result depends on it). Scenes may tune their own hash width:
    // the tag sits above the widest.
    uint32_t hash_bits = 0;
    for (uint32_t s = 0; s < count; ++s) {
        const rsh_config c = tuned_config(ctx->cfg, segs[s].scene);
        hash_bits = std::max(hash_bits, 3 * c.grid_bits + 2 * c.dir_log2);
    }
    pl.hash_drop = (hash_bits + tag_bits > 31) ? hash_bits + tag_bits - 31 : 0u;
    if (pl.hash_drop > hash_bits) {
        set_error("too many batch segments for a 31-bit key");
        return RSH_ERR_INVALID;
    }
    {
        // a last 8-bit digit pass for 1 or 2 leftover key bits would read and write every pair once more
        // for almost no order: those lowest hash bits are dropped instead (a frame's two segments over a
        // 24-bit hash sort in 3 passes, not 4)
        const uint32_t empty_bit = (ctx->cfg.flags & RSH_FLAG_NO_COMPRESS) ? 1u : 0u;  // sorts one more bit
        const uint32_t kb = hash_bits + tag_bits - pl.hash_drop + empty_bit, tail = kb % 8u;
        if (kb > 8u && tail != 0u && tail <= 2u && hash_bits - pl.hash_drop > tail) pl.hash_drop += tail;
    }
    pl.tag_shift = hash_bits - pl.hash_drop;
    pl.key_bits = pl.tag_shift + tag_bits;
    pl.P = ctx->cfg.packet_size;
    for (uint32_t s = 0; s < count; ++s)
        if (tuned_config(ctx->cfg, segs[s].scene).ray_level < segs[s].scene->h.levels) pl.rays_only = 0;
    // work units: 8 packets for the packet kernel, RSH_RAYS_UNIT sorted rays for the rays-only kernel
    pl.unit_rays = pl.rays_only ? (uint32_t)RSH_RAYS_UNIT : 8 * pl.P;
    pl.max_padded = pl.total + count * pl.unit_rays;
    const uint32_t n = pl.total ? pl.total : 1;
    pl.contiguous = count > 0;
    for (uint32_t s = 0, at = 0; s < count; at += segs[s].n, ++s)
        if (segs[s].n && segs[s].rays != segs[0].rays + at) pl.contiguous = false;
    // one ray array for the ray hierarchy and the packet kernel: the segments' own when they lie back to
    // back, else a gathered copy; the rays-only kernel reads every segment's rays in place
    pl.gather = !pl.contiguous && !pl.rays_only;
    if (pl.contiguous) pl.rays_all = const_cast<rsh_ray*>(segs[0].rays);
    else if (pl.gather) RSH_TRY(ensure(ctx, "b_rays", sizeof(rsh_ray) * (size_t)n, &pl.rays_all));
    else pl.rays_all = nullptr;
    RSH_TRY(ensure(ctx, "b_keys", 4ull * n, &pl.keys));
    RSH_TRY(ensure(ctx, "trimmed", 4ull * n, &pl.trimmed));
    RSH_TRY(ensure(ctx, "ckeys", 4ull * n + 4, &pl.ckeys));
    RSH_TRY(ensure(ctx, "cbases", 4ull * n + 4, &pl.cbases));
    RSH_TRY(ensure(ctx, "b_counts", 64, &pl.counts));
    RSH_TRY(ensure(ctx, "skeys", 4ull * n, &pl.skeys));
    RSH_TRY(ensure(ctx, "svals", 4ull * n, &pl.svals));
    RSH_TRY(ensure(ctx, "sorted_keys", 4ull * n, &pl.sorted_keys));
    RSH_TRY(ensure(ctx, "sorted_ids", 4ull * n, &pl.sorted_ids));
    size_t scr = std::max(compress_scratch_bytes(n), sort_scratch_bytes(n, pl.key_bits + 1u));
    scr = std::max(scr, decompress_scratch_bytes(n));
    RSH_TRY(ensure(ctx, "scratch", scr, &pl.scr));
    RSH_TRY(ensure(ctx, "b_padded", 4ull * pl.max_padded, &pl.padded));
    uint32_t off[4];
    const uint32_t capn = hierarchy_capacity(pl.max_padded, pl.P, off);
    RSH_TRY(ensure(ctx, "b_nodes", sizeof(rsh_node) * (size_t)capn, &pl.nodes));
    RSH_TRY(ensure(ctx, "b_prep", sizeof(PrepSeg) * (count ? count : 1), &pl.prep));
    RSH_TRY(ensure(ctx, "b_fsegs", sizeof(FusedSeg) * (count ? count : 1), &pl.fsegs));
    RSH_TRY(ensure(ctx, "b_seg_begin", 4ull * (count + 1), &pl.seg_begin));
    RSH_TRY(ensure(ctx, "b_seg_cnt", 4ull * (count + 1), &pl.seg_cnt));
    RSH_TRY(ensure(ctx, "b_pstart", 4ull * (count + 1), &pl.pstart));
    RSH_TRY(ensure(ctx, "b_totals", 64, &pl.totals));
    RSH_TRY(ensure(ctx, "b_work", 64, &pl.work));
    RSH_TRY(ensure(ctx, "b_sched", 4ull * (count + 1), &pl.sched));
    RSH_TRY(ensure(ctx, "b_seg_delta", 4ull * (count + 1), &pl.seg_delta));
    pl.h_prep.resize(count);
    pl.h_fsegs.resize(count);
    uint32_t start = 0;
    for (uint32_t s = 0; s < count; ++s) {
        const rsh_batch_segment& g = segs[s];
        const rsh_scene* sc = g.scene;
        PrepSeg& p = pl.h_prep[s];
        p.rays = g.rays;
        p.start = start;
        p.any_hit = g.any_hit ? 1u : 0u;
        p.flags = g.flags;
        p.hits = reinterpret_cast<unsigned long long*>(g.hits);
        const rsh_config tc = tuned_config(ctx->cfg, sc);
        RSH_TRY(make_hash_params(sc, tc, 0, p.hp));
        // per-ray job words and packet stack entries hold an object-node index of level >= 1 in 20 bits;
        // cluster triangles are staged in shared memory (at most 32)
        if ((sc->h.levels > 1 && sc->h.level_size[1] > (1u << 20)) || sc->h.cluster > 32) {
            set_error("batched traversal needs at most 1,048,576 level-1 object nodes and clusters of <= 32");
            return RSH_ERR_INVALID;
        }
        FusedSeg& f = pl.h_fsegs[s];
        std::memset(&f, 0, sizeof(f));
        f.spheres = sc->h.spheres;
        f.kids = sc->h.kids;
        f.tris = sc->h.tris;
        f.boxes = sc->h.boxes;
        f.wboxes = sc->h.wboxes;
        f.wtris = sc->h.wtris;
        f.wnodes = sc->h.wnodes;
        f.wnroot = sc->h.wnroot;
        f.tri_count = sc->tri_count;
        f.cluster = sc->h.cluster;
        f.levels = sc->h.levels;
        for (uint32_t l = 0; l < sc->h.levels; ++l) {
            f.lvl_off[l] = sc->h.level_off[l];
            f.lvl_size[l] = sc->h.level_size[l];
        }
        f.any_hit = p.any_hit;
        f.ray_level = tc.ray_level;
        f.rays = g.rays;
        f.flags = g.flags;
        f.hits = reinterpret_cast<unsigned long long*>(g.hits);
        f.slot_base = start;
        start += g.n;
    }
    // schedule: closest-hit segments first (incoherent, long rays), then by size, descending
    pl.h_sched.resize(count);
    for (uint32_t s = 0; s < count; ++s) pl.h_sched[s] = s;
    std::stable_sort(pl.h_sched.begin(), pl.h_sched.end(), [&](uint32_t a, uint32_t b) {
        if (segs[a].any_hit != segs[b].any_hit) return segs[a].any_hit == 0;
        return segs[a].n > segs[b].n;
    });
    std::vector<FusedSeg> by_seg(pl.h_fsegs);
    for (uint32_t k = 0; k < count; ++k) pl.h_fsegs[k] = by_seg[pl.h_sched[k]];
    return RSH_OK;
}

// Host staging of the segment tables (pinned, read by asynchronous copies): a ring of slots per context,
// each fenced by an event recorded after its copies, so a slot is never rewritten while a copy that reads
// it may still be pending. A captured graph gets its own staging buffer, alive as long as the graph.
struct StageSlot {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
    bool used = false;
};
struct HostStage {
    StageSlot slot[4];
    uint32_t next = 0;
};
std::map<const rsh_ctx*, HostStage> g_stage;
std::mutex g_stage_mu;

size_t table_bytes(const BatchPlan& pl) {
    return sizeof(PrepSeg) * pl.nseg + sizeof(FusedSeg) * pl.nseg + 4ull * pl.nseg + 256;
}

void fill_tables(const BatchPlan& pl, char* b) {
    std::memcpy(b, pl.h_prep.data(), sizeof(PrepSeg) * pl.nseg);
    std::memcpy(b + sizeof(PrepSeg) * pl.nseg, pl.h_fsegs.data(), sizeof(FusedSeg) * pl.nseg);
    std::memcpy(b + (sizeof(PrepSeg) + sizeof(FusedSeg)) * pl.nseg, pl.h_sched.data(), 4ull * pl.nseg);
}

// Returns pinned memory holding the tables in a ring slot whose fence the caller records with *fence after
// enqueuing the copies.
rsh_status stage_tables(rsh_ctx* ctx, const BatchPlan& pl, char** out, cudaEvent_t* fence) {
    const size_t need = table_bytes(pl);
    std::lock_guard<std::mutex> lk(g_stage_mu);
    HostStage& hs = g_stage[ctx];
    StageSlot& sl = hs.slot[hs.next];
    hs.next = (hs.next + 1) % 4;
    if (sl.used) RSH_CUDA(cudaEventSynchronize(sl.done));
    if (!sl.done) RSH_CUDA(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
    if (sl.bytes < need) {
        if (sl.ptr) cudaFreeHost(sl.ptr);
        sl.ptr = nullptr;
        RSH_CUDA(cudaMallocHost(&sl.ptr, need));
        sl.bytes = need;
    }
    fill_tables(pl, static_cast<char*>(sl.ptr));
    sl.used = true;
    *out = static_cast<char*>(sl.ptr);
    *fence = sl.done;
    return RSH_OK;
}

// pre_staged != nullptr: tables already in pinned memory owned by the caller (a captured graph, which must
// not allocate while capturing); otherwise a fenced ring slot of the context.
// reset_stats: zero the node / triangle test counters first (a frame keeps counting over its batches).
rsh_status batch_enqueue(rsh_ctx* ctx, BatchPlan& pl, cudaStream_t s, char* pre_staged = nullptr,
                         bool reset_stats = true, bool prekeyed = false) {
    if (pl.nseg == 0) return RSH_OK;
    char* tables = pre_staged;
    cudaEvent_t fence = nullptr;
    if (!tables) RSH_TRY(stage_tables(ctx, pl, &tables, &fence));
    RSH_CUDA(cudaMemcpyAsync(pl.prep, tables, sizeof(PrepSeg) * pl.nseg, cudaMemcpyHostToDevice, s));
    RSH_CUDA(cudaMemcpyAsync(pl.fsegs, tables + sizeof(PrepSeg) * pl.nseg, sizeof(FusedSeg) * pl.nseg,
                             cudaMemcpyHostToDevice, s));
    RSH_CUDA(cudaMemcpyAsync(pl.sched, tables + (sizeof(PrepSeg) + sizeof(FusedSeg)) * pl.nseg, 4ull * pl.nseg,
                             cudaMemcpyHostToDevice, s));
    if (fence) RSH_CUDA(cudaEventRecord(fence, s));
    if (reset_stats) RSH_CUDA(cudaMemsetAsync(ctx->d_stats, 0, 64, s));
    if (pl.total == 0) return RSH_OK;
    uint32_t* cnt = static_cast<uint32_t*>(pl.counts);
    uint32_t* totals = static_cast<uint32_t*>(pl.totals);
    int th = stage_begin(ctx, RSH_STAGE_RAYGEN, s);  // gather + hash + per-segment counts
    if (!prekeyed) {
        RSH_CUDA(cudaMemsetAsync(pl.seg_cnt, 0, 4ull * pl.nseg, s));
        k_batch_prep<<<(pl.total + 255) / 256, 256, 0, s>>>(
            static_cast<PrepSeg*>(pl.prep), pl.nseg, pl.total, pl.tag_shift, pl.hash_drop,
            static_cast<rsh_ray*>(pl.rays_all), pl.gather, static_cast<uint32_t*>(pl.keys),
            static_cast<uint32_t*>(pl.seg_cnt));
        note_launch();
        RSH_CUDA(cudaGetLastError());
    }
    k_batch_bounds<<<1, 1024, 0, s>>>(static_cast<uint32_t*>(pl.seg_cnt), pl.nseg, pl.unit_rays,
                                      static_cast<uint32_t*>(pl.seg_begin), static_cast<uint32_t*>(pl.pstart),
                                      static_cast<uint32_t*>(pl.seg_delta), static_cast<uint32_t*>(pl.sched),
                                      static_cast<FusedSeg*>(pl.fsegs), totals, static_cast<uint32_t*>(pl.padded),
                                      pl.max_padded);
    note_launch();
    RSH_CUDA(cudaGetLastError());
    stage_end(ctx, th, s);
    if (ctx->cfg.flags & RSH_FLAG_NO_COMPRESS) {
        // incoherent batches: sort the slots' own keys (one more bit, so that empty slots go last) and
        // scatter the sorted slots to the padded layout
        th = stage_begin(ctx, RSH_STAGE_SORT, s);
        RSH_CUDA(launch_sort_pairs(static_cast<uint32_t*>(pl.keys), nullptr, static_cast<uint32_t*>(pl.skeys),
                                   static_cast<uint32_t*>(pl.svals), pl.total, nullptr, pl.key_bits + 1u, pl.scr,
                                   ctx->d_err, s));
        stage_end(ctx, th, s);
        th = stage_begin(ctx, RSH_STAGE_DECOMPRESS, s);
        k_batch_scatter<<<(pl.total + 255) / 256, 256, 0, s>>>(
            static_cast<uint32_t*>(pl.skeys), static_cast<uint32_t*>(pl.svals), pl.total, pl.tag_shift,
            static_cast<const uint32_t*>(pl.seg_delta), static_cast<uint32_t*>(pl.padded), pl.max_padded,
            static_cast<uint32_t*>(pl.seg_cnt), pl.nseg, cnt);
        note_launch();
        RSH_CUDA(cudaGetLastError());
        stage_end(ctx, th, s);
    } else {
    th = stage_begin(ctx, RSH_STAGE_COMPRESS, s);
    RSH_CUDA(launch_compress(static_cast<uint32_t*>(pl.keys), pl.total, static_cast<uint32_t*>(pl.trimmed),
                             static_cast<uint32_t*>(pl.ckeys), static_cast<uint32_t*>(pl.cbases), cnt, pl.scr,
                             ctx->d_err, s));
    stage_end(ctx, th, s);
    th = stage_begin(ctx, RSH_STAGE_SORT, s);
    RSH_CUDA(launch_sort_pairs(static_cast<uint32_t*>(pl.ckeys), nullptr, static_cast<uint32_t*>(pl.skeys),
                               static_cast<uint32_t*>(pl.svals), pl.total, cnt + 1, pl.key_bits, pl.scr, ctx->d_err,
                               s));
    stage_end(ctx, th, s);
    th = stage_begin(ctx, RSH_STAGE_DECOMPRESS, s);
    // straight into the padded layout: ray k of the sorted order goes to k + seg_delta[its segment]
    PaddedOut po{static_cast<const uint32_t*>(pl.seg_delta), pl.tag_shift, pl.max_padded,
                 static_cast<uint32_t*>(pl.padded)};
    RSH_CUDA(launch_decompress(static_cast<uint32_t*>(pl.skeys), static_cast<uint32_t*>(pl.svals),
                               static_cast<uint32_t*>(pl.cbases), static_cast<uint32_t*>(pl.trimmed), cnt, pl.total,
                               nullptr, nullptr, pl.scr, ctx->d_err, s, &po));
    stage_end(ctx, th, s);
    }
    if (!pl.rays_only) {  // rays that leave their packets at the root never read the ray hierarchy
        th = stage_begin(ctx, RSH_STAGE_BUILD, s);
        RSH_CUDA(launch_build_rsh(static_cast<rsh_ray*>(pl.rays_all), static_cast<uint32_t*>(pl.padded),
                                  pl.max_padded, totals, pl.P, static_cast<rsh_node*>(pl.nodes), s));
        stage_end(ctx, th, s);
    }
    RSH_CUDA(cudaMemsetAsync(pl.work, 0, 16, s));
    FusedArgs fa{};
    fa.nodes = static_cast<rsh_node*>(pl.nodes);
    hierarchy_capacity(pl.max_padded, pl.P, fa.node_off);
    fa.packet = pl.P;
    fa.rays = static_cast<rsh_ray*>(pl.rays_all);
    fa.sorted_ids = static_cast<uint32_t*>(pl.padded);
    fa.segs = static_cast<FusedSeg*>(pl.fsegs);
    fa.nseg = pl.nseg;
    fa.unit_seg = nullptr;
    fa.units_max = pl.max_padded / pl.unit_rays;
    fa.d_units = totals + 1;
    fa.work = static_cast<uint32_t*>(pl.work);
    fa.rays_only = pl.rays_only;
    fa.blocks_per_sm = ctx->cfg.fused_blocks;
    fa.share_tail = (ctx->cfg.flags & RSH_FLAG_SEQUENTIAL_RAYS) ? 0u : 1u;
    fa.node_tests = ctx->d_stats;
    fa.tri_tests = ctx->d_stats + 1;
    fa.err = ctx->d_err;
    th = stage_begin(ctx, RSH_STAGE_TRAVERSE, s);  // traversal and intersection in one kernel
    RSH_CUDA(launch_fused(fa, s));
    stage_end(ctx, th, s);
    return RSH_OK;
}

struct GraphExec {
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    rsh_ctx* ctx = nullptr;
    void* stage = nullptr;  // pinned segment tables read by every replay
};

}  // namespace

namespace rsh {
// One segment whose rays are already in a coherent order (the frame's primary rays, generated tile by
// tile), traced by the rays-only kernel in that order: no hash, compression, sort or ray hierarchy.
// Scenes whose rays use packets below the root go through batch_trace.
rsh_status batch_trace_ordered(rsh_ctx* ctx, const rsh_batch_segment& seg, cudaStream_t s) {
    if (!ctx || !seg.scene) return RSH_ERR_INVALID;
    const rsh_config tc = tuned_config(ctx->cfg, seg.scene);
    if (seg.n == 0 || tc.ray_level < seg.scene->h.levels) return batch_trace(ctx, &seg, 1, s, false);
    BatchPlan pl;
    RSH_TRY(batch_prepare(ctx, &seg, 1, pl));
    pl.h_fsegs[0].unit_begin = 0;
    char* tables = nullptr;
    cudaEvent_t fence = nullptr;
    RSH_TRY(stage_tables(ctx, pl, &tables, &fence));
    RSH_CUDA(cudaMemcpyAsync(pl.fsegs, tables + sizeof(PrepSeg) * pl.nseg, sizeof(FusedSeg), cudaMemcpyHostToDevice,
                             s));
    RSH_CUDA(cudaEventRecord(fence, s));
    if (seg.any_hit) RSH_CUDA(cudaMemsetAsync(seg.flags, 0, 4ull * seg.n, s));
    else RSH_CUDA(launch_fill_u64(reinterpret_cast<unsigned long long*>(seg.hits), RSH_HIT_NONE, seg.n, s));
    RSH_CUDA(cudaMemsetAsync(pl.work, 0, 16, s));
    FusedArgs fa{};
    fa.packet = pl.P;
    fa.rays = seg.rays;
    fa.sorted_ids = nullptr;
    fa.ordered_n = seg.n;
    fa.segs = static_cast<FusedSeg*>(pl.fsegs);
    fa.nseg = 1;
    fa.unit_seg = nullptr;
    fa.units_max = (seg.n + pl.unit_rays - 1) / pl.unit_rays;
    fa.d_units = nullptr;
    fa.work = static_cast<uint32_t*>(pl.work);
    fa.rays_only = 1;
    fa.blocks_per_sm = ctx->cfg.fused_blocks;
    fa.share_tail = (ctx->cfg.flags & RSH_FLAG_SEQUENTIAL_RAYS) ? 0u : 1u;
    fa.node_tests = ctx->d_stats;
    fa.tri_tests = ctx->d_stats + 1;
    fa.err = ctx->d_err;
    ctx->last_stream = s;
    RSH_CUDA(launch_fused(fa, s));
    ctx->batch_counts_host.assign(1, seg.n);
    return RSH_OK;
}

// rsh_batch_trace without resetting the stage timers (a fused frame keeps its own).
rsh_status batch_key_layout(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count, BatchKeyLayout& out) {
    if (count > 2) return RSH_ERR_INVALID;
    BatchPlan pl;
    RSH_TRY(batch_prepare(ctx, segments, count, pl));
    if (pl.gather || (count && !pl.contiguous)) {
        set_error("keys from ray generation need the segments' rays back to back in one array");
        return RSH_ERR_INVALID;
    }
    out.keys = static_cast<uint32_t*>(pl.keys);
    out.seg_cnt = static_cast<uint32_t*>(pl.seg_cnt);
    out.tag_shift = pl.tag_shift;
    out.hash_drop = pl.hash_drop;
    for (uint32_t i = 0; i < count; ++i) {
        out.start[i] = pl.h_prep[i].start;
        out.hp[i] = pl.h_prep[i].hp;
    }
    return RSH_OK;
}

rsh_status batch_trace(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count, cudaStream_t stream,
                       bool reset_stats, bool prekeyed) {
    BatchPlan pl;
    RSH_TRY(batch_prepare(ctx, segments, count, pl));
    ctx->last_stream = stream;
    RSH_TRY(batch_enqueue(ctx, pl, stream, nullptr, reset_stats, prekeyed));
    ctx->batch_counts_host.assign(1, pl.total);
    return RSH_OK;
}

// Frees the context's staging ring (called by rsh_destroy).
void batch_release_ctx(const rsh_ctx* ctx) {
    std::lock_guard<std::mutex> lk(g_stage_mu);
    auto it = g_stage.find(ctx);
    if (it == g_stage.end()) return;
    for (StageSlot& sl : it->second.slot) {
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.ptr) cudaFreeHost(sl.ptr);
    }
    g_stage.erase(it);
}
}  // namespace rsh

extern "C" {

rsh_status rsh_batch_trace(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count, rsh_stream_t stream) {
    if (!ctx) return RSH_ERR_INVALID;
    ctx->tev_used = 0;  // stage timers (RSH_FLAG_STAGE_TIMERS) cover this call only
    ctx->tmarks.clear();
    return batch_trace(ctx, segments, count, stream, true);
}

rsh_status rsh_batch_graph_create(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count,
                                  rsh_stream_t stream, void** graph_exec) {
    if (!ctx || !graph_exec) return RSH_ERR_INVALID;
    if (stream == nullptr) {
        set_error("graph capture needs a non-default stream");
        return RSH_ERR_INVALID;
    }
    BatchPlan pl;
    RSH_TRY(batch_prepare(ctx, segments, count, pl));
    // warm-up run outside capture (sizes buffers, sets kernel attributes)
    RSH_TRY(batch_enqueue(ctx, pl, stream));
    RSH_CUDA(cudaStreamSynchronize(stream));
    GraphExec* g = new GraphExec();
    g->ctx = ctx;
    cudaError_t e = cudaMallocHost(&g->stage, table_bytes(pl));
    if (e != cudaSuccess) {
        delete g;
        return cuda_status(e, "rsh_batch_graph_create: staging");
    }
    fill_tables(pl, static_cast<char*>(g->stage));
    e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaFreeHost(g->stage);
        delete g;
        return cuda_status(e, "cudaStreamBeginCapture");
    }
    rsh_status st = batch_enqueue(ctx, pl, stream, static_cast<char*>(g->stage));
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(stream, &graph);
    if (st != RSH_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (g->stage) cudaFreeHost(g->stage);
        delete g;
        return st != RSH_OK ? st : cuda_status(e, "cudaStreamEndCapture");
    }
    g->graph = graph;
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        if (g->stage) cudaFreeHost(g->stage);
        delete g;
        return cuda_status(e, "cudaGraphInstantiate");
    }
    ctx->last_stream = stream;
    *graph_exec = g;
    return RSH_OK;
}

rsh_status rsh_batch_graph_launch(void* graph_exec, rsh_stream_t stream) {
    GraphExec* g = static_cast<GraphExec*>(graph_exec);
    if (!g || !g->exec) return RSH_ERR_INVALID;
    RSH_CUDA(cudaGraphLaunch(g->exec, stream));
    g->ctx->last_stream = stream;
    return RSH_OK;
}

rsh_status rsh_batch_graph_destroy(void* graph_exec) {
    GraphExec* g = static_cast<GraphExec*>(graph_exec);
    if (!g) return RSH_ERR_INVALID;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->stage) cudaFreeHost(g->stage);
    delete g;
    return RSH_OK;
}

rsh_status rsh_batch_stats_get(rsh_ctx* ctx, rsh_frame_stats* out) {
    if (!ctx || !out) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(ctx->last_stream));
    rsh_frame_stats st{};
    uint32_t cnt[2] = {0, 0};
    void* counts = ctx->bufs.count("b_counts") ? ctx->bufs["b_counts"].ptr : nullptr;
    if (counts) RSH_CUDA(cudaMemcpy(cnt, counts, 8, cudaMemcpyDeviceToHost));
    unsigned long long d[2] = {0, 0};
    RSH_CUDA(cudaMemcpy(d, ctx->d_stats, 16, cudaMemcpyDeviceToHost));
    st.reflection_rays = cnt[0];
    st.chunks = cnt[1];
    st.node_tests = d[0];
    st.tri_tests = d[1];
    for (const auto& m : ctx->tmarks) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ctx->tev[m.second], ctx->tev[m.second + 1]) == cudaSuccess && m.first < 12)
            st.stage_ms[m.first] += ms;
    }
    cudaGetLastError();
    *out = st;
    return RSH_OK;
}

rsh_status rsh_trace_rays_fused(rsh_ctx* ctx, const rsh_scene* sc, const rsh_ray* rays, uint32_t n, int any_hit,
                                uint64_t* hits, uint32_t* flags, rsh_stream_t stream) {
    if (!ctx || !sc || !rays) return RSH_ERR_INVALID;
    if (any_hit ? !flags : !hits) return RSH_ERR_INVALID;
    rsh_batch_segment seg;
    seg.scene = sc;
    seg.rays = rays;
    seg.n = n;
    seg.any_hit = any_hit;
    seg.hits = hits;
    seg.flags = flags;
    return rsh_batch_trace(ctx, &seg, 1, stream);
}

rsh_status rsh_autotune(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count, const uint32_t* grid_bits,
                        uint32_t n_grid, const uint32_t* dir_log2, uint32_t n_dir, const uint32_t* packet_sizes,
                        uint32_t n_packet, rsh_stream_t stream, rsh_config* best) {
    if (!ctx || !grid_bits || !dir_log2 || !packet_sizes || !n_grid || !n_dir || !n_packet) return RSH_ERR_INVALID;
    const rsh_config base = ctx->cfg;
    rsh_config best_cfg = base;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    RSH_CUDA(cudaEventCreate(&e0));
    RSH_CUDA(cudaEventCreate(&e1));
    for (uint32_t a = 0; a < n_grid; ++a)
        for (uint32_t b = 0; b < n_dir; ++b)
            for (uint32_t c = 0; c < n_packet; ++c) {
                rsh_config cfg = base;
                cfg.grid_bits = grid_bits[a];
                cfg.dir_log2 = dir_log2[b];
                cfg.packet_size = packet_sizes[c];
                if (rsh_set_config(ctx, &cfg) != RSH_OK) continue;
                BatchPlan pl;
                if (batch_prepare(ctx, segments, count, pl) != RSH_OK) continue;
                if (batch_enqueue(ctx, pl, stream) != RSH_OK) continue;  // warm-up
                cudaEventRecord(e0, stream);
                const int reps = 2;
                rsh_status st = RSH_OK;
                for (int r = 0; r < reps && st == RSH_OK; ++r) st = batch_enqueue(ctx, pl, stream);
                cudaEventRecord(e1, stream);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (st == RSH_OK && ms / reps < best_ms) {
                    best_ms = ms / reps;
                    best_cfg = cfg;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    rsh_set_config(ctx, &best_cfg);
    if (best) *best = best_cfg;
    return best_ms < 1e30f ? RSH_OK : RSH_ERR_INVALID;
}

rsh_status rsh_scene_set_tuning(rsh_scene* sc, const rsh_scene_tuning* t) {
    if (!sc || !t) return RSH_ERR_INVALID;
    const uint32_t D = RSH_TUNE_DEFAULT;
    if ((t->grid_bits != D && (t->grid_bits < 1 || t->grid_bits > 10)) ||
        (t->dir_log2 != D && (t->dir_log2 < 1 || t->dir_log2 > 6)) || (t->ray_level != D && t->ray_level > 15)) {
        set_error("scene tuning out of range");
        return RSH_ERR_INVALID;
    }
    sc->tune = *t;
    return RSH_OK;
}

rsh_status rsh_scene_get_tuning(const rsh_scene* sc, rsh_scene_tuning* out) {
    if (!sc || !out) return RSH_ERR_INVALID;
    *out = sc->tune;
    return RSH_OK;
}

}  // extern "C"

namespace {
// Mean time of one batch after a warm-up (CUDA events on the stream).
rsh_status time_batch(rsh_ctx* ctx, const rsh_batch_segment* segs, uint32_t count, uint32_t reps,
                      cudaStream_t stream, float* ms_out) {
    BatchPlan pl;
    RSH_TRY(batch_prepare(ctx, segs, count, pl));
    RSH_TRY(batch_enqueue(ctx, pl, stream));
    cudaEvent_t e0, e1;
    RSH_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return RSH_ERR_CUDA;
    }
    rsh_status st = RSH_OK;
    cudaEventRecord(e0, stream);
    for (uint32_t r = 0; r < reps && st == RSH_OK; ++r) st = batch_enqueue(ctx, pl, stream);
    cudaEventRecord(e1, stream);
    const cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != RSH_OK) return st;
    if (e != cudaSuccess) return RSH_ERR_CUDA;
    *ms_out = ms / (float)reps;
    return RSH_OK;
}

// Packet size on the whole batch: keeps the context's value unless another one is faster than cur_ms.
float tune_packet(rsh_ctx* ctx, const rsh_batch_segment* segs, uint32_t count, const rsh_tune_space& sp,
                  uint32_t reps, cudaStream_t stream, float cur_ms) {
    const rsh_config base = ctx->cfg;
    rsh_config best = base;
    for (uint32_t i = 0; i < sp.n_packet; ++i) {
        rsh_config c = base;
        c.packet_size = sp.packet_sizes[i];
        if (c.packet_size == base.packet_size || rsh_set_config(ctx, &c) != RSH_OK) continue;
        float ms;
        if (time_batch(ctx, segs, count, reps, stream, &ms) == RSH_OK && ms < cur_ms) {
            cur_ms = ms;
            best = c;
        }
    }
    rsh_set_config(ctx, &best);
    return cur_ms;
}

// CTAs per SM of the traversal launch on the whole batch, like the packet size.
float tune_blocks(rsh_ctx* ctx, const rsh_batch_segment* segs, uint32_t count, const rsh_tune_space& sp,
                  uint32_t reps, cudaStream_t stream, float cur_ms) {
    const rsh_config base = ctx->cfg;
    rsh_config best = base;
    for (uint32_t i = 0; i < sp.n_fused_blocks; ++i) {
        rsh_config c = base;
        c.fused_blocks = sp.fused_blocks[i];
        if (c.fused_blocks == base.fused_blocks || rsh_set_config(ctx, &c) != RSH_OK) continue;
        float ms;
        if (time_batch(ctx, segs, count, reps, stream, &ms) == RSH_OK && ms < cur_ms) {
            cur_ms = ms;
            best = c;
        }
    }
    rsh_set_config(ctx, &best);
    return cur_ms;
}
}  // namespace

extern "C" rsh_status rsh_autotune_scenes(rsh_ctx* ctx, const rsh_batch_segment* segs, uint32_t count,
                                          const rsh_tune_space* space, rsh_stream_t stream, float* best_ms,
                                          float* untuned_ms) {
    if (!ctx || !space || !segs || !count) return RSH_ERR_INVALID;
    if ((space->n_grid && !space->grid_bits) || (space->n_dir && !space->dir_log2) ||
        (space->n_ray_level && !space->ray_levels) || (space->n_packet && !space->packet_sizes) ||
        (space->n_fused_blocks && !space->fused_blocks))
        return RSH_ERR_INVALID;
    const uint32_t reps = space->reps ? space->reps : 2u;
    // hash widths that fit beside this batch's segment tag without dropping bits: wider points would be
    // tuned on a scene's own segments (a narrower tag) but lose their low bits in the whole batch
    uint32_t tag_bits = 0;
    while ((1u << tag_bits) < count) ++tag_bits;
    const uint32_t max_hash_bits = 31u - std::min(tag_bits, 31u);
    std::vector<rsh_scene*> scenes;
    for (uint32_t i = 0; i < count; ++i) {
        if (!segs[i].scene) return RSH_ERR_INVALID;
        rsh_scene* sc = const_cast<rsh_scene*>(segs[i].scene);
        if (std::find(scenes.begin(), scenes.end(), sc) == scenes.end()) scenes.push_back(sc);
    }
    const rsh_scene_tuning none{RSH_TUNE_DEFAULT, RSH_TUNE_DEFAULT, RSH_TUNE_DEFAULT};
    for (rsh_scene* sc : scenes) sc->tune = none;
    const rsh_config start = ctx->cfg;
    float ms;
    RSH_TRY(time_batch(ctx, segs, count, reps, stream, &ms));
    const float untuned = ms;
    if (untuned_ms) *untuned_ms = ms;
    ms = tune_packet(ctx, segs, count, *space, reps, stream, ms);
    // each scene on its own segments, one parameter at a time
    for (rsh_scene* sc : scenes) {
        std::vector<rsh_batch_segment> sub;
        for (uint32_t i = 0; i < count; ++i)
            if (segs[i].scene == sc) sub.push_back(segs[i]);
        rsh_scene_tuning t{ctx->cfg.grid_bits, ctx->cfg.dir_log2, ctx->cfg.ray_level};
        sc->tune = t;
        float cur;
        if (time_batch(ctx, sub.data(), (uint32_t)sub.size(), reps, stream, &cur) != RSH_OK) {
            sc->tune = none;
            continue;
        }
        for (int param = 0; param < 3; ++param) {
            const uint32_t* vals = param == 0 ? space->grid_bits : param == 1 ? space->dir_log2 : space->ray_levels;
            const uint32_t nv = param == 0 ? space->n_grid : param == 1 ? space->n_dir : space->n_ray_level;
            for (uint32_t k = 0; k < nv; ++k) {
                rsh_scene_tuning trial = t;
                uint32_t& field = param == 0 ? trial.grid_bits : param == 1 ? trial.dir_log2 : trial.ray_level;
                if (field == vals[k]) continue;
                field = vals[k];
                if (3u * trial.grid_bits + 2u * trial.dir_log2 > max_hash_bits) continue;
                if (rsh_scene_set_tuning(sc, &trial) != RSH_OK) continue;
                float m2;
                if (time_batch(ctx, sub.data(), (uint32_t)sub.size(), reps, stream, &m2) == RSH_OK && m2 < cur) {
                    cur = m2;
                    t = trial;
                }
            }
            sc->tune = t;
        }
    }
    RSH_TRY(time_batch(ctx, segs, count, reps, stream, &ms));
    // the rays-only kernel runs only when every segment's rays leave their packets at the root, which the
    // per-scene choices above cannot see: try all scenes there at once too
    {
        std::vector<rsh_scene_tuning> keep;
        for (rsh_scene* sc : scenes) keep.push_back(sc->tune);
        for (rsh_scene* sc : scenes) sc->tune.ray_level = 15u;
        float m2;
        if (time_batch(ctx, segs, count, reps, stream, &m2) == RSH_OK && m2 < ms) {
            ms = m2;
        } else {
            for (size_t k = 0; k < scenes.size(); ++k) scenes[k]->tune = keep[k];
        }
    }
    ms = tune_packet(ctx, segs, count, *space, reps, stream, ms);
    ms = tune_blocks(ctx, segs, count, *space, reps, stream, ms);
    // run compression on or off, then the launch's end shared among a drained warp's lanes or not, each on
    // the whole batch
    for (const uint32_t flag : {RSH_FLAG_NO_COMPRESS, RSH_FLAG_SEQUENTIAL_RAYS}) {
        rsh_config c = ctx->cfg;
        const rsh_config keep = c;
        c.flags ^= flag;
        float m2;
        if (rsh_set_config(ctx, &c) == RSH_OK && time_batch(ctx, segs, count, reps, stream, &m2) == RSH_OK &&
            m2 < ms)
            ms = m2;
        else
            rsh_set_config(ctx, &keep);
    }
    // keep the untuned configuration when the search found nothing faster on the whole batch (the
    // per-scene steps time sub-batches, which need not add up)
    if (!(ms < untuned)) {
        for (rsh_scene* sc : scenes) sc->tune = none;
        rsh_set_config(ctx, &start);
        ms = untuned;
    }
    if (best_ms) *best_ms = ms;
    return RSH_OK;
}
