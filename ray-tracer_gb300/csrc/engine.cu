// Engine + C ABI: context, budgeted device buffers, scenes, lights, camera, the per-frame path and the
// stage-level entry points of include/rsh.h.
//
// Reference host driver: display() (main.cpp:1077-1368) -> createShadowRays / castRays /
// colorShadowRays / createReflectionRays / colorReflectionRays (main.cpp:630-1054), buffers sized in
// reshape() (main.cpp:1371-1520), scene packing in init() (main.cpp:2374-2656). Differences by design:
// no GL (a primary ray cast writes the surface buffer), no host loop over 5000-triangle batches (the
// object hierarchy covers every triangle), counts stay on the device, errors are status codes.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "engine.h"

namespace rsh {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void note_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Every stage is also an NVTX range on the calling host thread (a no-op unless a profiler such as Nsight
// Systems is attached), so a timeline shows the pipeline's stages around their kernels.
static const char* const kStageNames[RSH_STAGE_COUNT] = {"rsh primary", "rsh raygen",     "rsh compress",
                                                         "rsh sort",    "rsh decompress", "rsh build",
                                                         "rsh traverse", "rsh intersect", "rsh shade"};

int stage_begin(rsh_ctx* ctx, int stage, cudaStream_t s) {
    nvtxRangePushA(stage >= 0 && stage < RSH_STAGE_COUNT ? kStageNames[stage] : "rsh stage");
    if (!(ctx->cfg.flags & RSH_FLAG_STAGE_TIMERS) || ctx->timers_paused) return -1;
    while (ctx->tev.size() < ctx->tev_used + 2) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) return -1;
        ctx->tev.push_back(ev);
    }
    const uint32_t i = ctx->tev_used;
    ctx->tev_used += 2;
    cudaEventRecord(ctx->tev[i], s);
    ctx->tmarks.push_back({stage, i});
    return (int)i;
}

void stage_end(rsh_ctx* ctx, int handle, cudaStream_t s) {
    nvtxRangePop();
    if (handle < 0) return;
    cudaEventRecord(ctx->tev[handle + 1], s);
}

void set_error(const std::string& msg) { g_last_error = msg; }

rsh_status cuda_status(cudaError_t e, const char* where) {
    set_error(std::string(where) + ": " + cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RSH_ERR_OOM : RSH_ERR_CUDA;
}

rsh_status ensure_buf(rsh_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 256;
    if (b.bytes >= bytes) return RSH_OK;
    const size_t want = ((bytes + (bytes >> 3)) + 255) & ~size_t(255);  // grow with 12.5% headroom
    if (ctx->allocated - b.bytes + want > ctx->budget) {
        set_error("HBM budget exceeded");
        return RSH_ERR_OOM;
    }
    if (b.ptr) {
        cudaFree(b.ptr);
        ctx->allocated -= b.bytes;
        b.ptr = nullptr;
        b.bytes = 0;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) return cuda_status(e, "cudaMalloc");
    b.ptr = p;
    b.bytes = want;
    ctx->allocated += want;
    return RSH_OK;
}

void release_buf(rsh_ctx* ctx, DevBuf& b) {
    if (b.ptr) {
        cudaFree(b.ptr);
        ctx->allocated -= b.bytes;
    }
    b.ptr = nullptr;
    b.bytes = 0;
}

rsh_status ensure(rsh_ctx* ctx, const char* name, size_t bytes, void** out) {
    DevBuf& b = ctx->bufs[name];
    RSH_TRY(ensure_buf(ctx, b, bytes));
    *out = b.ptr;
    return RSH_OK;
}

rsh_status make_hash_params(const rsh_scene* sc, const rsh_config& cfg, uint32_t tag_bits, HashP& out) {
    rsh_hash_params hp;
    rsh_status st = rsh_hash_params_make(sc->lo, sc->hi, cfg.grid_bits, cfg.dir_log2, tag_bits, &hp);
    if (st != RSH_OK) return st;
    out = to_hashp(hp);
    return RSH_OK;
}

static uint64_t cand_capacity(const rsh_ctx* ctx) {
    return ctx->cfg.candidate_capacity ? ctx->cfg.candidate_capacity : (1ull << 28);  // 2 GiB of candidates
}

// Traverse + intersect with the overflow/resume protocol: the traversal stops at the first work unit
// whose candidates do not fit, the host drains the buffer through the intersection kernel and restarts
// the traversal at that unit (a redone unit only repeats idempotent tests).
static rsh_status traverse_and_intersect(rsh_ctx* ctx, const rsh_scene* sc, const rsh_node* nodes,
                                         const rsh_ray* rays, const uint32_t* sorted_ids,
                                         uint32_t max_rays, const uint32_t* d_count, bool any_hit,
                                         uint32_t* flags, unsigned long long* hits, cudaStream_t s) {
    if (sc->tri_count == 0 || max_rays == 0) return RSH_OK;
    const uint32_t P = ctx->cfg.packet_size;
    const uint64_t cap = cand_capacity(ctx);
    void *cand = nullptr, *work = nullptr;
    RSH_TRY(ensure(ctx, "cand", cap * 8, &cand));
    RSH_TRY(ensure(ctx, "work", 64, &work));
    uint32_t* w = static_cast<uint32_t*>(work);
    unsigned long long* cc = reinterpret_cast<unsigned long long*>(w + 4);
    TravArgs ta{};
    ta.nodes = nodes;
    hierarchy_capacity(max_rays, P, ta.node_off);
    ta.max_rays = max_rays;
    ta.d_count = d_count;
    ta.packet = P;
    ta.spheres = sc->h.spheres;
    ta.kids = sc->h.kids;
    for (uint32_t l = 0; l < sc->h.levels; ++l) {
        ta.lvl_off[l] = sc->h.level_off[l];
        ta.lvl_size[l] = sc->h.level_size[l];
    }
    ta.levels = sc->h.levels;
    ta.cand = static_cast<unsigned long long*>(cand);
    ta.capacity = cap;
    ta.cand_count = cc;
    ta.work = w;
    ta.ray_level = ctx->cfg.plain_ray_level;
    ta.rays = rays;
    ta.sorted_ids = sorted_ids;
    ta.node_tests = ctx->d_stats + 0;
    ta.err = ctx->d_err;
    IsectArgs ia{};
    ia.spheres = sc->h.spheres;
    ia.kids = sc->h.kids;
    ia.tris = sc->h.tris;
    ia.tri_count = sc->tri_count;
    ia.cluster = sc->h.cluster;
    ia.rays = rays;
    ia.sorted_ids = sorted_ids;
    ia.max_rays = max_rays;
    ia.d_count = d_count;
    ia.packet = P;
    ia.cand = static_cast<const unsigned long long*>(cand);
    ia.cand_count = cc;
    ia.capacity = cap;
    ia.flags = flags;
    ia.hits = hits;
    ia.tri_tests = ctx->d_stats + 1;
    ia.per_ray = ctx->cfg.plain_ray_level > 0 ? 1u : 0u;
    // Passes over a window of work units [start, start + window). Without overflow the first pass covers
    // every unit. After an overflow the window restarts at the first unfinished unit; if a pass made no
    // progress the window shrinks (units of one pass race for the buffer), down to a single unit, which
    // then has the whole buffer to itself.
    const uint32_t units = (((max_rays + P - 1) / P) + 7) / 8;
    uint32_t start = 0, window = units;
    while (start < units) {
        ta.unit_end = (window >= units - start) ? units : start + window;
        uint32_t iw[4] = {start, 0xFFFFFFFFu, 0u, 0u};
        RSH_CUDA(cudaMemcpyAsync(w, iw, sizeof(iw), cudaMemcpyHostToDevice, s));
        RSH_CUDA(cudaMemsetAsync(cc, 0, 8, s));
        int th = stage_begin(ctx, RSH_STAGE_TRAVERSE, s);
        RSH_CUDA(launch_traverse(ta, s));
        stage_end(ctx, th, s);
        th = stage_begin(ctx, RSH_STAGE_INTERSECT, s);
        RSH_CUDA(launch_intersect(ia, any_hit, s));
        stage_end(ctx, th, s);
        RSH_CUDA(cudaMemcpyAsync(ctx->h_pinned, w, 16, cudaMemcpyDeviceToHost, s));
        RSH_CUDA(cudaMemcpyAsync(ctx->h_pinned + 4, cc, 8, cudaMemcpyDeviceToHost, s));
        RSH_CUDA(cudaStreamSynchronize(s));
        const uint32_t resume = ctx->h_pinned[1];
        unsigned long long got = 0;
        std::memcpy(&got, ctx->h_pinned + 4, 8);
        ctx->stats.candidates += got < cap ? got : cap;
        if (resume == 0xFFFFFFFFu) {
            start = ta.unit_end;
            continue;
        }
        ++ctx->overflow_passes;
        if (resume == start) {
            if (window == 1) {
                set_error("the candidates of one work unit exceed the candidate buffer");
                return RSH_ERR_OVERFLOW;
            }
            window = std::max<uint32_t>(1, window / 4);
        }
        start = resume;
    }
    return RSH_OK;
}

rsh_status trace_keyed(rsh_ctx* ctx, const rsh_scene* sc, const rsh_ray* rays, const uint32_t* keys,
                       uint32_t n_slots, uint32_t key_bits, bool any_hit, uint32_t* flags,
                       unsigned long long* hits, uint32_t* counts_out, cudaStream_t s) {
    if (n_slots == 0) return RSH_OK;
    const uint32_t P = ctx->cfg.packet_size;
    void *trimmed, *ckeys, *cbases, *counts, *skeys, *svals, *sorted_keys, *sorted_ids, *nodes, *scr;
    RSH_TRY(ensure(ctx, "trimmed", 4ull * n_slots, &trimmed));
    RSH_TRY(ensure(ctx, "ckeys", 4ull * n_slots + 4, &ckeys));
    RSH_TRY(ensure(ctx, "cbases", 4ull * n_slots + 4, &cbases));
    RSH_TRY(ensure(ctx, "counts", 64, &counts));
    RSH_TRY(ensure(ctx, "skeys", 4ull * n_slots, &skeys));
    RSH_TRY(ensure(ctx, "svals", 4ull * n_slots, &svals));
    RSH_TRY(ensure(ctx, "sorted_keys", 4ull * n_slots, &sorted_keys));
    RSH_TRY(ensure(ctx, "sorted_ids", 4ull * n_slots, &sorted_ids));
    uint32_t off[4];
    const uint32_t cap_nodes = hierarchy_capacity(n_slots, P, off);
    RSH_TRY(ensure(ctx, "nodes", sizeof(rsh_node) * (size_t)cap_nodes, &nodes));
    size_t scr_bytes = compress_scratch_bytes(n_slots);
    scr_bytes = std::max(scr_bytes, sort_scratch_bytes(n_slots, key_bits));
    scr_bytes = std::max(scr_bytes, decompress_scratch_bytes(n_slots));
    RSH_TRY(ensure(ctx, "scratch", scr_bytes, &scr));
    uint32_t* cnt = counts_out ? counts_out : static_cast<uint32_t*>(counts);
    int th = stage_begin(ctx, RSH_STAGE_COMPRESS, s);
    RSH_CUDA(launch_compress(keys, n_slots, static_cast<uint32_t*>(trimmed), static_cast<uint32_t*>(ckeys),
                             static_cast<uint32_t*>(cbases), cnt, scr, ctx->d_err, s));
    stage_end(ctx, th, s);
    if (ctx->cfg.flags & RSH_FLAG_RAH) {
        // ablation: no sort, packets of consecutive trimmed rays (the reference's RAH path)
        th = stage_begin(ctx, RSH_STAGE_BUILD, s);
        RSH_CUDA(launch_build_rsh(rays, static_cast<uint32_t*>(trimmed), n_slots, cnt, P,
                                  static_cast<rsh_node*>(nodes), s));
        stage_end(ctx, th, s);
        return traverse_and_intersect(ctx, sc, static_cast<rsh_node*>(nodes), rays,
                                      static_cast<uint32_t*>(trimmed), n_slots, cnt, any_hit, flags, hits, s);
    }
    th = stage_begin(ctx, RSH_STAGE_SORT, s);
    RSH_CUDA(launch_sort_pairs(static_cast<uint32_t*>(ckeys), nullptr, static_cast<uint32_t*>(skeys),
                               static_cast<uint32_t*>(svals), n_slots, cnt + 1, key_bits, scr, ctx->d_err, s));
    stage_end(ctx, th, s);
    th = stage_begin(ctx, RSH_STAGE_DECOMPRESS, s);
    RSH_CUDA(launch_decompress(static_cast<uint32_t*>(skeys), static_cast<uint32_t*>(svals),
                               static_cast<uint32_t*>(cbases), static_cast<uint32_t*>(trimmed), cnt,
                               n_slots, static_cast<uint32_t*>(sorted_keys),
                               static_cast<uint32_t*>(sorted_ids), scr, ctx->d_err, s));
    stage_end(ctx, th, s);
    th = stage_begin(ctx, RSH_STAGE_BUILD, s);
    RSH_CUDA(launch_build_rsh(rays, static_cast<uint32_t*>(sorted_ids), n_slots, cnt, P,
                              static_cast<rsh_node*>(nodes), s));
    stage_end(ctx, th, s);
    return traverse_and_intersect(ctx, sc, static_cast<rsh_node*>(nodes), rays,
                                  static_cast<uint32_t*>(sorted_ids), n_slots, cnt, any_hit, flags, hits, s);
}

rsh_status trace_ordered(rsh_ctx* ctx, const rsh_scene* sc, const rsh_ray* rays, uint32_t n,
                         bool any_hit, uint32_t* flags, unsigned long long* hits, cudaStream_t s) {
    if (n == 0) return RSH_OK;
    const uint32_t P = ctx->cfg.packet_size;
    uint32_t off[4];
    const uint32_t cap_nodes = hierarchy_capacity(n, P, off);
    void* nodes;
    RSH_TRY(ensure(ctx, "nodes_ordered", sizeof(rsh_node) * (size_t)cap_nodes, &nodes));
    RSH_CUDA(launch_build_rsh(rays, nullptr, n, nullptr, P, static_cast<rsh_node*>(nodes), s));
    return traverse_and_intersect(ctx, sc, static_cast<rsh_node*>(nodes), rays, nullptr, n, nullptr, any_hit,
                                  flags, hits, s);
}

}  // namespace rsh

using namespace rsh;

// =====================================================================================  C ABI
extern "C" {

const char* rsh_last_error_string(void) { return g_last_error.c_str(); }

void rsh_config_default(rsh_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->grid_bits = 4;
    c->dir_log2 = 6;
    c->packet_size = 8;
    c->cluster_size = 6;
    c->epsilon = 0.01f;
    c->hbm_budget = 0;
    c->candidate_capacity = 0;
    c->flags = 0;
    c->reflect_jitter = 0.0f;
    c->seed = 0x5EED0000u;
    c->ray_level = 15;
    c->plain_ray_level = 4;
}

static rsh_status validate_config(const rsh_config* c) {
    if (c->grid_bits < 1 || c->grid_bits > 10) return RSH_ERR_INVALID;
    if (c->dir_log2 < 1 || c->dir_log2 > 6) return RSH_ERR_INVALID;
    if (c->packet_size != 8 && c->packet_size != 16 && c->packet_size != 32) return RSH_ERR_INVALID;
    if (c->cluster_size < 1 || c->cluster_size > 64) return RSH_ERR_INVALID;
    if (!(c->epsilon >= 0.0f)) return RSH_ERR_INVALID;
    if (c->ray_level > 15 || c->plain_ray_level > 15 || c->fused_blocks > 64) return RSH_ERR_INVALID;
    return RSH_OK;
}

rsh_status rsh_create(const rsh_config* cfg, rsh_ctx** out) {
    if (!out) return RSH_ERR_INVALID;
    rsh_config c;
    if (cfg) c = *cfg; else rsh_config_default(&c);
    if (validate_config(&c) != RSH_OK) {
        set_error("invalid configuration");
        return RSH_ERR_INVALID;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    rsh_ctx* ctx = new rsh_ctx();
    ctx->cfg = c;
    ctx->device = dev;
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, dev);
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->budget = c.hbm_budget ? c.hbm_budget : (uint64_t)(0.9 * (double)free_b);
    if ((e = cudaMalloc(&ctx->d_err, 256)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->d_stats, 256)) != cudaSuccess ||
        (e = cudaMallocHost(&ctx->h_pinned, 4096)) != cudaSuccess) {
        rsh_status st = cuda_status(e, "rsh_create");
        rsh_destroy(ctx);
        return st;
    }
    cudaMemset(ctx->d_err, 0, 256);
    cudaMemset(ctx->d_stats, 0, 256);
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    *out = ctx;
    return RSH_OK;
}

rsh_status rsh_destroy(rsh_ctx* ctx) {
    if (!ctx) return RSH_ERR_INVALID;
    cudaDeviceSynchronize();
    batch_release_ctx(ctx);
    for (const cudaEvent_t ev : ctx->tev) cudaEventDestroy(ev);
    for (auto& kv : ctx->bufs) release_buf(ctx, kv.second);
    for (auto& b : ctx->bounce) {
        release_buf(ctx, b.shadow_rays);
        release_buf(ctx, b.shadow_flags);
        release_buf(ctx, b.refl_hits);
        release_buf(ctx, b.surf_pos);
        release_buf(ctx, b.surf_nrm);
    }
    release_buf(ctx, ctx->prim_rays);
    release_buf(ctx, ctx->prim_hits);
    release_buf(ctx, ctx->prim_pix);
    release_buf(ctx, ctx->surf0_pos);
    release_buf(ctx, ctx->surf0_nrm);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->d_stats) cudaFree(ctx->d_stats);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    for (auto& ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    delete ctx;
    return RSH_OK;
}

rsh_status rsh_get_config(const rsh_ctx* ctx, rsh_config* out) {
    if (!ctx || !out) return RSH_ERR_INVALID;
    *out = ctx->cfg;
    return RSH_OK;
}

rsh_status rsh_set_config(rsh_ctx* ctx, const rsh_config* cfg) {
    if (!ctx || !cfg || validate_config(cfg) != RSH_OK) return RSH_ERR_INVALID;
    ctx->cfg = *cfg;
    if (cfg->hbm_budget) ctx->budget = cfg->hbm_budget;
    return RSH_OK;
}

rsh_status rsh_selftest_wait_timeout(rsh_ctx* ctx, uint32_t spin_limit, rsh_stream_t stream) {
    if (!ctx || spin_limit == 0 || spin_limit > (1u << 22)) return RSH_ERR_INVALID;  // at most the kernels' own limit
    // start from a clean error word, so the bit read back below is this test's
    RSH_TRY(rsh_check_device_errors(ctx, stream));
    void* scr = nullptr;
    RSH_TRY(ensure(ctx, "selftest", sort_selftest_scratch_bytes(), &scr));
    RSH_CUDA(sort_selftest_timeout(scr, ctx->d_err, spin_limit, stream));
    return rsh_check_device_errors(ctx, stream);  // RSH_ERR_TIMEOUT: the wait gave up as designed
}

rsh_status rsh_check_device_errors(rsh_ctx* ctx, rsh_stream_t stream) {
    if (!ctx) return RSH_ERR_INVALID;
    uint32_t v = 0;
    RSH_CUDA(cudaMemcpyAsync(&v, ctx->d_err, 4, cudaMemcpyDeviceToHost, stream));
    RSH_CUDA(cudaStreamSynchronize(stream));
    RSH_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, stream));
    if (v & RSH_DEVERR_TIMEOUT) {
        set_error("a device-side look-back wait timed out");
        return RSH_ERR_TIMEOUT;
    }
    if (v & RSH_DEVERR_OVERFLOW) {
        set_error("a device-side buffer overflowed");
        return RSH_ERR_OVERFLOW;
    }
    return RSH_OK;
}

uint64_t rsh_bytes_allocated(const rsh_ctx* ctx) { return ctx ? ctx->allocated : 0; }

rsh_status rsh_malloc(void** ptr, size_t bytes) {
    if (!ptr) return RSH_ERR_INVALID;
    RSH_CUDA(cudaMalloc(ptr, bytes ? bytes : 1));
    return RSH_OK;
}
rsh_status rsh_free(void* ptr) {
    RSH_CUDA(cudaFree(ptr));
    return RSH_OK;
}
rsh_status rsh_malloc_host(void** ptr, size_t bytes) {
    if (!ptr) return RSH_ERR_INVALID;
    RSH_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
    return RSH_OK;
}
rsh_status rsh_free_host(void* ptr) {
    RSH_CUDA(cudaFreeHost(ptr));
    return RSH_OK;
}
rsh_status rsh_memcpy_h2d(void* dst, const void* src, size_t bytes, rsh_stream_t stream) {
    if (bytes == 0) return RSH_OK;
    RSH_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
    return RSH_OK;
}
rsh_status rsh_memcpy_d2h(void* dst, const void* src, size_t bytes, rsh_stream_t stream) {
    if (bytes == 0) return RSH_OK;
    RSH_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream));
    return RSH_OK;
}
rsh_status rsh_memset(void* dst, int value, size_t bytes, rsh_stream_t stream) {
    if (bytes == 0) return RSH_OK;
    RSH_CUDA(cudaMemsetAsync(dst, value, bytes, stream));
    return RSH_OK;
}
rsh_status rsh_stream_create(rsh_stream_t* out) {
    if (!out) return RSH_ERR_INVALID;
    cudaStream_t s;
    RSH_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *out = s;
    return RSH_OK;
}
rsh_status rsh_stream_destroy(rsh_stream_t s) {
    RSH_CUDA(cudaStreamDestroy(s));
    return RSH_OK;
}
rsh_status rsh_stream_synchronize(rsh_stream_t s) {
    RSH_CUDA(cudaStreamSynchronize(s));
    return RSH_OK;
}
rsh_status rsh_device_synchronize(void) {
    RSH_CUDA(cudaDeviceSynchronize());
    return RSH_OK;
}
rsh_status rsh_event_create(void** ev) {
    if (!ev) return RSH_ERR_INVALID;
    cudaEvent_t e;
    RSH_CUDA(cudaEventCreate(&e));
    *ev = e;
    return RSH_OK;
}
rsh_status rsh_event_destroy(void* ev) {
    RSH_CUDA(cudaEventDestroy(static_cast<cudaEvent_t>(ev)));
    return RSH_OK;
}
rsh_status rsh_event_record(void* ev, rsh_stream_t stream) {
    RSH_CUDA(cudaEventRecord(static_cast<cudaEvent_t>(ev), stream));
    return RSH_OK;
}
rsh_status rsh_event_elapsed(void* start, void* stop, float* ms) {
    if (!ms) return RSH_ERR_INVALID;
    RSH_CUDA(cudaEventSynchronize(static_cast<cudaEvent_t>(stop)));
    RSH_CUDA(cudaEventElapsedTime(ms, static_cast<cudaEvent_t>(start), static_cast<cudaEvent_t>(stop)));
    return RSH_OK;
}
int rsh_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
uint64_t rsh_kernel_launches(void) { return g_launches.load(); }

int rsh_sm_count(void) {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
}

rsh_status rsh_device_memory(uint64_t* free_bytes, uint64_t* total_bytes) {
    if (!free_bytes || !total_bytes) return RSH_ERR_INVALID;
    size_t f = 0, t = 0;
    const cudaError_t e = cudaMemGetInfo(&f, &t);
    if (e != cudaSuccess) return cuda_status(e, "cudaMemGetInfo");
    *free_bytes = f;
    *total_bytes = t;
    return RSH_OK;
}

// ------------------------------------------------------------------------------------ hashing
rsh_status rsh_hash_params_make(const float lo[3], const float hi[3], uint32_t grid_bits,
                                uint32_t dir_log2, uint32_t tag_bits, rsh_hash_params* out) {
    if (!lo || !hi || !out) return RSH_ERR_INVALID;
    if (grid_bits < 1 || grid_bits > 10 || dir_log2 < 1 || dir_log2 > 6) return RSH_ERR_INVALID;
    const uint32_t kb = tag_bits + 3 * grid_bits + 2 * dir_log2;
    if (kb > 31) {
        set_error("hash key wider than 31 bits");
        return RSH_ERR_INVALID;
    }
    const float G = (float)(1u << grid_bits);
    for (int i = 0; i < 3; ++i) {
        out->lo[i] = lo[i];
        const float ext = hi[i] - lo[i];
        out->scale[i] = ext > 0.0f ? G / ext : 0.0f;
    }
    out->grid_bits = grid_bits;
    out->dir_log2 = dir_log2;
    out->tag_bits = tag_bits;
    out->key_bits = kb;
    return RSH_OK;
}

// ------------------------------------------------------------------------------------ scenes
rsh_status rsh_scene_upload(rsh_ctx* ctx, const rsh_scene_desc* d, rsh_scene** out) {
    if (!ctx || !d || !out || !d->positions) return RSH_ERR_INVALID;
    if (d->material_count > 0 && !d->materials) return RSH_ERR_INVALID;
    const uint32_t T = d->triangle_count;
    rsh_scene* sc = new rsh_scene();
    sc->owner = ctx;
    sc->tri_count = T;
    // exact bounds and validity
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint64_t v = 0; v < 3ull * T; ++v)
        for (int a = 0; a < 3; ++a) {
            const float x = d->positions[4 * v + a];
            if (!std::isfinite(x)) {
                delete sc;
                set_error("non-finite vertex coordinate");
                return RSH_ERR_INVALID;
            }
            lo[a] = std::min(lo[a], x);
            hi[a] = std::max(hi[a], x);
        }
    if (T == 0)
        for (int a = 0; a < 3; ++a) lo[a] = hi[a] = 0.0f;
    std::memcpy(sc->lo, lo, sizeof(lo));
    std::memcpy(sc->hi, hi, sizeof(hi));
    if (d->material_ids)
        for (uint32_t t = 0; t < T; ++t)
            if (d->material_count && d->material_ids[t] >= d->material_count) {
                delete sc;
                set_error("material id out of range");
                return RSH_ERR_INVALID;
            }
    const size_t need = T * (48ull * 2 + 48 + 4 + 4) + 64ull * d->material_count + 4096;
    if (ctx->allocated + need > ctx->budget) {
        delete sc;
        set_error("HBM budget exceeded by the scene");
        return RSH_ERR_OOM;
    }
    cudaError_t e;
    std::vector<float> nrm_host;
    const float* nrm = d->normals;
    if (!nrm) {  // flat normals
        nrm_host.resize(12ull * T);
        for (uint32_t t = 0; t < T; ++t) {
            const float* p = d->positions + 12ull * t;
            const float e1[3] = {p[4] - p[0], p[5] - p[1], p[6] - p[2]};
            const float e2[3] = {p[8] - p[0], p[9] - p[1], p[10] - p[2]};
            float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                          e1[0] * e2[1] - e1[1] * e2[0]};
            const float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int a = 0; a < 3; ++a) n[a] = l > 0 ? n[a] / l : 0.0f;
            for (int v = 0; v < 3; ++v)
                for (int a = 0; a < 3; ++a) nrm_host[12ull * t + 4 * v + a] = n[a];
        }
        nrm = nrm_host.data();
    }
    rsh_material defmat = {{0.8f, 0.8f, 0.8f, 0.5f}, {0.5f, 0.5f, 0.5f, 32.0f}};
    const rsh_material* mats = d->material_count ? d->materials : &defmat;
    sc->material_count = d->material_count ? d->material_count : 1;
    const size_t tri_bytes = 48ull * (T ? T : 1);
    if ((e = cudaMalloc(&sc->pos, tri_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&sc->nrm, tri_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&sc->mat, 4ull * (T ? T : 1))) != cudaSuccess ||
        (e = cudaMalloc(&sc->obj, 4ull * (T ? T : 1))) != cudaSuccess ||
        (e = cudaMalloc(&sc->materials, sizeof(rsh_material) * sc->material_count)) != cudaSuccess) {
        rsh_scene_destroy(ctx, sc);
        return cuda_status(e, "rsh_scene_upload");
    }
    cudaStream_t s = nullptr;
    cudaMemcpy(sc->pos, d->positions, 48ull * T, cudaMemcpyHostToDevice);
    cudaMemcpy(sc->nrm, nrm, 48ull * T, cudaMemcpyHostToDevice);
    if (d->material_ids) cudaMemcpy(sc->mat, d->material_ids, 4ull * T, cudaMemcpyHostToDevice);
    else cudaMemset(sc->mat, 0, 4ull * (T ? T : 1));
    if (d->object_ids) {
        cudaMemcpy(sc->obj, d->object_ids, 4ull * T, cudaMemcpyHostToDevice);
        for (uint32_t t = 0; t < T; ++t) sc->object_count = std::max(sc->object_count, d->object_ids[t] + 1);
    } else {
        cudaMemset(sc->obj, 0, 4ull * (T ? T : 1));
    }
    cudaMemcpy(sc->materials, mats, sizeof(rsh_material) * sc->material_count, cudaMemcpyHostToDevice);
    void* scr = nullptr;
    const size_t scr_bytes = objh_scratch_bytes(T ? T : 1);
    if ((e = cudaMalloc(&scr, scr_bytes)) != cudaSuccess) {
        rsh_scene_destroy(ctx, sc);
        return cuda_status(e, "rsh_scene_upload scratch");
    }
    e = build_object_hierarchy(sc->pos, T, ctx->cfg.cluster_size, lo, hi, sc->h, scr, scr_bytes,
                               ctx->d_err, s);
    cudaFree(scr);
    if (e != cudaSuccess) {
        rsh_scene_destroy(ctx, sc);
        return cuda_status(e, "build_object_hierarchy");
    }
    uint32_t total = 0;
    for (uint32_t l = 0; l < sc->h.levels; ++l) total += sc->h.level_size[l];
    // + the single-ray box tree: 2 float4 per slot (at most 2T + 8), its traversal records (224 B per node,
    // at most T + 4 nodes) and its own copy of the triangles
    sc->bytes = tri_bytes * 3 + 8ull * T + 48ull * total + 32ull * (2ull * T + 8) + 224ull * (T + 4) + 48ull * T +
                sizeof(rsh_material) * sc->material_count;
    ctx->allocated += sc->bytes;
    *out = sc;
    return RSH_OK;
}

rsh_status rsh_scene_destroy(rsh_ctx* ctx, rsh_scene* sc) {
    if (!sc) return RSH_ERR_INVALID;
    cudaDeviceSynchronize();
    if (sc->pos) cudaFree(sc->pos);
    if (sc->nrm) cudaFree(sc->nrm);
    if (sc->mat) cudaFree(sc->mat);
    if (sc->obj) cudaFree(sc->obj);
    if (sc->pos_rest) cudaFree(sc->pos_rest);
    if (sc->nrm_rest) cudaFree(sc->nrm_rest);
    if (sc->materials) cudaFree(sc->materials);
    if (sc->h.spheres) cudaFree(sc->h.spheres);
    if (sc->h.kids) cudaFree(sc->h.kids);
    if (sc->h.tris) cudaFree(sc->h.tris);
    if (sc->h.order) cudaFree(sc->h.order);
    if (sc->h.boxes) cudaFree(sc->h.boxes);
    if (sc->h.wboxes) cudaFree(sc->h.wboxes);
    if (sc->h.wtris) cudaFree(sc->h.wtris);
    if (sc->h.wnodes) cudaFree(sc->h.wnodes);
    if (ctx && ctx->allocated >= sc->bytes) ctx->allocated -= sc->bytes;
    delete sc;
    return RSH_OK;
}

rsh_status rsh_build_object_hierarchy(rsh_ctx* ctx, rsh_scene* sc, rsh_stream_t stream) {
    if (!ctx || !sc || sc->owner != ctx) return RSH_ERR_INVALID;
    const uint32_t T = sc->tri_count;
    cudaStream_t s = stream;
    // exact bounds of the current positions (the hash and the Morton codes are built over them)
    if (T) {
        void* bscr = nullptr;
        RSH_TRY(ensure(ctx, "bounds", bounds_scratch_bytes(), &bscr));
        float* b6 = static_cast<float*>(bscr) + 6 * 608;
        RSH_CUDA(launch_bounds(sc->pos, T, bscr, b6, s));
        float hb[6];
        RSH_CUDA(cudaMemcpyAsync(hb, b6, sizeof hb, cudaMemcpyDeviceToHost, s));
        RSH_CUDA(cudaStreamSynchronize(s));
        for (int a = 0; a < 3; ++a) {
            if (!std::isfinite(hb[a]) || !std::isfinite(hb[3 + a])) {
                set_error("non-finite vertex coordinate after the transform");
                return RSH_ERR_INVALID;
            }
            sc->lo[a] = hb[a];
            sc->hi[a] = hb[3 + a];
        }
    }
    RSH_CUDA(cudaStreamSynchronize(s));
    for (void* p : {(void*)sc->h.spheres, (void*)sc->h.kids, (void*)sc->h.tris, (void*)sc->h.order,
                    (void*)sc->h.boxes, (void*)sc->h.wboxes, (void*)sc->h.wtris, (void*)sc->h.wnodes})
        if (p) cudaFree(p);
    sc->h = ObjHierarchy();
    void* scr = nullptr;
    const size_t scr_bytes = objh_scratch_bytes(T ? T : 1);
    RSH_CUDA(cudaMalloc(&scr, scr_bytes));
    const cudaError_t e = build_object_hierarchy(sc->pos, T, ctx->cfg.cluster_size, sc->lo, sc->hi, sc->h, scr,
                                                 scr_bytes, ctx->d_err, s);
    cudaFree(scr);
    if (e != cudaSuccess) return cuda_status(e, "rsh_build_object_hierarchy");
    return RSH_OK;
}

rsh_status rsh_scene_set_transforms(rsh_ctx* ctx, rsh_scene* sc, const float* model_matrices,
                                    const float* normal_matrices, uint32_t object_count, rsh_stream_t stream) {
    if (!ctx || !sc || sc->owner != ctx || !model_matrices || object_count < sc->object_count) return RSH_ERR_INVALID;
    for (uint64_t i = 0; i < 16ull * object_count; ++i)
        if (!std::isfinite(model_matrices[i]) || (normal_matrices && !std::isfinite(normal_matrices[i]))) {
            set_error("non-finite transform");
            return RSH_ERR_INVALID;
        }
    const uint32_t T = sc->tri_count;
    cudaStream_t s = stream;
    const size_t tri_bytes = 48ull * (T ? T : 1);
    if (!sc->pos_rest) {  // the uploaded pose becomes the rest pose
        RSH_CUDA(cudaMalloc(&sc->pos_rest, tri_bytes));
        RSH_CUDA(cudaMalloc(&sc->nrm_rest, tri_bytes));
        RSH_CUDA(cudaMemcpyAsync(sc->pos_rest, sc->pos, tri_bytes, cudaMemcpyDeviceToDevice, s));
        RSH_CUDA(cudaMemcpyAsync(sc->nrm_rest, sc->nrm, tri_bytes, cudaMemcpyDeviceToDevice, s));
    }
    void* mbuf = nullptr;
    RSH_TRY(ensure(ctx, "transforms", 2ull * 64 * object_count, &mbuf));
    float* dm = static_cast<float*>(mbuf);
    float* dn = dm + 16ull * object_count;
    RSH_CUDA(cudaMemcpyAsync(dm, model_matrices, 64ull * object_count, cudaMemcpyHostToDevice, s));
    if (normal_matrices)
        RSH_CUDA(cudaMemcpyAsync(dn, normal_matrices, 64ull * object_count, cudaMemcpyHostToDevice, s));
    RSH_CUDA(launch_transform(sc->pos_rest, sc->nrm_rest, sc->obj, T, object_count, dm,
                              normal_matrices ? dn : nullptr, sc->pos, sc->nrm, s));
    return rsh_build_object_hierarchy(ctx, sc, stream);
}

rsh_status rsh_scene_bounds(const rsh_scene* sc, float lo[3], float hi[3]) {
    if (!sc || !lo || !hi) return RSH_ERR_INVALID;
    for (int i = 0; i < 3; ++i) {
        lo[i] = sc->lo[i];
        hi[i] = sc->hi[i];
    }
    return RSH_OK;
}
uint32_t rsh_scene_triangle_count(const rsh_scene* sc) { return sc ? sc->tri_count : 0; }
uint32_t rsh_scene_levels(const rsh_scene* sc) { return sc ? sc->h.levels : 0; }
uint32_t rsh_scene_box_tree(const rsh_scene* sc, uint32_t* root, float* boxes, float* tris) {
    if (!sc) return 0;
    if (root) *root = sc->h.wroot;
    if (boxes && sc->h.wslots &&
        cudaMemcpy(boxes, sc->h.wboxes, 32ull * sc->h.wslots, cudaMemcpyDeviceToHost) != cudaSuccess)
        return 0;
    if (tris && sc->tri_count &&
        cudaMemcpy(tris, sc->h.wtris, 48ull * sc->tri_count, cudaMemcpyDeviceToHost) != cudaSuccess)
        return 0;
    return sc->h.wslots;
}
uint32_t rsh_scene_level_size(const rsh_scene* sc, uint32_t level) {
    return (sc && level < sc->h.levels) ? sc->h.level_size[level] : 0;
}
rsh_status rsh_scene_get_level(const rsh_scene* sc, uint32_t level, rsh_object_node* out) {
    if (!sc || !out || level >= sc->h.levels) return RSH_ERR_INVALID;
    const uint32_t n = sc->h.level_size[level];
    std::vector<float4> sp(n);
    RSH_CUDA(cudaMemcpy(sp.data(), sc->h.spheres + sc->h.level_off[level], 16ull * n, cudaMemcpyDeviceToHost));
    // child ranges of every level up to this one; a node's triangles = those of its children's range
    const uint32_t nk = sc->h.level_off[level] + sc->h.level_size[level] + level + 1;
    std::vector<uint32_t> kids(nk);
    RSH_CUDA(cudaMemcpy(kids.data(), sc->h.kids, 4ull * nk, cudaMemcpyDeviceToHost));
    std::vector<uint32_t> tstart(kids.begin(), kids.begin() + sc->h.level_size[0] + 1);
    for (uint32_t l = 1; l <= level; ++l) {
        const uint32_t* k = kids.data() + sc->h.level_off[l] + l;
        std::vector<uint32_t> ts(sc->h.level_size[l] + 1);
        for (uint32_t j = 0; j <= sc->h.level_size[l]; ++j) ts[j] = tstart[k[j]];
        tstart.swap(ts);
    }
    const uint32_t* kl = kids.data() + sc->h.level_off[level] + level;
    for (uint32_t j = 0; j < n; ++j) {
        rsh_object_node& o = out[j];
        o.c[0] = sp[j].x;
        o.c[1] = sp[j].y;
        o.c[2] = sp[j].z;
        o.radius = sp[j].w;
        o.first_tri = tstart[j];
        o.tri_count = tstart[j + 1] - tstart[j];
        o.first_child = level == 0 ? 0u : kl[j];
        o.child_count = level == 0 ? 0u : kl[j + 1] - kl[j];
    }
    return RSH_OK;
}
rsh_status rsh_scene_get_order(const rsh_scene* sc, uint32_t* out) {
    if (!sc || !out) return RSH_ERR_INVALID;
    if (sc->tri_count) RSH_CUDA(cudaMemcpy(out, sc->h.order, 4ull * sc->tri_count, cudaMemcpyDeviceToHost));
    return RSH_OK;
}
const void* rsh_scene_device_triangles(const rsh_scene* sc) { return sc ? sc->h.tris : nullptr; }

rsh_status rsh_lights_set(rsh_ctx* ctx, const rsh_light* lights, uint32_t count) {
    if (!ctx || count > 8 || (count && !lights)) return RSH_ERR_INVALID;
    for (uint32_t i = 0; i < count; ++i) ctx->lights[i] = lights[i];
    ctx->light_count = count;
    return RSH_OK;
}
rsh_status rsh_camera_set(rsh_ctx* ctx, const rsh_camera* cam) {
    if (!ctx || !cam) return RSH_ERR_INVALID;
    ctx->cam = *cam;
    ctx->cam_set = true;
    return RSH_OK;
}
rsh_status rsh_camera_look_at(const float eye[3], const float target[3], const float up[3],
                              float fov_degrees, uint32_t width, uint32_t height, rsh_camera* out) {
    if (!eye || !target || !up || !out || width == 0 || height == 0) return RSH_ERR_INVALID;
    double dir[3] = {target[0] - (double)eye[0], target[1] - (double)eye[1], target[2] - (double)eye[2]};
    const double dist = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (!(dist > 0)) return RSH_ERR_INVALID;
    const double theta = 0.5 * fov_degrees * 3.14159265358979323846 / 180.0;
    const double half_h = 2.0 * dist * std::tan(theta);
    const double half_w = half_h * (double)width / (double)height;
    double f[3] = {dir[0] / dist, dir[1] / dist, dir[2] / dist};
    auto cross = [](const double* a, const double* b, double* r) {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto normalize = [](double* v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (l > 0) for (int i = 0; i < 3; ++i) v[i] /= l;
    };
    double u0[3] = {up[0], up[1], up[2]}, r[3], u[3];
    cross(f, u0, r);
    normalize(r);
    cross(r, f, u);
    normalize(u);
    for (int i = 0; i < 3; ++i) {
        out->eye[i] = eye[i];
        out->direction[i] = (float)(f[i] * dist);
        out->right[i] = (float)(r[i] * half_w);
        out->up[i] = (float)(u[i] * half_h);
    }
    return RSH_OK;
}

// ------------------------------------------------------------------------------------ stages
static CameraP to_camp(const rsh_camera& c) {
    CameraP p;
    for (int i = 0; i < 3; ++i) {
        p.eye[i] = c.eye[i];
        p.dir[i] = c.direction[i];
        p.right[i] = c.right[i];
        p.up[i] = c.up[i];
    }
    return p;
}

rsh_status rsh_raygen_primary(const rsh_camera* cam, uint32_t width, uint32_t height, rsh_ray* rays,
                              uint32_t* pixel_of_ray, rsh_stream_t stream) {
    if (!cam || !rays) return RSH_ERR_INVALID;
    RSH_CUDA(launch_raygen_primary(to_camp(*cam), width, height, rays, pixel_of_ray, stream));
    return RSH_OK;
}

rsh_status rsh_raygen_shadow(const float* surface_pos, const float* surface_nrm, uint32_t width,
                             uint32_t height, const rsh_light* lights_host, uint32_t light_count,
                             float epsilon, const rsh_hash_params* hp, rsh_ray* rays, uint32_t* keys,
                             rsh_stream_t stream) {
    if (!surface_pos || !surface_nrm || !lights_host || !hp || !rays || !keys) return RSH_ERR_INVALID;
    if (light_count == 0 || light_count > 8) return RSH_ERR_INVALID;
    if (light_count > (1u << hp->tag_bits)) return RSH_ERR_INVALID;
    LightsP lp{};
    lp.count = light_count;
    lp.samples = 1;
    for (uint32_t l = 0; l < light_count; ++l)
        for (int i = 0; i < 3; ++i) lp.pos[l][i] = lights_host[l].position[i];
    RSH_CUDA(launch_raygen_shadow(reinterpret_cast<const float4*>(surface_pos),
                                  reinterpret_cast<const float4*>(surface_nrm), width, height, lp, epsilon,
                                  to_hashp(*hp), rays, keys, stream));
    return RSH_OK;
}

rsh_status rsh_raygen_soft_shadow(const float* surface_pos, const float* surface_nrm, uint32_t width,
                                  uint32_t height, const rsh_light* lights_host, uint32_t light_count,
                                  float epsilon, const rsh_hash_params* hp, rsh_ray* rays, uint32_t* keys,
                                  rsh_stream_t stream) {
    if (!surface_pos || !surface_nrm || !lights_host || !hp || !rays || !keys) return RSH_ERR_INVALID;
    if (light_count == 0 || light_count > 8) return RSH_ERR_INVALID;
    if (16ull * light_count > (1ull << hp->tag_bits)) return RSH_ERR_INVALID;
    if ((uint64_t)width * height * light_count * 16 >= (1ull << 31)) return RSH_ERR_INVALID;
    LightsP lp{};
    lp.count = light_count;
    lp.samples = 16;
    for (uint32_t l = 0; l < light_count; ++l)
        for (int i = 0; i < 3; ++i) lp.pos[l][i] = lights_host[l].position[i];
    RSH_CUDA(launch_raygen_shadow(reinterpret_cast<const float4*>(surface_pos),
                                  reinterpret_cast<const float4*>(surface_nrm), width, height, lp, epsilon,
                                  to_hashp(*hp), rays, keys, stream));
    return RSH_OK;
}

rsh_status rsh_raygen_refract(const float* surface_pos, const float* surface_nrm, const rsh_ray* prev_rays,
                              const float eye[3], uint32_t width, uint32_t height, float epsilon, float eta,
                              const rsh_hash_params* hp, rsh_ray* rays, uint32_t* keys, rsh_stream_t stream) {
    if (!surface_pos || !surface_nrm || !hp || !rays || !keys || (!prev_rays && !eye)) return RSH_ERR_INVALID;
    if (!(eta > 0.0f)) return RSH_ERR_INVALID;
    const float zero[3] = {0, 0, 0};
    RSH_CUDA(launch_raygen_refract(reinterpret_cast<const float4*>(surface_pos),
                                   reinterpret_cast<const float4*>(surface_nrm), prev_rays, eye ? eye : zero, width,
                                   height, epsilon, eta, to_hashp(*hp), rays, keys, stream));
    return RSH_OK;
}

rsh_status rsh_raygen_reflect(const float* surface_pos, const float* surface_nrm, const rsh_ray* prev_rays,
                              const float eye[3], uint32_t width, uint32_t height, float epsilon,
                              float jitter, uint32_t seed, uint32_t bounce, const rsh_hash_params* hp,
                              rsh_ray* rays, uint32_t* keys, rsh_stream_t stream) {
    if (!surface_pos || !surface_nrm || !hp || !rays || !keys || (!prev_rays && !eye)) return RSH_ERR_INVALID;
    const float zero[3] = {0, 0, 0};
    RSH_CUDA(launch_raygen_reflect(reinterpret_cast<const float4*>(surface_pos),
                                   reinterpret_cast<const float4*>(surface_nrm), prev_rays, eye ? eye : zero,
                                   width, height, epsilon, jitter, seed, bounce, to_hashp(*hp), rays, keys,
                                   stream));
    return RSH_OK;
}

rsh_status rsh_hash(const rsh_ray* rays, uint32_t n, const rsh_hash_params* hp, uint32_t tag,
                    uint32_t* keys, rsh_stream_t stream) {
    if (!rays || !hp || !keys) return RSH_ERR_INVALID;
    if (hp->tag_bits < 32 && tag >= (1u << hp->tag_bits) && !(hp->tag_bits == 0 && tag == 0)) return RSH_ERR_INVALID;
    RSH_CUDA(launch_hash(rays, n, to_hashp(*hp), tag, keys, stream));
    return RSH_OK;
}

rsh_status rsh_compress(rsh_ctx* ctx, const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                        uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* chunk_sizes,
                        uint32_t* counts, rsh_stream_t stream) {
    if (!ctx || !keys || !trimmed_ids || !chunk_keys || !chunk_bases || !counts) return RSH_ERR_INVALID;
    void* scr;
    RSH_TRY(ensure(ctx, "scratch", compress_scratch_bytes(n_slots), &scr));
    RSH_CUDA(launch_compress(keys, n_slots, trimmed_ids, chunk_keys, chunk_bases, counts, scr, ctx->d_err, stream));
    if (chunk_sizes) RSH_CUDA(launch_chunk_sizes(chunk_bases, counts, n_slots, chunk_sizes, stream));
    return RSH_OK;
}

rsh_status rsh_sort_pairs(rsh_ctx* ctx, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                          uint32_t* vals_out, uint32_t n_max, const uint32_t* d_count, uint32_t key_bits,
                          rsh_stream_t stream) {
    if (!ctx || !keys_in || !keys_out || !vals_out || key_bits > 32) return RSH_ERR_INVALID;
    if (keys_in == keys_out || (vals_in && vals_in == vals_out)) {
        set_error("rsh_sort_pairs: input and output must not alias");
        return RSH_ERR_INVALID;
    }
    void* scr;
    RSH_TRY(ensure(ctx, "scratch", sort_scratch_bytes(n_max, key_bits), &scr));
    RSH_CUDA(launch_sort_pairs(keys_in, vals_in, keys_out, vals_out, n_max, d_count, key_bits, scr, ctx->d_err,
                               stream));
    return RSH_OK;
}

rsh_status rsh_decompress(rsh_ctx* ctx, const uint32_t* sorted_chunk_keys, const uint32_t* sorted_chunk_vals,
                          const uint32_t* chunk_bases, const uint32_t* trimmed_ids, const uint32_t* counts,
                          uint32_t max_rays, uint32_t* sorted_keys, uint32_t* sorted_ids, rsh_stream_t stream) {
    if (!ctx || !sorted_chunk_vals || !chunk_bases || !trimmed_ids || !counts || !sorted_ids)
        return RSH_ERR_INVALID;
    void* scr;
    RSH_TRY(ensure(ctx, "scratch", decompress_scratch_bytes(max_rays), &scr));
    RSH_CUDA(launch_decompress(sorted_chunk_keys, sorted_chunk_vals, chunk_bases, trimmed_ids, counts, max_rays,
                               sorted_keys, sorted_ids, scr, ctx->d_err, stream));
    return RSH_OK;
}

uint32_t rsh_hierarchy_capacity(uint32_t max_rays, uint32_t packet_size, uint32_t offsets[4]) {
    uint32_t tmp[4];
    return hierarchy_capacity(max_rays, packet_size ? packet_size : 8, offsets ? offsets : tmp);
}

rsh_status rsh_build_rsh(const rsh_ray* rays, const uint32_t* sorted_ids, uint32_t max_rays,
                         const uint32_t* d_count, uint32_t packet_size, rsh_node* nodes, rsh_stream_t stream) {
    if (!rays || !nodes) return RSH_ERR_INVALID;
    if (packet_size != 8 && packet_size != 16 && packet_size != 32) return RSH_ERR_INVALID;
    RSH_CUDA(launch_build_rsh(rays, sorted_ids, max_rays, d_count, packet_size, nodes, stream));
    return RSH_OK;
}

rsh_status rsh_traverse(rsh_ctx* ctx, const rsh_scene* sc, const rsh_node* nodes, uint32_t max_rays,
                        const uint32_t* d_count, uint32_t packet_size, uint64_t* candidates, uint64_t capacity,
                        uint64_t* d_cand_count, rsh_stream_t stream) {
    if (!ctx || !sc || !nodes || !candidates || !d_cand_count) return RSH_ERR_INVALID;
    if (packet_size != 8 && packet_size != 16 && packet_size != 32) return RSH_ERR_INVALID;
    void* work;
    RSH_TRY(ensure(ctx, "work_stage", 64, &work));
    uint32_t* w = static_cast<uint32_t*>(work);
    const uint32_t iw[4] = {0u, 0xFFFFFFFFu, 0u, 0u};
    RSH_CUDA(cudaMemcpyAsync(w, iw, sizeof(iw), cudaMemcpyHostToDevice, stream));
    RSH_CUDA(cudaMemsetAsync(d_cand_count, 0, 8, stream));
    if (sc->tri_count == 0 || max_rays == 0) return RSH_OK;
    TravArgs ta{};
    ta.nodes = nodes;
    hierarchy_capacity(max_rays, packet_size, ta.node_off);
    ta.max_rays = max_rays;
    ta.d_count = d_count;
    ta.packet = packet_size;
    ta.spheres = sc->h.spheres;
    ta.kids = sc->h.kids;
    for (uint32_t l = 0; l < sc->h.levels; ++l) {
        ta.lvl_off[l] = sc->h.level_off[l];
        ta.lvl_size[l] = sc->h.level_size[l];
    }
    ta.levels = sc->h.levels;
    ta.cand = reinterpret_cast<unsigned long long*>(candidates);
    ta.capacity = capacity;
    ta.cand_count = reinterpret_cast<unsigned long long*>(d_cand_count);
    ta.work = w;
    ta.unit_end = 0xFFFFFFFFu;
    ta.node_tests = ctx->d_stats;
    ta.err = ctx->d_err;
    RSH_CUDA(launch_traverse(ta, stream));
    uint32_t hw[4];
    RSH_CUDA(cudaMemcpyAsync(hw, w, sizeof(hw), cudaMemcpyDeviceToHost, stream));
    RSH_CUDA(cudaStreamSynchronize(stream));
    if (hw[1] != 0xFFFFFFFFu) {
        set_error("rsh_traverse: candidate buffer full");
        return RSH_ERR_OVERFLOW;
    }
    return RSH_OK;
}

static rsh_status isect_stage(const rsh_scene* sc, const rsh_ray* rays, const uint32_t* sorted_ids,
                              uint32_t max_rays, const uint32_t* d_count, uint32_t packet_size,
                              const uint64_t* candidates, const uint64_t* d_cand_count, bool any,
                              uint32_t* flags, uint64_t* hits, rsh_stream_t stream) {
    if (!sc || !rays || !candidates || !d_cand_count) return RSH_ERR_INVALID;
    if (packet_size != 8 && packet_size != 16 && packet_size != 32) return RSH_ERR_INVALID;
    if (sc->tri_count == 0 || max_rays == 0) return RSH_OK;
    IsectArgs ia{};
    ia.spheres = sc->h.spheres;
    ia.kids = sc->h.kids;
    ia.tris = sc->h.tris;
    ia.tri_count = sc->tri_count;
    ia.cluster = sc->h.cluster;
    ia.rays = rays;
    ia.sorted_ids = sorted_ids;
    ia.max_rays = max_rays;
    ia.d_count = d_count;
    ia.packet = packet_size;
    ia.cand = reinterpret_cast<const unsigned long long*>(candidates);
    ia.cand_count = reinterpret_cast<const unsigned long long*>(d_cand_count);
    ia.capacity = ~0ull;
    ia.flags = flags;
    ia.hits = reinterpret_cast<unsigned long long*>(hits);
    ia.tri_tests = nullptr;
    RSH_CUDA(launch_intersect(ia, any, stream));
    return RSH_OK;
}

rsh_status rsh_intersect_any(const rsh_scene* sc, const rsh_ray* rays, const uint32_t* sorted_ids,
                             uint32_t max_rays, const uint32_t* d_count, uint32_t packet_size,
                             const uint64_t* candidates, const uint64_t* d_cand_count, uint32_t* flags,
                             rsh_stream_t stream) {
    if (!flags) return RSH_ERR_INVALID;
    return isect_stage(sc, rays, sorted_ids, max_rays, d_count, packet_size, candidates, d_cand_count, true,
                       flags, nullptr, stream);
}

rsh_status rsh_intersect_closest(const rsh_scene* sc, const rsh_ray* rays, const uint32_t* sorted_ids,
                                 uint32_t max_rays, const uint32_t* d_count, uint32_t packet_size,
                                 const uint64_t* candidates, const uint64_t* d_cand_count, uint64_t* hits,
                                 rsh_stream_t stream) {
    if (!hits) return RSH_ERR_INVALID;
    return isect_stage(sc, rays, sorted_ids, max_rays, d_count, packet_size, candidates, d_cand_count, false,
                       nullptr, hits, stream);
}

rsh_status rsh_resolve_hits(const rsh_scene* sc, const rsh_ray* rays, const uint64_t* hits,
                            const uint32_t* pixel_of_ray, uint32_t n, float* surface_pos, float* surface_nrm,
                            rsh_stream_t stream) {
    if (!sc || !rays || !hits || !surface_pos || !surface_nrm) return RSH_ERR_INVALID;
    RSH_CUDA(launch_resolve(sc->pos, sc->nrm, sc->mat, rays, reinterpret_cast<const unsigned long long*>(hits),
                            pixel_of_ray, n, reinterpret_cast<float4*>(surface_pos),
                            reinterpret_cast<float4*>(surface_nrm), stream));
    return RSH_OK;
}

rsh_status rsh_trace_rays(rsh_ctx* ctx, const rsh_scene* sc, const rsh_ray* rays, uint32_t n, int any_hit,
                          uint64_t* hits, uint32_t* flags, rsh_stream_t stream) {
    if (!ctx || !sc || !rays) return RSH_ERR_INVALID;
    if (any_hit ? !flags : !hits) return RSH_ERR_INVALID;
    if (n == 0) return RSH_OK;
    HashP hp;
    RSH_TRY(make_hash_params(sc, ctx->cfg, 0, hp));
    void* keys;
    RSH_TRY(ensure(ctx, "keys", 4ull * n, &keys));
    if (any_hit) RSH_CUDA(cudaMemsetAsync(flags, 0, 4ull * n, stream));
    else RSH_CUDA(launch_fill_u64(reinterpret_cast<unsigned long long*>(hits), RSH_HIT_NONE, n, stream));
    RSH_CUDA(launch_hash(rays, n, hp, 0, static_cast<uint32_t*>(keys), stream));
    return trace_keyed(ctx, sc, rays, static_cast<uint32_t*>(keys), n, hp.key_bits, any_hit != 0, flags,
                       reinterpret_cast<unsigned long long*>(hits), nullptr, stream);
}

// ------------------------------------------------------------------------------------ frame
rsh_status rsh_render_frame(rsh_ctx* ctx, const rsh_scene* sc, uint32_t W, uint32_t H, uint32_t depth,
                            uint32_t* rgba_out, rsh_stream_t stream) {
    if (!ctx || !sc || W == 0 || H == 0 || !ctx->cam_set) return RSH_ERR_INVALID;
    if (ctx->light_count == 0 && depth > 0) return RSH_ERR_INVALID;
    // soft shadows: 16 shadow rays per light (RayTracer.cu:1550-1603), shaded by :1680-1696
    const uint32_t S = (ctx->cfg.flags & RSH_FLAG_SOFT_SHADOWS) ? 16u : 1u;
    if ((uint64_t)W * H * (ctx->light_count ? ctx->light_count : 1) * S >= (1ull << 31)) return RSH_ERR_INVALID;
    cudaStream_t s = stream;
    const uint32_t L = ctx->light_count;
    const uint32_t npix = W * H;
    const bool fused = (ctx->cfg.flags & RSH_FLAG_FUSED) != 0;
    ctx->fw = W;
    ctx->fh = H;
    ctx->fdepth = depth;
    ctx->flights = L * S;  // shadow slots per pixel
    ctx->last_stream = s;
    ctx->overflow_passes = 0;
    ctx->tev_used = 0;
    ctx->tmarks.clear();
    std::memset(&ctx->stats, 0, sizeof(ctx->stats));
    RSH_CUDA(cudaMemsetAsync(ctx->d_stats, 0, 64, s));
    const uint32_t LS = L * S;  // light samples per pixel
    uint32_t lbits = 0;
    while ((1u << lbits) < LS) ++lbits;
    HashP hp_s, hp_r;
    RSH_TRY(make_hash_params(sc, ctx->cfg, 0, hp_r));
    // the batched form re-keys every segment itself (segment tag instead of the light tag)
    if (fused) hp_s = hp_r;
    else RSH_TRY(make_hash_params(sc, ctx->cfg, lbits, hp_s));
    if (ctx->bounce.size() < depth) ctx->bounce.resize(depth);

    // primary rays (tile order) -> surface buffer 0
    const uint32_t tx = (W + 7) / 8, ty = (H + 7) / 8, np = tx * ty * 64;
    RSH_TRY(ensure_buf(ctx, ctx->prim_rays, sizeof(rsh_ray) * (size_t)np));
    RSH_TRY(ensure_buf(ctx, ctx->prim_hits, 8ull * np));
    RSH_TRY(ensure_buf(ctx, ctx->prim_pix, 4ull * np));
    RSH_TRY(ensure_buf(ctx, ctx->surf0_pos, 16ull * npix));
    RSH_TRY(ensure_buf(ctx, ctx->surf0_nrm, 16ull * npix));
    void *accum, *keys;
    RSH_TRY(ensure(ctx, "accum", 16ull * npix, &accum));
    RSH_TRY(ensure(ctx, "keys", 4ull * npix * (LS ? LS : 1), &keys));
    for (uint32_t b = 0; b < depth; ++b) {
        BounceBufs& bb = ctx->bounce[b];
        // shadow slots, then the reflection slots right behind them: the batched form traces both
        // segments from this one array without gathering them
        RSH_TRY(ensure_buf(ctx, bb.shadow_rays, sizeof(rsh_ray) * (size_t)npix * (LS + 1)));
        RSH_TRY(ensure_buf(ctx, bb.shadow_flags, 4ull * npix * LS));
        RSH_TRY(ensure_buf(ctx, bb.refl_hits, 8ull * npix));
        RSH_TRY(ensure_buf(ctx, bb.surf_pos, 16ull * npix));
        RSH_TRY(ensure_buf(ctx, bb.surf_nrm, 16ull * npix));
    }
    void* cnt_acc;
    RSH_TRY(ensure(ctx, "frame_counts", 8ull * 2 * (depth + 1), &cnt_acc));
    uint32_t* fc = static_cast<uint32_t*>(cnt_acc);
    RSH_CUDA(cudaMemsetAsync(fc, 0, 8ull * 2 * (depth + 1), s));
    RSH_CUDA(cudaEventRecord(ctx->ev[0], s));
    int th = stage_begin(ctx, RSH_STAGE_PRIMARY, s);
    rsh_ray* prays = static_cast<rsh_ray*>(ctx->prim_rays.ptr);
    unsigned long long* phits = static_cast<unsigned long long*>(ctx->prim_hits.ptr);
    uint32_t* ppix = static_cast<uint32_t*>(ctx->prim_pix.ptr);
    RSH_CUDA(launch_raygen_primary(to_camp(ctx->cam), W, H, prays, ppix, s));
    if (fused) {
        rsh_batch_segment seg{sc, prays, np, 0, reinterpret_cast<uint64_t*>(phits), nullptr};
        ctx->timers_paused = true;  // the primary window times the whole primary pass
        const rsh_status pst = batch_trace_ordered(ctx, seg, s);  // tile order is already coherent
        ctx->timers_paused = false;
        RSH_TRY(pst);
    } else {
        RSH_CUDA(launch_fill_u64(phits, RSH_HIT_NONE, np, s));
        ctx->timers_paused = true;
        const rsh_status pst = trace_ordered(ctx, sc, prays, np, false, nullptr, phits, s);
        ctx->timers_paused = false;
        RSH_TRY(pst);
    }
    RSH_CUDA(launch_resolve(sc->pos, sc->nrm, sc->mat, prays, phits, ppix, np,
                            static_cast<float4*>(ctx->surf0_pos.ptr), static_cast<float4*>(ctx->surf0_nrm.ptr), s));
    stage_end(ctx, th, s);
    RSH_CUDA(cudaMemsetAsync(ctx->d_stats, 0, 64, s));  // the frame's test counters cover secondary rays
    RSH_CUDA(cudaEventRecord(ctx->ev[1], s));  // secondary window starts

    const float4* spos = static_cast<const float4*>(ctx->surf0_pos.ptr);
    const float4* snrm = static_cast<const float4*>(ctx->surf0_nrm.ptr);
    const rsh_ray* incident = nullptr;
    LightsP lp{};
    lp.count = L;
    lp.samples = S;
    for (uint32_t l = 0; l < L; ++l)
        for (int i = 0; i < 3; ++i) lp.pos[l][i] = ctx->lights[l].position[i];
    ShadeArgs sa{};
    sa.materials = sc->materials;
    sa.material_count = sc->material_count;
    sa.accum = static_cast<float4*>(accum);
    sa.w = W;
    sa.h = H;
    sa.lights = L;
    sa.samples = S;
    for (uint32_t l = 0; l < L; ++l) sa.light[l] = ctx->lights[l];
    for (int i = 0; i < 3; ++i) sa.eye[i] = ctx->cam.eye[i];
    for (uint32_t b = 0; b < depth; ++b) {
        BounceBufs& bb = ctx->bounce[b];
        rsh_ray* srays = static_cast<rsh_ray*>(bb.shadow_rays.ptr);
        uint32_t* sflags = static_cast<uint32_t*>(bb.shadow_flags.ptr);
        rsh_ray* rrays = srays + (size_t)npix * LS;
        unsigned long long* rhits = static_cast<unsigned long long*>(bb.refl_hits.ptr);
        if (fused) {
            // both batches of the bounce in one batched call: 2 segments, one persistent launch; ray
            // generation writes the batch's keys, segment counts and prefilled results itself
            rsh_batch_segment segs[2] = {
                {sc, srays, npix * LS, 1, nullptr, sflags},
                {sc, rrays, npix, 0, reinterpret_cast<uint64_t*>(rhits), nullptr}};
            BatchKeyLayout kl;
            RSH_TRY(batch_key_layout(ctx, segs, 2, kl));
            BatchKeyOut bs, br;
            bs.keys = kl.keys + kl.start[0];
            bs.tag = 0u;
            bs.drop = kl.hash_drop;
            bs.hp = kl.hp[0];
            bs.count = kl.seg_cnt;
            bs.flags = sflags;
            br.keys = kl.keys + kl.start[1];
            br.tag = 1u << kl.tag_shift;
            br.drop = kl.hash_drop;
            br.hp = kl.hp[1];
            br.count = kl.seg_cnt + 1;
            br.hits = rhits;
            th = stage_begin(ctx, RSH_STAGE_RAYGEN, s);
            RSH_CUDA(cudaMemsetAsync(kl.seg_cnt, 0, 8, s));
            RSH_CUDA(launch_raygen_shadow(spos, snrm, W, H, lp, ctx->cfg.epsilon, hp_s, srays, nullptr, s, bs));
            RSH_CUDA(launch_raygen_reflect(spos, snrm, incident, ctx->cam.eye, W, H, ctx->cfg.epsilon,
                                           ctx->cfg.reflect_jitter, ctx->cfg.seed, b, hp_r, rrays, nullptr, s, br));
            stage_end(ctx, th, s);
            RSH_TRY(batch_trace(ctx, segs, 2, s, false, true));
            const uint32_t* seg_cnt = static_cast<const uint32_t*>(ctx->bufs["b_seg_cnt"].ptr);
            const uint32_t* bcnt = static_cast<const uint32_t*>(ctx->bufs["b_counts"].ptr);
            RSH_CUDA(cudaMemcpyAsync(fc + 4 * b, seg_cnt, 4, cudaMemcpyDeviceToDevice, s));
            RSH_CUDA(cudaMemcpyAsync(fc + 4 * b + 2, seg_cnt + 1, 4, cudaMemcpyDeviceToDevice, s));
            RSH_CUDA(cudaMemcpyAsync(fc + 4 * b + 1, bcnt + 1, 4, cudaMemcpyDeviceToDevice, s));
        } else {
            // shadow batch
            th = stage_begin(ctx, RSH_STAGE_RAYGEN, s);
            RSH_CUDA(launch_raygen_shadow(spos, snrm, W, H, lp, ctx->cfg.epsilon, hp_s, srays,
                                          static_cast<uint32_t*>(keys), s));
            RSH_CUDA(cudaMemsetAsync(sflags, 0, 4ull * npix * LS, s));
            stage_end(ctx, th, s);
            RSH_TRY(trace_keyed(ctx, sc, srays, static_cast<uint32_t*>(keys), npix * LS, hp_s.key_bits, true, sflags,
                                nullptr, fc + 4 * b, s));
            // reflection batch
            th = stage_begin(ctx, RSH_STAGE_RAYGEN, s);
            RSH_CUDA(launch_raygen_reflect(spos, snrm, incident, ctx->cam.eye, W, H, ctx->cfg.epsilon,
                                           ctx->cfg.reflect_jitter, ctx->cfg.seed, b, hp_r, rrays,
                                           static_cast<uint32_t*>(keys), s));
            RSH_CUDA(launch_fill_u64(rhits, RSH_HIT_NONE, npix, s));
            stage_end(ctx, th, s);
            RSH_TRY(trace_keyed(ctx, sc, rrays, static_cast<uint32_t*>(keys), npix, hp_r.key_bits, false, nullptr,
                                rhits, fc + 4 * b + 2, s));
        }
        // shade this bounce's surface, then resolve the reflection hits into the next surface
        th = stage_begin(ctx, RSH_STAGE_SHADE, s);
        if (rgba_out) {
            sa.spos = spos;
            sa.snrm = snrm;
            sa.shadow = sflags;
            sa.bounce = b;
            sa.incident = incident;
            RSH_CUDA(launch_shade(sa, s));
        }
        RSH_CUDA(launch_resolve(sc->pos, sc->nrm, sc->mat, rrays, rhits, nullptr, npix,
                                static_cast<float4*>(bb.surf_pos.ptr), static_cast<float4*>(bb.surf_nrm.ptr), s));
        stage_end(ctx, th, s);
        spos = static_cast<const float4*>(bb.surf_pos.ptr);
        snrm = static_cast<const float4*>(bb.surf_nrm.ptr);
        incident = rrays;
    }
    RSH_CUDA(cudaEventRecord(ctx->ev[2], s));  // secondary window ends
    if (rgba_out) {
        th = stage_begin(ctx, RSH_STAGE_SHADE, s);
        sa.spos = spos;
        sa.snrm = snrm;
        sa.shadow = nullptr;
        sa.bounce = depth;
        sa.incident = incident;
        RSH_CUDA(launch_shade(sa, s));
        RSH_CUDA(launch_pack_rgba(static_cast<float4*>(accum), npix, rgba_out, s));
        stage_end(ctx, th, s);
    }
    RSH_CUDA(cudaEventRecord(ctx->ev[3], s));
    // counters (async; read by rsh_frame_stats_get)
    RSH_CUDA(cudaMemcpyAsync(ctx->h_pinned + 16, fc, 8ull * 2 * (depth + 1), cudaMemcpyDeviceToHost, s));
    RSH_CUDA(cudaMemcpyAsync(ctx->h_pinned + 256, ctx->d_stats, 64, cudaMemcpyDeviceToHost, s));
    ctx->stats.primary_rays = (uint64_t)W * H;
    return RSH_OK;
}

rsh_status rsh_test_counters(rsh_ctx* ctx, uint64_t* node_tests, uint64_t* tri_tests, int32_t reset,
                             rsh_stream_t stream) {
    if (!ctx) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(stream));
    unsigned long long d[2] = {0, 0};
    RSH_CUDA(cudaMemcpy(d, ctx->d_stats, 16, cudaMemcpyDeviceToHost));
    if (node_tests) *node_tests = d[0];
    if (tri_tests) *tri_tests = d[1];
    if (reset) RSH_CUDA(cudaMemset(ctx->d_stats, 0, 16));
    return RSH_OK;
}

rsh_status rsh_frame_stats_get(rsh_ctx* ctx, rsh_frame_stats* out) {
    if (!ctx || !out) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(ctx->last_stream));
    rsh_frame_stats st = ctx->stats;
    st.shadow_rays = st.reflection_rays = st.chunks = 0;
    const uint32_t* fc = ctx->h_pinned + 16;
    for (uint32_t b = 0; b < ctx->fdepth; ++b) {
        st.shadow_rays += fc[4 * b];
        st.chunks += fc[4 * b + 1] + fc[4 * b + 3];
        st.reflection_rays += fc[4 * b + 2];
    }
    unsigned long long d[8];
    std::memcpy(d, ctx->h_pinned + 256, 64);
    st.node_tests = d[0];
    st.tri_tests = d[1];
    cudaEventElapsedTime(&st.secondary_ms, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&st.frame_ms, ctx->ev[0], ctx->ev[3]);
    for (float& v : st.stage_ms) v = 0.0f;
    for (const auto& m : ctx->tmarks) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ctx->tev[m.second], ctx->tev[m.second + 1]) == cudaSuccess && m.first < 12)
            st.stage_ms[m.first] += ms;
    }
    cudaGetLastError();
    st.overflow_passes = ctx->overflow_passes;
    *out = st;
    return RSH_OK;
}

rsh_status rsh_frame_hits(rsh_ctx* ctx, int32_t bounce, uint64_t* host_out) {
    if (!ctx || !host_out) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(ctx->last_stream));
    const size_t npix = (size_t)ctx->fw * ctx->fh;
    if (bounce < 0) {
        // primary hits in pixel order
        const uint32_t tx = (ctx->fw + 7) / 8, ty = (ctx->fh + 7) / 8, np = tx * ty * 64;
        std::vector<unsigned long long> h(np);
        std::vector<uint32_t> pix(np);
        RSH_CUDA(cudaMemcpy(h.data(), ctx->prim_hits.ptr, 8ull * np, cudaMemcpyDeviceToHost));
        RSH_CUDA(cudaMemcpy(pix.data(), ctx->prim_pix.ptr, 4ull * np, cudaMemcpyDeviceToHost));
        for (uint32_t k = 0; k < np; ++k)
            if (pix[k] != 0xFFFFFFFFu) host_out[pix[k]] = h[k];
        return RSH_OK;
    }
    if ((uint32_t)bounce >= ctx->fdepth) return RSH_ERR_INVALID;
    RSH_CUDA(cudaMemcpy(host_out, ctx->bounce[bounce].refl_hits.ptr, 8 * npix, cudaMemcpyDeviceToHost));
    return RSH_OK;
}

rsh_status rsh_frame_shadow(rsh_ctx* ctx, int32_t bounce, uint32_t* host_out) {
    if (!ctx || !host_out || bounce < 0 || (uint32_t)bounce >= ctx->fdepth) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(ctx->last_stream));
    const size_t n = (size_t)ctx->fw * ctx->fh * ctx->flights;
    RSH_CUDA(cudaMemcpy(host_out, ctx->bounce[bounce].shadow_flags.ptr, 4 * n, cudaMemcpyDeviceToHost));
    return RSH_OK;
}

rsh_status rsh_frame_rays(rsh_ctx* ctx, int32_t bounce, int32_t shadow, rsh_ray* host_out) {
    if (!ctx || !host_out) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(ctx->last_stream));
    const size_t npix = (size_t)ctx->fw * ctx->fh;
    if (bounce < 0) {
        const uint32_t tx = (ctx->fw + 7) / 8, ty = (ctx->fh + 7) / 8, np = tx * ty * 64;
        RSH_CUDA(cudaMemcpy(host_out, ctx->prim_rays.ptr, sizeof(rsh_ray) * (size_t)np, cudaMemcpyDeviceToHost));
        return RSH_OK;
    }
    if ((uint32_t)bounce >= ctx->fdepth) return RSH_ERR_INVALID;
    const BounceBufs& bb = ctx->bounce[bounce];
    if (shadow)
        RSH_CUDA(cudaMemcpy(host_out, bb.shadow_rays.ptr, sizeof(rsh_ray) * npix * ctx->flights,
                            cudaMemcpyDeviceToHost));
    else
        RSH_CUDA(cudaMemcpy(host_out, static_cast<rsh_ray*>(bb.shadow_rays.ptr) + npix * ctx->flights,
                            sizeof(rsh_ray) * npix, cudaMemcpyDeviceToHost));
    return RSH_OK;
}

rsh_status rsh_frame_surface(rsh_ctx* ctx, int32_t bounce, float* host_pos, float* host_nrm) {
    if (!ctx || !host_pos || !host_nrm) return RSH_ERR_INVALID;
    RSH_CUDA(cudaStreamSynchronize(ctx->last_stream));
    const size_t npix = (size_t)ctx->fw * ctx->fh;
    const void *p, *n;
    if (bounce < 0) {
        p = ctx->surf0_pos.ptr;
        n = ctx->surf0_nrm.ptr;
    } else {
        if ((uint32_t)bounce >= ctx->fdepth) return RSH_ERR_INVALID;
        p = ctx->bounce[bounce].surf_pos.ptr;
        n = ctx->bounce[bounce].surf_nrm.ptr;
    }
    RSH_CUDA(cudaMemcpy(host_pos, p, 16 * npix, cudaMemcpyDeviceToHost));
    RSH_CUDA(cudaMemcpy(host_nrm, n, 16 * npix, cudaMemcpyDeviceToHost));
    return RSH_OK;
}

}  // extern "C"
