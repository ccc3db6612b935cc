// Internal engine state shared by the C-ABI translation units (engine.cu, batch.cu, server.cpp).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rsh.h"
#include "kernels.h"

namespace rsh {

void set_error(const std::string& msg);
rsh_status cuda_status(cudaError_t e, const char* where);

#define RSH_CUDA(call)                                                       \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return ::rsh::cuda_status(_e, #call);         \
    } while (0)
#define RSH_TRY(call)                              \
    do {                                           \
        rsh_status _s = (call);                    \
        if (_s != RSH_OK) return _s;               \
    } while (0)

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace rsh

struct rsh_scene {
    rsh_ctx* owner = nullptr;
    uint32_t tri_count = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    float4* pos = nullptr;       // original order, 3 per triangle
    float4* nrm = nullptr;       // original order, 3 per triangle
    uint32_t* mat = nullptr;     // per triangle
    uint32_t* obj = nullptr;     // object id per triangle (transforms)
    uint32_t object_count = 1;
    float4* pos_rest = nullptr;  // rest pose for rsh_scene_set_transforms (kept from the first call on)
    float4* nrm_rest = nullptr;
    rsh_material* materials = nullptr;
    uint32_t material_count = 0;
    rsh::ObjHierarchy h;
    size_t bytes = 0;
    rsh_scene_tuning tune{RSH_TUNE_DEFAULT, RSH_TUNE_DEFAULT, RSH_TUNE_DEFAULT};  // batched form only
};

struct BounceBufs {
    rsh::DevBuf shadow_rays, shadow_flags, refl_hits, surf_pos, surf_nrm;  // shadow_rays: then the reflection rays
};

struct rsh_ctx {
    rsh_config cfg{};
    int device = 0;
    int sms = 152;
    uint64_t budget = 0;
    uint64_t allocated = 0;
    std::map<std::string, rsh::DevBuf> bufs;
    uint32_t* d_err = nullptr;
    unsigned long long* d_stats = nullptr;   // [0] node tests [1] tri tests [2] candidates [3..] spare
    uint32_t* h_pinned = nullptr;            // small pinned readback area
    rsh_light lights[8]{};
    uint32_t light_count = 0;
    rsh_camera cam{};
    bool cam_set = false;
    // frame state
    uint32_t fw = 0, fh = 0, fdepth = 0, flights = 0;  // flights: shadow slots per pixel (lights x samples)
    std::vector<BounceBufs> bounce;
    rsh::DevBuf prim_rays, prim_hits, prim_pix, surf0_pos, surf0_nrm;
    rsh_frame_stats stats{};
    rsh_frame_stats batch_stats{};
    cudaEvent_t ev[16] = {};
    cudaStream_t last_stream = nullptr;
    std::vector<uint32_t> batch_counts_host;
    uint32_t overflow_passes = 0;
    // per-stage CUDA events (RSH_FLAG_STAGE_TIMERS): pool and the (stage, start event) pairs of a frame
    std::vector<cudaEvent_t> tev;
    std::vector<std::pair<int, uint32_t>> tmarks;
    uint32_t tev_used = 0;
    bool timers_paused = false;  // stages inside an already-timed window record no marks of their own
};

namespace rsh {

rsh_status ensure(rsh_ctx* ctx, const char* name, size_t bytes, void** out);
// Stage timers: begin returns a handle (or -1 when timers are off); end records the closing event.
int stage_begin(rsh_ctx* ctx, int stage, cudaStream_t s);
void stage_end(rsh_ctx* ctx, int handle, cudaStream_t s);
rsh_status ensure_buf(rsh_ctx* ctx, DevBuf& b, size_t bytes);
void release_buf(rsh_ctx* ctx, DevBuf& b);
rsh_status make_hash_params(const rsh_scene* sc, const rsh_config& cfg, uint32_t tag_bits, HashP& out);
void batch_release_ctx(const rsh_ctx* ctx);
// rsh_batch_trace without resetting the stage timers (used inside a fused frame, which also keeps its
// node / triangle test counters running: reset_stats false).
// prekeyed: the segments' keys, ray counts and prefilled results were already written where
// batch_key_layout says (by the frame's ray generation), so the batch does not read the rays to hash them.
rsh_status batch_trace(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count, cudaStream_t stream,
                       bool reset_stats, bool prekeyed = false);
// Where ray generation writes a batched call's keys itself: segment s's keys at keys + start[s], key =
// s << tag_shift | (hash with hp[s] >> hash_drop) or RSH_KEY_NONE; its ray count into seg_cnt[s] (zeroed
// by the caller first). For at most 2 segments whose rays lie back to back in one array.
struct BatchKeyLayout {
    uint32_t* keys = nullptr;
    uint32_t* seg_cnt = nullptr;
    uint32_t tag_shift = 0, hash_drop = 0;
    uint32_t start[2] = {0, 0};
    HashP hp[2]{};
};
rsh_status batch_key_layout(rsh_ctx* ctx, const rsh_batch_segment* segments, uint32_t count, BatchKeyLayout& out);
// One segment of rays already in a coherent order, traced in that order (rays-only kernel); adds to the
// test counters.
rsh_status batch_trace_ordered(rsh_ctx* ctx, const rsh_batch_segment& seg, cudaStream_t stream);

// One secondary batch through compress -> sort -> decompress -> build -> traverse -> intersect.
// keys: per slot (RSH_KEY_NONE = no ray); rays indexed by slot. Output flags/hits indexed by slot
// (caller initialises). Accumulates counters into ctx->d_stats; counts_out (device, 2 words) gets
// (rays, chunks) if non-null.
rsh_status trace_keyed(rsh_ctx* ctx, const rsh_scene* sc, const rsh_ray* rays, const uint32_t* keys,
                       uint32_t n_slots, uint32_t key_bits, bool any_hit, uint32_t* flags,
                       unsigned long long* hits, uint32_t* counts_out, cudaStream_t s);
// Rays already in traversal order (no hash/sort), e.g. primary rays in tile order.
rsh_status trace_ordered(rsh_ctx* ctx, const rsh_scene* sc, const rsh_ray* rays, uint32_t n,
                         bool any_hit, uint32_t* flags, unsigned long long* hits, cudaStream_t s);

}  // namespace rsh
