// Trim + compress without any allocation: the scratch of the compress kernels (a 4-word summary and a
// 4-word prefix per tile) lives in a fixed static device array, so the call needs no context and never
// calls cudaMalloc/cudaFree.
//
// Who needs this: host applications that own every byte of device memory and forbid a plug-in from
// allocating (pre-partitioned memory on a shared or real-time device), and loops that allocate once at
// start-up and then only launch work. They pass keys, outputs and counts they allocated themselves; this
// file supplies the small scratch.
#include <mutex>

#include "common.cuh"
#include "engine.h"

namespace {

// Largest slot count one call accepts (16,777,216 = e.g. 1920 x 1080 pixels x 8 lights).
constexpr uint32_t kMaxSlots = 1u << 24;
// Room for compress tiles of 3072 slots or more at 9 words per tile; the current kernels use 4096-slot
// tiles at 8 words per tile (compress_scratch_bytes), checked against the array below on every call.
constexpr uint32_t kTileSlots = 3072u;
constexpr uint32_t kMaxTiles = (kMaxSlots + kTileSlots - 1) / kTileSlots + 1;
constexpr uint32_t kScratchWords = 4u + 9u * kMaxTiles;   // 49,171 words = 196,684 bytes

// Shared by every call on a device and kept until the process exits; calls that overlap on the GPU
// (two streams at once) would race on it.
static __device__ __align__(256) uint32_t g_compress_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

}  // namespace

extern "C" rsh_status rsh_compress_noalloc(const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                                           uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* chunk_sizes,
                                           uint32_t* counts, rsh_stream_t stream) {
    if (!keys || !trimmed_ids || !chunk_keys || !chunk_bases || !counts) return RSH_ERR_INVALID;
    if (n_slots > kMaxSlots) {
        rsh::set_error("rsh_compress_noalloc: n_slots exceeds the static scratch limit of 16777216 slots");
        return RSH_ERR_INVALID;
    }
    if (rsh::compress_scratch_bytes(n_slots) > sizeof(g_compress_scratch)) {
        rsh::set_error("rsh_compress_noalloc: static scratch too small for n_slots");
        return RSH_ERR_INVALID;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return rsh::cuda_status(e, "rsh_compress_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return RSH_ERR_INVALID;
    void* scratch = nullptr;
    {
        // once per device, with that device current: the device address of the static array (the
        // array's name in host code is only a host-side stand-in, not a device address)
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_compress_scratch);
            if (e != cudaSuccess) return rsh::cuda_status(e, "rsh_compress_noalloc: cudaGetSymbolAddress");
            g_scratch_addr[dev] = p;
        }
        scratch = g_scratch_addr[dev];
    }
    // nothing in the scratch has to start at zero: every word is written before it is read, within the
    // call, on `stream`

    e = rsh::launch_compress(keys, n_slots, trimmed_ids, chunk_keys, chunk_bases, counts, scratch, nullptr,
                             stream);
    if (e != cudaSuccess) return rsh::cuda_status(e, "rsh_compress_noalloc");
    if (chunk_sizes) {
        e = rsh::launch_chunk_sizes(chunk_bases, counts, n_slots, chunk_sizes, stream);
        if (e != cudaSuccess) return rsh::cuda_status(e, "rsh_compress_noalloc: sizes");
    }
    return RSH_OK;
}
