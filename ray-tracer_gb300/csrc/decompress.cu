// Decompression of sorted chunks into the sorted ray permutation.
//
// Reference: RayDecompressionWrapper (RayTracer.cu:2411-2467): CreateSortedRaySkeleton (:993-1010,
// skeleton[x] = size[sortedValue[x]]) -> cub ExclusiveSum -> CreateSortedRays (:1012-1059), where one
// thread copies a whole chunk serially (load-imbalanced; the largest sort-stage cost in the thesis
// timings). Here:
//  1. exclusive scan of the sorted chunk sizes -> off[x], reduce-then-scan (k_dc_reduce: one sum per
//     2048-chunk tile; k_dc_tscan: one CTA scans the tile sums; k_dc_write: per tile, the chunk
//     offsets); every chunk also records itself as the first chunk of each 2048-output expand tile
//     that starts inside it (tile_chunk[m]);
//  2. k_dc_expand: every CTA owns 2048 consecutive OUTPUT rays, reads its chunk range from tile_chunk,
//     stages those chunks' offsets/bases/keys in shared memory, and each thread binary-searches its
//     ray's chunk there: work per CTA is fixed whatever the chunk sizes.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr int DS_THREADS = 256;
constexpr int DS_ITEMS = 8;
constexpr int DS_TILE = DS_THREADS * DS_ITEMS;  // chunks per scan tile
constexpr int DE_THREADS = 256;
constexpr int DE_ITEMS = 8;
constexpr uint32_t DE_TILE = DE_THREADS * DE_ITEMS;  // output rays per expand CTA
}  // namespace

// block-wide exclusive prefix of each thread's sum; *total (all threads) = the tile's sum
RSH_DEV uint32_t block_excl(uint32_t tsum, uint32_t* s_warp, uint32_t* total) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t inc = tsum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= (uint32_t)d) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t r = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; ++w) {
            const uint32_t v = s_warp[w];
            s_warp[w] = r;
            r += v;
        }
        s_warp[32] = r;
    }
    __syncthreads();
    *total = s_warp[32];
    return s_warp[warp] + inc - tsum;
}

// Gathers each sorted chunk's base and size once (the only random reads of the chunk table) into
// sorted order, and sums the tile's sizes.
__global__ void __launch_bounds__(DS_THREADS)
k_dc_reduce(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ bases,
            const uint32_t* __restrict__ counts, uint32_t max_chunks, uint32_t* __restrict__ tsum,
            uint32_t* __restrict__ sbase, uint32_t* __restrict__ ssize) {
    __shared__ uint32_t s_warp[33];
    const uint32_t C = counts[1] < max_chunks ? counts[1] : max_chunks;
    if (blockIdx.x * DS_TILE >= C) return;  // whole CTA: tiles past the chunk count are never read
    uint32_t tsum_t = 0;
    for (uint32_t i = 0; i < DS_ITEMS; ++i) {  // x strided by the block: coalesced
        const uint32_t x = blockIdx.x * DS_TILE + i * DS_THREADS + threadIdx.x;
        if (x < C) {
            const uint32_t c = __ldg(vals + x);
            uint32_t b = 0, v = 0;
            if (c < C) {
                b = __ldg(bases + c);
                v = __ldg(bases + c + 1) - b;
            }
            sbase[x] = b;
            ssize[x] = v;
            tsum_t += v;
        }
    }
    uint32_t tot;
    block_excl(tsum_t, s_warp, &tot);
    if (threadIdx.x == 0) tsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024)
k_dc_tscan(const uint32_t* __restrict__ tsum, const uint32_t* __restrict__ counts, uint32_t max_chunks,
           uint32_t* __restrict__ tpre) {
    __shared__ uint32_t s_warp[33];
    const uint32_t C = counts[1] < max_chunks ? counts[1] : max_chunks;
    const uint32_t tiles = (C + DS_TILE - 1) / DS_TILE;
    const uint32_t per = (tiles + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(b + per, tiles);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += __ldg(tsum + i);
    uint32_t tot;
    uint32_t run = block_excl(s, s_warp, &tot);
    for (uint32_t i = b; i < e; ++i) {
        tpre[i] = run;
        run += __ldg(tsum + i);
    }
}

__global__ void __launch_bounds__(DS_THREADS)
k_dc_write(const uint32_t* __restrict__ ssize, const uint32_t* __restrict__ counts, uint32_t max_chunks,
           const uint32_t* __restrict__ tpre, uint32_t* __restrict__ off, uint32_t* __restrict__ tile_chunk,
           uint32_t mcap) {
    __shared__ uint32_t s_warp[33];
    const uint32_t C = counts[1] < max_chunks ? counts[1] : max_chunks;
    const uint32_t x0 = blockIdx.x * DS_TILE + threadIdx.x * DS_ITEMS;
    if (blockIdx.x * DS_TILE >= C) return;
    uint32_t sz[DS_ITEMS];
    uint32_t ts = 0;
#pragma unroll
    for (int i = 0; i < DS_ITEMS; ++i) {
        sz[i] = (x0 + i < C) ? __ldg(ssize + x0 + i) : 0u;
        ts += sz[i];
    }
    uint32_t tot;
    uint32_t run = __ldg(tpre + blockIdx.x) + block_excl(ts, s_warp, &tot);
#pragma unroll
    for (int i = 0; i < DS_ITEMS; ++i) {
        const uint32_t x = x0 + i;
        if (x < C) {
            off[x] = run;
            // expand tiles whose first output lies in this chunk (sizes are >= 1)
            if (sz[i] > 0u)
                for (uint32_t m = (run + DE_TILE - 1u) / DE_TILE; m <= (run + sz[i] - 1u) / DE_TILE && m < mcap; ++m)
                    tile_chunk[m] = x;
        }
        run += sz[i];
    }
}

__global__ void __launch_bounds__(DE_THREADS)
k_dc_expand(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ sbase,
            const uint32_t* __restrict__ trimmed,
            const uint32_t* __restrict__ counts, uint32_t max_rays, const uint32_t* __restrict__ off,
            const uint32_t* __restrict__ tile_chunk, uint32_t* __restrict__ sorted_keys,
            uint32_t* __restrict__ sorted_ids, PaddedOut po) {
    __shared__ uint32_t s_off[DE_TILE + 1];
    __shared__ uint32_t s_base[DE_TILE + 1];
    __shared__ uint32_t s_key[DE_TILE + 1];
    const uint32_t R = counts[0] < max_rays ? counts[0] : max_rays;
    const uint32_t C = counts[1];
    const uint32_t k0 = blockIdx.x * DE_TILE;
    if (k0 >= R || C == 0) return;
    const uint32_t k1 = (k0 + DE_TILE < R ? k0 + DE_TILE : R) - 1;  // last output of the tile
    // chunks x0..x1 cover outputs k0..k1: x0 holds k0, and the chunk holding the next tile's first
    // output is at or after the one holding k1 (one extra chunk may be staged)
    const uint32_t ntiles = (R + DE_TILE - 1) / DE_TILE;
    const uint32_t x0 = __ldg(tile_chunk + blockIdx.x);
    uint32_t x1 = (blockIdx.x + 1 < ntiles) ? __ldg(tile_chunk + blockIdx.x + 1) : C - 1;
    if (x1 >= C) x1 = C - 1;
    if (x1 < x0) x1 = x0;
    const uint32_t m = (x1 - x0 + 1 < DE_TILE + 1) ? x1 - x0 + 1 : DE_TILE + 1;
    for (uint32_t i = threadIdx.x; i < m; i += DE_THREADS) {
        const uint32_t x = x0 + i;
        s_off[i] = __ldg(off + x);
        s_base[i] = __ldg(sbase + x);
        s_key[i] = skeys ? __ldg(skeys + x) : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < DE_ITEMS; ++it) {
        const uint32_t k = k0 + it * DE_THREADS + threadIdx.x;
        if (k > k1) break;
        uint32_t lo = 0, hi = m;  // last staged chunk with off <= k
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_off[mid] <= k) lo = mid; else hi = mid;
        }
        const uint32_t src = s_base[lo] + (k - s_off[lo]);
        const uint32_t id = src < R ? __ldg(trimmed + src) : 0u;
        if (po.padded) {
            const uint32_t q = k + __ldg(po.seg_delta + (s_key[lo] >> po.tag_shift));
            if (q < po.max_padded) po.padded[q] = id;
        } else {
            sorted_ids[k] = id;
        }
        if (sorted_keys) sorted_keys[k] = s_key[lo];
    }
}

size_t decompress_scratch_bytes(uint32_t max_chunks) {
    const size_t tiles = (max_chunks + DS_TILE - 1) / DS_TILE + 1;
    const size_t etiles = (max_chunks + DE_TILE - 1) / DE_TILE + 1;
    return 64 + tiles * 8 + (size_t)max_chunks * 12 + etiles * 4 + 512;
}

cudaError_t launch_decompress(const uint32_t* sorted_chunk_keys, const uint32_t* sorted_chunk_vals,
                              const uint32_t* chunk_bases, const uint32_t* trimmed_ids,
                              const uint32_t* counts, uint32_t max_rays, uint32_t* sorted_keys,
                              uint32_t* sorted_ids, void* scratch, uint32_t* err, cudaStream_t s,
                              const PaddedOut* padded_out) {
    (void)err;  // no step of this form waits on another CTA
    if (max_rays == 0) return cudaSuccess;
    const uint32_t max_chunks = max_rays;
    const size_t tiles = (max_chunks + DS_TILE - 1) / DS_TILE + 1;
    char* b = static_cast<char*>(scratch);
    uint32_t* tsum = reinterpret_cast<uint32_t*>(b + 64);
    uint32_t* tpre = tsum + tiles;
    uint32_t* off = reinterpret_cast<uint32_t*>(b + 64 + tiles * 8);
    uint32_t* sbase = off + max_chunks;   // sorted chunk bases and sizes
    uint32_t* ssize = sbase + max_chunks;
    uint32_t* tile_chunk = ssize + max_chunks;
    const uint32_t mcap = (uint32_t)((max_chunks + DE_TILE - 1) / DE_TILE + 1);
    const uint32_t grid = (uint32_t)(tiles - 1 > 0 ? tiles - 1 : 1);
    k_dc_reduce<<<grid, DS_THREADS, 0, s>>>(sorted_chunk_vals, chunk_bases, counts, max_chunks, tsum, sbase, ssize);
    note_launch();
    k_dc_tscan<<<1, 1024, 0, s>>>(tsum, counts, max_chunks, tpre);
    note_launch();
    k_dc_write<<<grid, DS_THREADS, 0, s>>>(ssize, counts, max_chunks, tpre, off, tile_chunk, mcap);
    note_launch();
    k_dc_expand<<<(max_rays + DE_TILE - 1) / DE_TILE, DE_THREADS, 0, s>>>(
        sorted_chunk_keys, sbase, trimmed_ids, counts, max_rays, off, tile_chunk, sorted_keys, sorted_ids,
        padded_out ? *padded_out : PaddedOut{nullptr, 0u, 0u, nullptr});
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
