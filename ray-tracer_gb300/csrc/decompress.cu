// Decompression of sorted chunks into the sorted ray permutation.
//
// Reference: RayDecompressionWrapper (RayTracer.cu:2411-2467): CreateSortedRaySkeleton (:993-1010,
// skeleton[x] = size[sortedValue[x]]) -> cub ExclusiveSum -> CreateSortedRays (:1012-1059), where one
// thread copies a whole chunk serially (load-imbalanced; the largest sort-stage cost in the thesis
// timings). Here:
//  1. k_dc_scan: single-pass exclusive scan of the sorted chunk sizes (decoupled look-back on 64-bit
//     flag|value words) -> off[x];
//  2. k_dc_expand: every CTA owns 2048 consecutive OUTPUT rays, locates its chunk range by binary
//     search, stages those chunks' offsets/bases/keys in shared memory, and each thread binary-searches
//     its ray's chunk there: work per CTA is fixed whatever the chunk sizes.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr int DS_THREADS = 256;
constexpr int DS_ITEMS = 8;
constexpr int DS_TILE = DS_THREADS * DS_ITEMS;  // chunks per scan tile
constexpr int DE_THREADS = 256;
constexpr int DE_ITEMS = 8;
constexpr int DE_TILE = DE_THREADS * DE_ITEMS;  // output rays per expand CTA
constexpr unsigned long long F_AGG = 1ull << 62;
constexpr unsigned long long F_PRE = 2ull << 62;
constexpr unsigned long long V_MASK = (1ull << 62) - 1ull;
}  // namespace

__global__ void __launch_bounds__(DS_THREADS)
k_dc_scan(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ bases,
          const uint32_t* __restrict__ counts, uint32_t max_chunks, uint32_t* __restrict__ off,
          unsigned long long* __restrict__ status, uint32_t* __restrict__ ticket, uint32_t* err) {
    __shared__ uint32_t s_warp[DS_THREADS / 32];
    __shared__ uint32_t s_tile, s_excl, s_tot;
    const uint32_t C = counts[1] < max_chunks ? counts[1] : max_chunks;
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t num_tiles = (C + DS_TILE - 1) / DS_TILE;
    if (tile >= num_tiles) return;
    const uint32_t x0 = tile * DS_TILE + tid * DS_ITEMS;
    uint32_t sz[DS_ITEMS];
    uint32_t tsum = 0;
#pragma unroll
    for (int i = 0; i < DS_ITEMS; ++i) {
        const uint32_t x = x0 + i;
        uint32_t v = 0;
        if (x < C) {
            const uint32_t c = __ldg(vals + x);
            v = __ldg(bases + c + 1) - __ldg(bases + c);
        }
        sz[i] = v;
        tsum += v;
    }
    uint32_t inc = tsum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= (uint32_t)d) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (tid == 0) {
        uint32_t r = 0;
        for (int w = 0; w < DS_THREADS / 32; ++w) {
            const uint32_t t = s_warp[w];
            s_warp[w] = r;
            r += t;
        }
        s_tot = r;
    }
    __syncthreads();
    if (warp == 0) {
        // decoupled look-back, 32 predecessors per step (lane l reads tile j - l), summing up to the
        // newest predecessor that already holds its inclusive prefix
        const uint32_t r = s_tot;
        unsigned long long* st = status + tile;
        uint32_t excl = 0;
        if (tile == 0) {
            if (lane == 0) st_release_u64(st, F_PRE | r);
        } else {
            if (lane == 0) st_release_u64(st, F_AGG | r);
            int64_t j = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (j >= 0) {
                const int64_t idx = j - (int64_t)lane;
                // flag and value share one word, so a relaxed load suffices
                const unsigned long long s = idx >= 0 ? ld_relaxed_u64(status + idx) : F_PRE;
                const unsigned long long f = s & ~V_MASK;
                const uint32_t pre = __ballot_sync(0xffffffffu, f == F_PRE);
                const uint32_t lim = pre ? (uint32_t)(__ffs(pre) - 1) : 31u;
                const uint32_t upto = lim == 31u ? 0xffffffffu : ((2u << lim) - 1u);
                if (__ballot_sync(0xffffffffu, f == 0ull) & upto) {
                    if (++spins > RSH_SPIN_LIMIT) {
                        raise_device_error(err, RSH_DEVERR_TIMEOUT);
                        break;
                    }
                    if (spins > 16) __nanosleep(32);
                    continue;
                }
                uint32_t v = lane <= lim ? (uint32_t)(s & V_MASK) : 0u;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
                excl += v;
                if (pre) break;
                j -= 32;
            }
            if (lane == 0) st_release_u64(st, F_PRE | (unsigned long long)(excl + r));
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    uint32_t run = s_excl + s_warp[warp] + inc - tsum;
#pragma unroll
    for (int i = 0; i < DS_ITEMS; ++i) {
        const uint32_t x = x0 + i;
        if (x < C) off[x] = run;
        run += sz[i];
    }
}

__global__ void __launch_bounds__(DE_THREADS)
k_dc_expand(const uint32_t* __restrict__ skeys, const uint32_t* __restrict__ vals,
            const uint32_t* __restrict__ bases, const uint32_t* __restrict__ trimmed,
            const uint32_t* __restrict__ counts, uint32_t max_rays, const uint32_t* __restrict__ off,
            uint32_t* __restrict__ sorted_keys, uint32_t* __restrict__ sorted_ids) {
    __shared__ uint32_t s_off[DE_TILE + 1];
    __shared__ uint32_t s_base[DE_TILE + 1];
    __shared__ uint32_t s_key[DE_TILE + 1];
    __shared__ uint32_t s_x0, s_m;
    const uint32_t R = counts[0] < max_rays ? counts[0] : max_rays;
    const uint32_t C = counts[1];
    const uint32_t k0 = blockIdx.x * DE_TILE;
    if (k0 >= R || C == 0) return;
    const uint32_t k1 = (k0 + DE_TILE < R ? k0 + DE_TILE : R) - 1;  // last output of the tile
    if (threadIdx.x == 0) {
        // chunk of k: the last x with off[x] <= k
        uint32_t lo = 0, hi = C;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(off + mid) <= k0) lo = mid; else hi = mid;
        }
        const uint32_t xa = lo;
        lo = xa;
        hi = C;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(off + mid) <= k1) lo = mid; else hi = mid;
        }
        s_x0 = xa;
        const uint32_t m = lo - xa + 1;  // <= DE_TILE: every chunk in range covers >= 1 output of the tile
        s_m = m < (uint32_t)DE_TILE ? m : (uint32_t)DE_TILE;
    }
    __syncthreads();
    const uint32_t x0 = s_x0, m = s_m;
    for (uint32_t i = threadIdx.x; i < m; i += DE_THREADS) {
        const uint32_t x = x0 + i;
        s_off[i] = __ldg(off + x);
        s_base[i] = __ldg(bases + __ldg(vals + x));
        s_key[i] = skeys ? __ldg(skeys + x) : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < DE_ITEMS; ++it) {
        const uint32_t k = k0 + it * DE_THREADS + threadIdx.x;
        if (k > k1) break;
        uint32_t lo = 0, hi = m;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_off[mid] <= k) lo = mid; else hi = mid;
        }
        const uint32_t src = s_base[lo] + (k - s_off[lo]);
        sorted_ids[k] = src < R ? __ldg(trimmed + src) : 0u;
        if (sorted_keys) sorted_keys[k] = s_key[lo];
    }
}

size_t decompress_scratch_bytes(uint32_t max_chunks) {
    const size_t tiles = (max_chunks + DS_TILE - 1) / DS_TILE + 1;
    return 64 + tiles * 8 + (size_t)max_chunks * 4 + 512;
}

cudaError_t launch_decompress(const uint32_t* sorted_chunk_keys, const uint32_t* sorted_chunk_vals,
                              const uint32_t* chunk_bases, const uint32_t* trimmed_ids,
                              const uint32_t* counts, uint32_t max_rays, uint32_t* sorted_keys,
                              uint32_t* sorted_ids, void* scratch, uint32_t* err, cudaStream_t s) {
    if (max_rays == 0) return cudaSuccess;
    const uint32_t max_chunks = max_rays;
    const size_t tiles = (max_chunks + DS_TILE - 1) / DS_TILE + 1;
    char* b = static_cast<char*>(scratch);
    uint32_t* ticket = reinterpret_cast<uint32_t*>(b);
    unsigned long long* status = reinterpret_cast<unsigned long long*>(b + 64);
    uint32_t* off = reinterpret_cast<uint32_t*>(b + 64 + tiles * 8);
    cudaError_t e = cudaMemsetAsync(b, 0, 64 + tiles * 8, s);
    if (e != cudaSuccess) return e;
    k_dc_scan<<<(unsigned)(tiles - 1 > 0 ? tiles - 1 : 1), DS_THREADS, 0, s>>>(
        sorted_chunk_vals, chunk_bases, counts, max_chunks, off, status, ticket, err);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_dc_expand<<<(max_rays + DE_TILE - 1) / DE_TILE, DE_THREADS, 0, s>>>(
        sorted_chunk_keys, sorted_chunk_vals, chunk_bases, trimmed_ids, counts, max_rays, off,
        sorted_keys, sorted_ids);
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
