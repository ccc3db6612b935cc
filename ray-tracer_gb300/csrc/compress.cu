// Trim + compress in one pass over the ray keys.
//
// Reference: RayTrimmingWrapper (RayTracer.cu:2276-2324: CUB InclusiveSum of "no ray" flags, then
// CreateTrimmedRays :844-884, then a blocking D2H of the count) followed by RayCompressionWrapper
// (:2326-2383: CreateChunkFlags :886-918 -> InclusiveSum -> D2H -> CreateChunkBases :920-954 ->
// CreateChunkSizes :956-991). Semantics kept: trimmed order = slot order; a chunk is a maximal run of
// equal keys in trimmed order; chunk c has key, base (trimmed index of its head) and size.
//
// GB300 form: reduce-then-scan in three launches, with no inter-CTA waiting at all:
//   k_compress_reduce  one CTA per 4096-slot tile reduces the tile to the associative summary (valid
//                      count, head count, first key, last key);
//   k_compress_scan    one CTA scans the tile summaries into tile prefixes (and writes the counts and
//                      the sentinel chunk_bases[C] = R);
//   k_compress_write   one CTA per tile re-reads its keys (an L2 hit at frame sizes), combines tile,
//                      warp and lane prefixes, and writes trimmed ids, chunk keys and chunk bases
//                      through one shared-memory staging buffer, coalesced.
// At frame sizes (2-10 M slots, one or a few waves of tiles) a single-pass decoupled look-back spends
// most of its time in the first wave's look-back chain (every predecessor holds an aggregate only),
// which this form does not have. Counts stay on the device.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr int CT_THREADS = 256;
constexpr int CT_ITEMS = 16;
constexpr int CT_TILE = CT_THREADS * CT_ITEMS;  // 4096
constexpr int CS_THREADS = 1024;                // the summary scan

struct Summ {  // summary of a key range: valid count, heads (first valid counted), first/last key
    uint32_t n, h, first, last;
};
RSH_DEV Summ combine(const Summ& a, const Summ& b) {
    Summ r;
    r.n = a.n + b.n;
    r.h = a.h + b.h - ((a.n > 0u && b.n > 0u && a.last == b.first) ? 1u : 0u);
    r.first = a.n > 0u ? a.first : b.first;
    r.last = b.n > 0u ? b.last : a.last;
    return r;
}
RSH_DEV Summ shfl_up(const Summ& s, int d) {
    Summ r;
    r.n = __shfl_up_sync(0xffffffffu, s.n, d);
    r.h = __shfl_up_sync(0xffffffffu, s.h, d);
    r.first = __shfl_up_sync(0xffffffffu, s.first, d);
    r.last = __shfl_up_sync(0xffffffffu, s.last, d);
    return r;
}
RSH_DEV uint4 to4(const Summ& s) { return make_uint4(s.n, s.h, s.first, s.last); }
RSH_DEV Summ from4(const uint4& v) { return Summ{v.x, v.y, v.z, v.w}; }

// The tile's keys, 16 consecutive slots per thread (vector loads when aligned and whole).
RSH_DEV void load_tile(const uint32_t* __restrict__ keys, uint32_t n_slots, bool vec_ok, uint32_t t0,
                       uint32_t (&k)[CT_ITEMS]) {
    if (vec_ok && t0 + CT_ITEMS <= n_slots) {
        const uint4* p = reinterpret_cast<const uint4*>(keys + t0);
#pragma unroll
        for (int q = 0; q < CT_ITEMS / 4; ++q) {
            const uint4 v = __ldg(p + q);
            k[4 * q] = v.x;
            k[4 * q + 1] = v.y;
            k[4 * q + 2] = v.z;
            k[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < CT_ITEMS; ++i) k[i] = (t0 + i < n_slots) ? __ldg(keys + t0 + i) : RSH_KEY_NONE;
    }
}

RSH_DEV Summ thread_summary(const uint32_t (&k)[CT_ITEMS]) {
    Summ ts{0u, 0u, 0u, 0u};
#pragma unroll
    for (int i = 0; i < CT_ITEMS; ++i) {
        if (k[i] != RSH_KEY_NONE) {
            if (ts.n == 0u) {
                ts.first = k[i];
                ts.h = 1u;
            } else if (k[i] != ts.last) {
                ts.h += 1u;
            }
            ts.last = k[i];
            ts.n += 1u;
        }
    }
    return ts;
}

// Block-wide: warp-inclusive scan of the thread summaries; s_warp[w] becomes the exclusive prefix of
// warp w inside the tile; returns the thread's warp-inclusive summary; *tile_total (thread 0) the tile's.
RSH_DEV Summ block_scan(const Summ& ts, Summ* s_warp, Summ* tile_total) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    Summ inc = ts;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const Summ o = shfl_up(inc, d);
        if (lane >= (uint32_t)d) inc = combine(o, inc);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        Summ run{0u, 0u, 0u, 0u};
        for (int w = 0; w < CT_THREADS / 32; ++w) {
            const Summ wv = s_warp[w];
            s_warp[w] = run;
            run = combine(run, wv);
        }
        *tile_total = run;
    }
    __syncthreads();
    return inc;
}
}  // namespace

__global__ void __launch_bounds__(CT_THREADS)
k_compress_reduce(const uint32_t* __restrict__ keys, uint32_t n_slots, bool vec_ok, uint4* __restrict__ tsumm) {
    __shared__ Summ s_warp[CT_THREADS / 32];
    __shared__ Summ s_tot;
    const uint32_t t0 = blockIdx.x * CT_TILE + threadIdx.x * CT_ITEMS;
    uint32_t k[CT_ITEMS];
    load_tile(keys, n_slots, vec_ok, t0, k);
    block_scan(thread_summary(k), s_warp, &s_tot);
    if (threadIdx.x == 0) tsumm[blockIdx.x] = to4(s_tot);
}

// One CTA: exclusive prefixes of the tile summaries (each thread folds a run of consecutive tiles).
__global__ void __launch_bounds__(CS_THREADS)
k_compress_scan(const uint4* __restrict__ tsumm, uint32_t tiles, uint32_t n_slots, uint4* __restrict__ tpre,
                uint32_t* __restrict__ counts, uint32_t* __restrict__ chunk_bases) {
    __shared__ Summ s_w[CS_THREADS / 32];
    const uint32_t per = (tiles + CS_THREADS - 1) / CS_THREADS;
    const uint32_t b = threadIdx.x * per, e = min(b + per, tiles);
    Summ ts{0u, 0u, 0u, 0u};
    for (uint32_t i = b; i < e; ++i) ts = combine(ts, from4(__ldg(tsumm + i)));
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    Summ inc = ts;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const Summ o = shfl_up(inc, d);
        if (lane >= (uint32_t)d) inc = combine(o, inc);
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        Summ run{0u, 0u, 0u, 0u};
        for (int w = 0; w < CS_THREADS / 32; ++w) {
            const Summ wv = s_w[w];
            s_w[w] = run;
            run = combine(run, wv);
        }
        const uint32_t R = run.n < n_slots ? run.n : n_slots;
        const uint32_t C = run.h < n_slots ? run.h : n_slots;
        counts[0] = R;
        counts[1] = C;
        chunk_bases[C] = R;
    }
    __syncthreads();
    Summ lane_ex = shfl_up(inc, 1);
    if (lane == 0) lane_ex = Summ{0u, 0u, 0u, 0u};
    Summ run = combine(s_w[warp], lane_ex);
    for (uint32_t i = b; i < e; ++i) {
        tpre[i] = to4(run);
        run = combine(run, from4(__ldg(tsumm + i)));
    }
}

__global__ void __launch_bounds__(CT_THREADS)
k_compress_write(const uint32_t* __restrict__ keys, uint32_t n_slots, bool vec_ok, const uint4* __restrict__ tpre,
                 uint32_t* __restrict__ trimmed_ids, uint32_t* __restrict__ chunk_keys,
                 uint32_t* __restrict__ chunk_bases) {
    __shared__ uint32_t s_buf[CT_TILE];
    __shared__ Summ s_warp[CT_THREADS / 32];
    __shared__ Summ s_tot;
    __shared__ uint32_t s_tn, s_th;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t t0 = blockIdx.x * CT_TILE + threadIdx.x * CT_ITEMS;
    uint32_t k[CT_ITEMS];
    load_tile(keys, n_slots, vec_ok, t0, k);
    const Summ inc = block_scan(thread_summary(k), s_warp, &s_tot);
    // exclusive prefix of this thread = tile prefix (x) warp prefix (x) lane-exclusive
    Summ lane_ex = shfl_up(inc, 1);
    if (lane == 0) lane_ex = Summ{0u, 0u, 0u, 0u};
    const Summ tile_pre = from4(__ldg(tpre + blockIdx.x));
    const Summ run0 = combine(combine(tile_pre, s_warp[warp]), lane_ex);
    const uint32_t r_base = tile_pre.n;  // trimmed index of the tile's first valid slot
    // chunk index of the tile's first head: a tile that starts inside a run from the previous tile
    // has no head there, which combine() already accounted for in tile_pre.h
    const uint32_t h_tile0 = tile_pre.h;
    // pass 1: trimmed ids
    Summ run = run0;
#pragma unroll
    for (int i = 0; i < CT_ITEMS; ++i) {
        if (k[i] != RSH_KEY_NONE) {
            const uint32_t r = run.n - r_base;
            if (r < (uint32_t)CT_TILE) s_buf[r] = t0 + i;
            run.n += 1u;
        }
    }
    if (threadIdx.x == CT_THREADS - 1) s_tn = min(run.n - r_base, (uint32_t)CT_TILE);
    __syncthreads();
    const uint32_t tn = s_tn;
    for (uint32_t i = threadIdx.x; i < tn; i += CT_THREADS)
        if (r_base + i < n_slots) trimmed_ids[r_base + i] = s_buf[i];
    __syncthreads();
    // pass 2: chunk keys of the heads
    run = run0;
#pragma unroll
    for (int i = 0; i < CT_ITEMS; ++i) {
        const uint32_t key = k[i];
        if (key != RSH_KEY_NONE) {
            if ((run.n == 0u) || (key != run.last)) {
                const uint32_t c = run.h - h_tile0;
                if (c < (uint32_t)CT_TILE) s_buf[c] = key;
                run.h += 1u;
            }
            run.n += 1u;
            run.last = key;
        }
    }
    if (threadIdx.x == CT_THREADS - 1) s_th = min(run.h - h_tile0, (uint32_t)CT_TILE);
    __syncthreads();
    const uint32_t th = s_th;
    for (uint32_t i = threadIdx.x; i < th; i += CT_THREADS)
        if (h_tile0 + i < n_slots) chunk_keys[h_tile0 + i] = s_buf[i];
    __syncthreads();
    // pass 3: chunk bases (trimmed index of each head)
    run = run0;
#pragma unroll
    for (int i = 0; i < CT_ITEMS; ++i) {
        const uint32_t key = k[i];
        if (key != RSH_KEY_NONE) {
            if ((run.n == 0u) || (key != run.last)) {
                const uint32_t c = run.h - h_tile0;
                if (c < (uint32_t)CT_TILE) s_buf[c] = run.n;
                run.h += 1u;
            }
            run.n += 1u;
            run.last = key;
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < th; i += CT_THREADS)
        if (h_tile0 + i < n_slots) chunk_bases[h_tile0 + i] = s_buf[i];
}

size_t compress_scratch_bytes(uint32_t n_slots) {
    const size_t tiles = (n_slots + CT_TILE - 1) / CT_TILE + 1;
    return tiles * 2 * sizeof(uint4) + 256;
}

cudaError_t launch_compress(const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                            uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* counts,
                            void* scratch, uint32_t* err, cudaStream_t s) {
    (void)err;  // no step of this form waits on another CTA
    if (n_slots == 0) {
        cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), s);
        cudaMemsetAsync(chunk_bases, 0, sizeof(uint32_t), s);
        return cudaGetLastError();
    }
    const uint32_t tiles = (n_slots + CT_TILE - 1) / CT_TILE;
    uint4* tsumm = static_cast<uint4*>(scratch);
    uint4* tpre = tsumm + tiles;
    const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
    k_compress_reduce<<<tiles, CT_THREADS, 0, s>>>(keys, n_slots, vec_ok, tsumm);
    note_launch();
    k_compress_scan<<<1, CS_THREADS, 0, s>>>(tsumm, tiles, n_slots, tpre, counts, chunk_bases);
    note_launch();
    k_compress_write<<<tiles, CT_THREADS, 0, s>>>(keys, n_slots, vec_ok, tpre, trimmed_ids, chunk_keys, chunk_bases);
    note_launch();
    return cudaGetLastError();
}

__global__ void k_chunk_sizes(const uint32_t* __restrict__ bases, const uint32_t* __restrict__ counts,
                              uint32_t max_chunks, uint32_t* sizes) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t C = counts[1] < max_chunks ? counts[1] : max_chunks;
    if (c >= C) return;
    sizes[c] = bases[c + 1] - bases[c];
}

cudaError_t launch_chunk_sizes(const uint32_t* chunk_bases, const uint32_t* counts, uint32_t max_chunks,
                               uint32_t* chunk_sizes, cudaStream_t s) {
    if (max_chunks == 0) return cudaSuccess;
    k_chunk_sizes<<<(max_chunks + 255) / 256, 256, 0, s>>>(chunk_bases, counts, max_chunks, chunk_sizes);
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
