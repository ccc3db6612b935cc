// Trim + compress in one pass over the ray keys.
//
// Reference: RayTrimmingWrapper (RayTracer.cu:2276-2324: CUB InclusiveSum of "no ray" flags, then
// CreateTrimmedRays :844-884, then a blocking D2H of the count) followed by RayCompressionWrapper
// (:2326-2383: CreateChunkFlags :886-918 -> InclusiveSum -> D2H -> CreateChunkBases :920-954 ->
// CreateChunkSizes :956-991). Semantics kept: trimmed order = slot order; a chunk is a maximal run of
// equal keys in trimmed order; chunk c has key, base (trimmed index of its head) and size.
//
// GB300 form: ONE kernel. Each CTA takes a 3072-slot tile by atomic ticket (in-order forward progress),
// reduces it to the associative summary (valid count, head count, first key, last key), publishes it
// and resolves its exclusive prefix by decoupled look-back (Merrill & Garland 2016) over predecessor
// tiles. Outputs are staged in shared memory and written coalesced. Counts stay on the device; the
// last tile also writes the sentinel chunk_bases[C] = R so sizes are base differences.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr int CT_THREADS = 256;
constexpr int CT_ITEMS = 12;
constexpr int CT_TILE = CT_THREADS * CT_ITEMS;  // 3072

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
RSH_DEV Summ shfl_down(const Summ& s, int d) {
    Summ r;
    r.n = __shfl_down_sync(0xffffffffu, s.n, d);
    r.h = __shfl_down_sync(0xffffffffu, s.h, d);
    r.first = __shfl_down_sync(0xffffffffu, s.first, d);
    r.last = __shfl_down_sync(0xffffffffu, s.last, d);
    return r;
}
RSH_DEV Summ shfl_idx0(const Summ& s) {
    Summ r;
    r.n = __shfl_sync(0xffffffffu, s.n, 0);
    r.h = __shfl_sync(0xffffffffu, s.h, 0);
    r.first = __shfl_sync(0xffffffffu, s.first, 0);
    r.last = __shfl_sync(0xffffffffu, s.last, 0);
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

// Scratch layout: [0] ticket, [1] pad, then flags[tiles], agg[tiles*4], inc[tiles*4]
struct CScratch {
    uint32_t* ticket;
    uint32_t* flags;
    uint32_t* agg;
    uint32_t* inc;
};
RSH_DEV void publish(uint32_t* dst4, uint32_t* flag, uint32_t fval, const Summ& s) {
    dst4[0] = s.n;
    dst4[1] = s.h;
    dst4[2] = s.first;
    dst4[3] = s.last;
    __threadfence();
    st_release_u32(flag, fval);
}
RSH_DEV Summ read4(const uint32_t* p) {
    Summ s;
    s.n = __ldcg(p);
    s.h = __ldcg(p + 1);
    s.first = __ldcg(p + 2);
    s.last = __ldcg(p + 3);
    return s;
}
}  // namespace

__global__ void __launch_bounds__(CT_THREADS)
k_compress(const uint32_t* __restrict__ keys, uint32_t n_slots, uint32_t num_tiles, bool vec_ok,
           uint32_t* __restrict__ trimmed_ids, uint32_t* __restrict__ chunk_keys,
           uint32_t* __restrict__ chunk_bases, uint32_t* __restrict__ counts, CScratch sc,
           uint32_t* err) {
    __shared__ uint32_t s_ids[CT_TILE];
    __shared__ uint32_t s_ckey[CT_TILE];
    __shared__ uint32_t s_cbase[CT_TILE];
    __shared__ Summ s_warp[CT_THREADS / 32];
    __shared__ Summ s_prefix, s_run;
    __shared__ uint32_t s_tile, s_tn, s_th;

    if (threadIdx.x == 0) s_tile = atomicAdd(sc.ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= num_tiles) return;
    const uint32_t base = tile * CT_TILE;
    const uint32_t t0 = base + threadIdx.x * CT_ITEMS;

    uint32_t k[CT_ITEMS];
    if (vec_ok && t0 + CT_ITEMS <= n_slots) {
        const uint4* p = reinterpret_cast<const uint4*>(keys + t0);
#pragma unroll
        for (int q = 0; q < CT_ITEMS / 4; ++q) {
            uint4 v = __ldg(p + q);
            k[4 * q] = v.x;
            k[4 * q + 1] = v.y;
            k[4 * q + 2] = v.z;
            k[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < CT_ITEMS; ++i) k[i] = (t0 + i < n_slots) ? __ldg(keys + t0 + i) : RSH_KEY_NONE;
    }

    // thread summary
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
    // warp inclusive scan (Kogge-Stone) of the summaries
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    Summ inc = ts;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        Summ o = shfl_up(inc, d);
        if (lane >= (uint32_t)d) inc = combine(o, inc);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        // tile aggregate and the warp-exclusive prefixes (serial over 8 warps)
        Summ run{0u, 0u, 0u, 0u};
        for (int w = 0; w < CT_THREADS / 32; ++w) {
            Summ wv = s_warp[w];
            s_warp[w] = run;
            run = combine(run, wv);
        }
        s_run = run;
    }
    __syncthreads();
    if (warp == 0) {
        // decoupled look-back, 32 predecessors per step: lane l reads tile j - l; the window is folded
        // (oldest first) up to the newest predecessor that already holds its inclusive prefix
        const Summ run = s_run;
        Summ excl{0u, 0u, 0u, 0u};
        if (tile == 0) {
            if (lane == 0) publish(sc.inc, sc.flags, 2u, run);
        } else {
            if (lane == 0) publish(sc.agg + 4ull * tile, sc.flags + tile, 1u, run);
            int64_t j = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (j >= 0) {
                const int64_t idx = j - (int64_t)lane;
                const uint32_t f = idx >= 0 ? ld_acquire_u32(sc.flags + idx) : 2u;
                const uint32_t incl = __ballot_sync(0xffffffffu, f == 2u);
                const uint32_t lim = incl ? (uint32_t)(__ffs(incl) - 1) : 31u;
                const uint32_t upto = lim == 31u ? 0xffffffffu : ((2u << lim) - 1u);
                if (__ballot_sync(0xffffffffu, f == 0u) & upto) {
                    if (++spins > RSH_SPIN_LIMIT) {
                        raise_device_error(err, RSH_DEVERR_TIMEOUT);
                        break;
                    }
                    if (spins > 16) __nanosleep(32);
                    continue;
                }
                Summ v{0u, 0u, 0u, 0u};
                if (lane <= lim && idx >= 0) v = read4((f == 2u ? sc.inc : sc.agg) + 4ull * idx);
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const Summ o = shfl_down(v, d);
                    if ((lane & (2u * d - 1u)) == 0u) v = combine(o, v);
                }
                v = shfl_idx0(v);
                excl = combine(v, excl);
                if (incl) break;
                j -= 32;
            }
            if (lane == 0) publish(sc.inc + 4ull * tile, sc.flags + tile, 2u, combine(excl, run));
        }
        if (lane == 0) {
            s_prefix = excl;
            if (tile == num_tiles - 1) {
                const Summ tot = combine(excl, run);
                counts[0] = tot.n < n_slots ? tot.n : n_slots;
                counts[1] = tot.h < n_slots ? tot.h : n_slots;
                chunk_bases[counts[1]] = counts[0];
            }
        }
    }
    __syncthreads();
    // exclusive prefix of this thread = tile prefix (x) warp prefix (x) lane-exclusive
    Summ lane_ex = shfl_up(inc, 1);
    if (lane == 0) lane_ex = Summ{0u, 0u, 0u, 0u};
    const Summ tile_pre = s_prefix;
    Summ run = combine(combine(tile_pre, s_warp[warp]), lane_ex);
    const uint32_t r_base = tile_pre.n;  // trimmed index of the tile's first valid slot
    // chunk index of the tile's first head: a tile that starts inside a run from the previous tile
    // has no head there, which combine() already accounted for in tile_pre.h
    const uint32_t h_tile0 = tile_pre.h;
#pragma unroll
    for (int i = 0; i < CT_ITEMS; ++i) {
        const uint32_t key = k[i];
        if (key != RSH_KEY_NONE) {
            const bool head = (run.n == 0u) || (key != run.last);
            const uint32_t r = run.n;
            if (r - r_base < (uint32_t)CT_TILE) s_ids[r - r_base] = t0 + i;
            if (head) {
                const uint32_t c = run.h;
                if (c - h_tile0 < (uint32_t)CT_TILE) {
                    s_ckey[c - h_tile0] = key;
                    s_cbase[c - h_tile0] = r;
                }
            }
            run.h += head ? 1u : 0u;
            run.n += 1u;
            run.last = key;
        }
    }
    __syncthreads();
    // tile totals: the last thread's running summary is inclusive of the whole tile
    if (threadIdx.x == CT_THREADS - 1) {
        s_tn = min(run.n - r_base, (uint32_t)CT_TILE);
        s_th = min(run.h - h_tile0, (uint32_t)CT_TILE);
    }
    __syncthreads();
    const uint32_t tn = s_tn, th = s_th;
    // bounds hold by construction; the checks only matter after a look-back timeout
    for (uint32_t i = threadIdx.x; i < tn; i += CT_THREADS)
        if (r_base + i < n_slots) trimmed_ids[r_base + i] = s_ids[i];
    for (uint32_t i = threadIdx.x; i < th; i += CT_THREADS) {
        if (h_tile0 + i < n_slots) {
            chunk_keys[h_tile0 + i] = s_ckey[i];
            chunk_bases[h_tile0 + i] = s_cbase[i];
        }
    }
}

size_t compress_scratch_bytes(uint32_t n_slots) {
    const size_t tiles = (n_slots + CT_TILE - 1) / CT_TILE + 1;
    return (4 + tiles * 9) * sizeof(uint32_t) + 256;
}

cudaError_t launch_compress(const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                            uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* counts,
                            void* scratch, uint32_t* err, cudaStream_t s) {
    if (n_slots == 0) {
        cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), s);
        cudaMemsetAsync(chunk_bases, 0, sizeof(uint32_t), s);
        return cudaGetLastError();
    }
    const uint32_t tiles = (n_slots + CT_TILE - 1) / CT_TILE;
    uint32_t* w = static_cast<uint32_t*>(scratch);
    CScratch sc;
    sc.ticket = w;
    sc.flags = w + 4;
    sc.agg = sc.flags + tiles;
    sc.inc = sc.agg + 4ull * tiles;
    cudaError_t e = cudaMemsetAsync(w, 0, (4 + tiles) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
    k_compress<<<tiles, CT_THREADS, 0, s>>>(keys, n_slots, tiles, vec_ok, trimmed_ids, chunk_keys,
                                            chunk_bases, counts, sc, err);
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
