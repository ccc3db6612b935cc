// Stable LSD radix sort of (u32 key, u32 value) pairs, onesweep form (Adinets & Merrill 2022).
//
// Reference: RaySortingWrapper -> cub::DeviceRadixSort::SortPairs over all 32 key bits
// (RayTracer.cu:2385-2409, temp storage sized at :2127-2139). Here: our own kernels, and only the
// ceil(key_bits / 8) digit passes the hash actually uses.
//
//  1. one histogram kernel reads the keys once and builds all passes' 256-bin digit histograms; its last
//     CTA turns them into per-pass exclusive digit offsets;
//  2. one kernel per 8-bit digit pass: each CTA takes a 3840-key tile by atomic ticket, ranks its keys
//     stably (warp peer masks: every third item by match_any, the others from 8 ballots, 9 in a partial
//     tile; per-warp digit counters), publishes its per-digit counts,
//     resolves the per-digit exclusive prefix over earlier tiles by decoupled look-back (bounded spin),
//     then scatters through shared memory so that global writes are runs of one digit. A status word
//     holds flag and count together and nothing else is read through it, so it is published and read
//     with relaxed (not release / acquire) accesses: no memory barrier per tile.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace rsh {

namespace {
constexpr int SR_THREADS = 256;
constexpr int SR_WARPS = SR_THREADS / 32;
constexpr int SR_ITEMS = 15;
constexpr int SR_TILE = SR_THREADS * SR_ITEMS;  // 3840
constexpr uint32_t FLAG_AGG = 1u << 30;
constexpr uint32_t FLAG_PRE = 2u << 30;
constexpr uint32_t VAL_MASK = (1u << 30) - 1u;

#ifndef RSH_SORT_MATCH_EVERY
#define RSH_SORT_MATCH_EVERY 3
#endif
#ifndef RSH_SORT_FULL8
#define RSH_SORT_FULL8 1
#endif

inline uint32_t num_passes(uint32_t key_bits) { return key_bits == 0 ? 1u : (key_bits + 7u) / 8u; }
}  // namespace

// --- histograms of every pass in one read; also clears the look-back status rows of the tiles that
// the passes will use (ceil(n / SR_TILE) rows of 256 words per pass, pass stride `stride` words)
__global__ void k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n_max,
                            const uint32_t* __restrict__ d_count, uint32_t passes,
                            uint32_t* __restrict__ hist, uint32_t* __restrict__ status, size_t stride,
                            uint32_t* __restrict__ done) {
    __shared__ uint32_t sh[4][256];
    __shared__ uint32_t s_last;
    for (uint32_t i = threadIdx.x; i < 4u * 256u; i += blockDim.x) (&sh[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t n = dev_count(d_count, n_max);
    {
        const size_t words = (size_t)((n + SR_TILE - 1) / SR_TILE) * 256u;  // multiple of 4
        const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
        for (uint32_t p = 0; p < passes; ++p) {
            uint4* row = reinterpret_cast<uint4*>(status + p * stride);
            for (size_t i = tid; i < words / 4; i += nth) row[i] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    // each thread counts a contiguous run of keys and adds equal consecutive digits up before one shared
    // atomic: the keys arrive coherent (hash runs in ray order), so their upper digits repeat in long runs
    // that would otherwise pile up on one shared counter. The run is loaded once into registers (four
    // 16-byte loads when the keys are 16-byte aligned) and every pass counts from there: one 4-byte load
    // per key and pass, with the lanes' runs 64 bytes apart, kept the L1 busy a line per lane.
    {
        constexpr uint32_t RUN = 16;
        const uint32_t nth = gridDim.x * blockDim.x;
        const bool a16 = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0u;
        for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * RUN; base < n; base += nth * RUN) {
            const uint32_t cnt = min(n - base, RUN);
            uint32_t k[RUN];
            if (a16 && cnt == RUN) {
                const uint4* q = reinterpret_cast<const uint4*>(keys + base);
#pragma unroll
                for (uint32_t j = 0; j < RUN / 4u; ++j) {
                    const uint4 v = __ldg(q + j);
                    k[4u * j] = v.x;
                    k[4u * j + 1u] = v.y;
                    k[4u * j + 2u] = v.z;
                    k[4u * j + 3u] = v.w;
                }
            } else {
#pragma unroll
                for (uint32_t i = 0; i < RUN; ++i) k[i] = i < cnt ? __ldg(keys + base + i) : 0u;
            }
            for (uint32_t p = 0; p < passes; ++p) {
                const uint32_t sh_p = 8u * p;
                uint32_t prev = (k[0] >> sh_p) & 255u, run = 0;
#pragma unroll
                for (uint32_t i = 0; i < RUN; ++i) {
                    if (i < cnt) {
                        const uint32_t d = (k[i] >> sh_p) & 255u;
                        if (d != prev) {
                            atomicAdd(&sh[p][prev], run);
                            prev = d;
                            run = 0;
                        }
                        ++run;
                    }
                }
                atomicAdd(&sh[p][prev], run);
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * 256u; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
    // the last CTA to finish turns the counts into exclusive digit offsets, in place
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(done, 1u) == gridDim.x - 1u) ? 1u : 0u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // exclusive digit offsets of every pass: one block-wide scan of the 256 bins per pass
    for (uint32_t p = 0; p < passes; ++p) {
        uint32_t* h = hist + 256u * p;
        const uint32_t t = threadIdx.x;  // blockDim.x == 256
        const uint32_t v = __ldcg(h + t);
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((t & 31u) >= (uint32_t)o) x += y;
        }
        if ((t & 31u) == 31u) sh[0][t >> 5] = x;  // the shared counters are free now
        __syncthreads();
        if (t < 32) {
            uint32_t ws = t < 8u ? sh[0][t] : 0u;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, ws, o);
                if (t >= (uint32_t)o) ws += y;
            }
            if (t < 8u) sh[1][t] = ws;
        }
        __syncthreads();
        const uint32_t warp_off = (t >= 32u) ? sh[1][(t >> 5) - 1] : 0u;
        h[t] = warp_off + x - v;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(SR_THREADS, 3)
k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
           uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n_max,
           const uint32_t* __restrict__ d_count, uint32_t shift, const uint32_t* __restrict__ hist,
           uint32_t* __restrict__ status, uint32_t* __restrict__ ticket, uint32_t* err, uint32_t spin_limit) {
    __shared__ uint32_t s_wc[SR_WARPS][256];    // per-warp digit counts -> exclusive warp offsets
    __shared__ uint32_t s_keys[SR_TILE];
    __shared__ uint32_t s_vals[SR_TILE];
    __shared__ uint32_t s_start[256];            // tile-local digit start
    __shared__ uint32_t s_gbase[256];            // global position of the tile's first key of a digit
    __shared__ uint32_t s_scan[SR_WARPS];
    __shared__ uint32_t s_tile;

    const uint32_t n = dev_count(d_count, n_max);
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t num_tiles = (n + SR_TILE - 1) / SR_TILE;
  for (;;) {  // tiles by ticket until none is left (the grid is capped at the resident CTAs)
    if (tid == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= num_tiles) return;
    for (uint32_t i = tid; i < SR_WARPS * 256u; i += SR_THREADS) (&s_wc[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t base = tile * SR_TILE;
    const uint32_t wbase = base + warp * (SR_ITEMS * 32u);

    uint32_t key[SR_ITEMS], val[SR_ITEMS], rank[SR_ITEMS];
#pragma unroll
    for (int j = 0; j < SR_ITEMS; ++j) {
        const uint32_t idx = wbase + j * 32u + lane;
        if (idx < n) {
            key[j] = __ldg(keys_in + idx);
            val[j] = vals_in ? __ldg(vals_in + idx) : idx;
        } else {
            key[j] = 0xFFFFFFFFu;
            val[j] = 0u;
        }
    }
    const bool full = base + SR_TILE <= n;  // the whole tile holds valid items
    // stable in-warp ranking: items in (j, lane) order = index order
#pragma unroll
    for (int j = 0; j < SR_ITEMS; ++j) {
        const uint32_t idx = wbase + j * 32u + lane;
        const bool valid = idx < n;
        const uint32_t d = valid ? ((key[j] >> shift) & 255u) : 256u;
        uint32_t peers;  // lanes holding the same digit (or also invalid)
        if (RSH_SORT_MATCH_EVERY && (j % RSH_SORT_MATCH_EVERY) == RSH_SORT_MATCH_EVERY - 1) {
            // some items by match_any (the MIO pipe), the others by ballots (the ALU pipe): the two
            // pipes share the ranking instead of one of them bounding it
            peers = __match_any_sync(0xffffffffu, d);
        } else {
            peers = 0xffffffffu;
            if (RSH_SORT_FULL8 && full) {  // a full tile has no invalid items: 8 digit bits decide
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const bool bit = (d >> b) & 1u;
                    const uint32_t bal = __ballot_sync(0xffffffffu, bit);
                    peers &= bit ? bal : ~bal;
                }
            } else {
#pragma unroll
                for (int b = 0; b < 9; ++b) {
                    const bool bit = (d >> b) & 1u;
                    const uint32_t bal = __ballot_sync(0xffffffffu, bit);
                    peers &= bit ? bal : ~bal;
                }
            }
        }
        const uint32_t before = __popc(peers & lanemask_lt());
        uint32_t cnt = 0u;
        if (valid) cnt = s_wc[warp][d];
        __syncwarp();
        if (valid && before == 0u) s_wc[warp][d] = cnt + __popc(peers);
        __syncwarp();
        rank[j] = cnt + before;
    }
    __syncthreads();
    // per digit (thread = digit): warp-exclusive offsets and the tile count
    const uint32_t dg = tid;  // SR_THREADS == 256
    uint32_t tcount = 0u;
#pragma unroll
    for (int w = 0; w < SR_WARPS; ++w) {
        const uint32_t c = s_wc[w][dg];
        s_wc[w][dg] = tcount;
        tcount += c;
    }
    // publish the tile's count for this digit early so successors can proceed
    uint32_t* st = status + (size_t)tile * 256u + dg;
    if (tile == 0) st_relaxed_u32(st, FLAG_PRE | tcount);
    else st_relaxed_u32(st, FLAG_AGG | tcount);
    // exclusive scan over digits of tcount -> s_start
    {
        uint32_t x = tcount;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= (uint32_t)d) x += y;
        }
        if (lane == 31) s_scan[warp] = x;
        __syncthreads();
        if (tid == 0) {
            uint32_t r = 0;
            for (int w = 0; w < SR_WARPS; ++w) {
                const uint32_t t = s_scan[w];
                s_scan[w] = r;
                r += t;
            }
        }
        __syncthreads();
        const uint32_t start = s_scan[warp] + x - tcount;
        s_start[dg] = start;
#pragma unroll
        for (int w = 0; w < SR_WARPS; ++w) s_wc[w][dg] += start;  // tile-local position of each warp's run
    }
    // global digit offset of this pass (exclusive, from the histogram kernel)
    const uint32_t gex = __ldg(hist + dg);
    // decoupled look-back for this digit, LB predecessors per step: their status words are loaded
    // together (flag and count share one word, so relaxed loads suffice) and folded newest first up to
    // the first one holding an inclusive prefix; a not-yet-published word restarts the step there
    uint32_t excl = 0u;
    if (tile > 0) {
#ifndef RSH_SORT_LB
#define RSH_SORT_LB 8
#endif
        constexpr int LB = RSH_SORT_LB;
        int64_t j = (int64_t)tile - 1;
        uint32_t spins = 0;
        while (j >= 0) {
            uint32_t sv[LB];
#pragma unroll
            for (int q = 0; q < LB; ++q)
                sv[q] = (j - q >= 0) ? ld_relaxed_u32(status + (size_t)(j - q) * 256u + dg) : FLAG_PRE;
            int used = 0;
            bool done = false, stall = false;
#pragma unroll
            for (int q = 0; q < LB; ++q) {
                if (done || stall) continue;
                const uint32_t f = sv[q] & ~VAL_MASK;
                if (f == 0u) {
                    stall = true;
                    continue;
                }
                excl += sv[q] & VAL_MASK;
                ++used;
                if (f == FLAG_PRE) done = true;
            }
            if (done) break;
            j -= used;
            if (stall) {
                if (++spins > spin_limit) {
                    raise_device_error(err, RSH_DEVERR_TIMEOUT);
                    break;
                }
                if (spins > 16) __nanosleep(32);
            }
        }
        st_relaxed_u32(st, FLAG_PRE | (excl + tcount));
    }
    s_gbase[dg] = gex + excl - s_start[dg];
    __syncthreads();
    // scatter into shared memory in tile-sorted order
#pragma unroll
    for (int j = 0; j < SR_ITEMS; ++j) {
        const uint32_t idx = wbase + j * 32u + lane;
        if (idx < n) {
            const uint32_t d = (key[j] >> shift) & 255u;
            const uint32_t pos = s_wc[warp][d] + rank[j];
            s_keys[pos] = key[j];
            s_vals[pos] = val[j];
        }
    }
    __syncthreads();
    const uint32_t tn = (n - base) < (uint32_t)SR_TILE ? (n - base) : (uint32_t)SR_TILE;
    for (uint32_t i = tid; i < tn; i += SR_THREADS) {
        const uint32_t k = s_keys[i];
        const uint32_t d = (k >> shift) & 255u;
        const uint32_t g = s_gbase[d] + i;
        if (g < n) {  // only false after a look-back timeout (error word raised)
            keys_out[g] = k;
            vals_out[g] = s_vals[i];
        }
    }
    __syncthreads();  // shared state is reused by the next tile
  }
}

size_t sort_scratch_bytes(uint32_t n_max, uint32_t key_bits) {
    const size_t passes = num_passes(key_bits);
    const size_t tiles = (n_max + SR_TILE - 1) / SR_TILE + 1;
    const size_t words = 4 * 256 + 16 + passes * tiles * 256;
    return words * 4 + 2 * (size_t)n_max * 4 + 1024;
}

cudaError_t launch_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                              uint32_t* vals_out, uint32_t n_max, const uint32_t* d_count,
                              uint32_t key_bits, void* scratch, uint32_t* err, cudaStream_t s) {
    if (n_max == 0) return cudaSuccess;
    const uint32_t passes = num_passes(key_bits);
    const size_t tiles = (n_max + SR_TILE - 1) / SR_TILE + 1;
    uint32_t* w = static_cast<uint32_t*>(scratch);
    uint32_t* hist = w;                       // passes * 256 (room for 4)
    uint32_t* tickets = w + 4 * 256;          // 16: one per pass, [8] = histogram CTAs done
    uint32_t* status = tickets + 16;          // passes * tiles * 256
    uint32_t* alt_keys = status + passes * tiles * 256;
    alt_keys = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(alt_keys) + 255) & ~uintptr_t(255));
    uint32_t* alt_vals = alt_keys + n_max;
    cudaError_t e = cudaMemsetAsync(w, 0, (4 * 256 + 16) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    k_sort_hist<<<152 * 2, 256, 0, s>>>(keys_in, n_max, d_count, passes, hist, status, tiles * 256, tickets + 8);
    // at most the CTAs resident at once: tiles beyond the device count cost nothing, and every ticket
    // below a CTA's tile is held by a running CTA (forward progress of the look-back)
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_onesweep, SR_THREADS, 0);
    if (per_sm < 1) per_sm = 1;
    const uint32_t resident = (uint32_t)(sms * per_sm);
    note_launch();
    // ping-pong so that the last pass lands in the output
    const uint32_t* ki = keys_in;
    const uint32_t* vi = vals_in;
    for (uint32_t p = 0; p < passes; ++p) {
        const bool last = (p + 1 == passes);
        // choose destinations: passes alternate between out and alt, ending in out
        const bool to_out = ((passes - 1 - p) % 2u) == 0u;
        uint32_t* ko = to_out ? keys_out : alt_keys;
        uint32_t* vo = to_out ? vals_out : alt_vals;
        (void)last;
        const uint32_t grid = std::min<uint32_t>((uint32_t)(tiles - 1 > 0 ? tiles - 1 : 1), resident);
        k_onesweep<<<grid, SR_THREADS, 0, s>>>(ki, vi, ko, vo, n_max, d_count, 8u * p, hist + 256u * p,
                                               status + p * tiles * 256, tickets + p, err, RSH_SPIN_LIMIT);
        note_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        ki = ko;
        vi = vo;
    }
    return cudaSuccess;
}

// Self-test of the bounded look-back wait: one sort pass over two tiles whose first tile is never run
// (its ticket is taken before the launch), so the second tile waits on a status word that nothing
// publishes. The wait must give up after `spin_limit` polls and raise RSH_DEVERR_TIMEOUT in *err
// instead of hanging; every write stays in bounds. Buffers (2 tiles of keys in/out, status, tickets)
// come from the caller's scratch of sort_selftest_scratch_bytes().
size_t sort_selftest_scratch_bytes() { return (size_t)(4 * 2 * SR_TILE + 2 * 256 + 256 + 8) * 4 + 1024; }

cudaError_t sort_selftest_timeout(void* scratch, uint32_t* err, uint32_t spin_limit, cudaStream_t s) {
    uint32_t* w = static_cast<uint32_t*>(scratch);
    const uint32_t n = 2 * SR_TILE;
    uint32_t* keys_in = w;
    uint32_t* vals_in = keys_in + n;
    uint32_t* keys_out = vals_in + n;
    uint32_t* vals_out = keys_out + n;
    uint32_t* status = vals_out + n;      // 2 tiles x 256 digits, all "not yet published"
    uint32_t* hist = status + 2 * 256;    // 256 exclusive digit offsets: all 0 (every key is digit 0)
    uint32_t* ticket = hist + 256;
    cudaError_t e = cudaMemsetAsync(w, 0, sort_selftest_scratch_bytes() - 1024, s);
    if (e != cudaSuccess) return e;
    const uint32_t one = 1u;  // tile 0's ticket is already gone: the one CTA gets tile 1
    if ((e = cudaMemcpyAsync(ticket, &one, 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    k_onesweep<<<1, SR_THREADS, 0, s>>>(keys_in, vals_in, keys_out, vals_out, n, nullptr, 0u, hist, status, ticket, err,
                                        spin_limit);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

}  // namespace rsh
