// Ray generation fused with the 32-bit ray hash.
//
// Reference: CreateShadowRays (RayTracer.cu:682-740), CreateReflectionRays (:742-791), the ray
// creation tail of ColorAndCreateReflectionRay (:1995-2016), the camera ray of RayTracer.cu:666-667 /
// CUDA-Naive-Ray-Tracer RayTracer.cu:606-607. The reference hash (CreateShadowRayIndex :147-168,
// CreateReflectionRayIndex :170-198) used atan2(x, x), which is constant, so the key is redefined:
//   key = tag << (3g + 2b) | morton3(origin cell, g bits per axis) << 2b | morton2(octahedral bin)
// using only +, -, *, /, abs, min/max and truncation, so a CPU restatement reproduces it bit for bit.
#include "common.cuh"
#include "hash.cuh"
#include "kernels.h"

namespace rsh {

// ------------------------------------------------------------------ primary rays (tile order)
// Tile row r of the ray order is image tile row tile_row(r): from the middle outwards (m, m - 1, m + 1,
// m - 2, ... with m = rows / 2). Primary rays run longest in the view's centre band (on typical views the
// horizon, where rays travel far), so a persistent traversal starts them first instead of ending on them.
RSH_DEV uint32_t tile_row(uint32_t r, uint32_t rows) {
    const uint32_t m = rows >> 1;
    return (r & 1u) ? m - ((r + 1u) >> 1) : m + (r >> 1);
}

__global__ void k_raygen_primary(CameraP cam, uint32_t w, uint32_t h, uint32_t tiles_x, uint32_t tiles_y, uint32_t n,
                                 rsh_ray* rays, uint32_t* pixel_of_ray) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t tile = k >> 6, within = k & 63u;
    const uint32_t x = (tile % tiles_x) * 8u + (within & 7u);
    const uint32_t y = tile_row(tile / tiles_x, tiles_y) * 8u + (within >> 3);
    float4 o = make_float4(cam.eye[0], cam.eye[1], cam.eye[2], 0.0f);
    float4 d;
    if (x < w && y < h) {
        const float a = (float)x / (float)w - 0.5f;
        const float b = (float)y / (float)h - 0.5f;
        v3 q = mk3((cam.dir[0] + cam.right[0] * a) + cam.up[0] * b,
                   (cam.dir[1] + cam.right[1] * a) + cam.up[1] * b,
                   (cam.dir[2] + cam.right[2] * a) + cam.up[2] * b);
        v3 dn = norm3(q);
        d = make_float4(dn.x, dn.y, dn.z, __int_as_float(0x7f800000));  // tmax = +inf
        if (pixel_of_ray) pixel_of_ray[k] = y * w + x;
    } else {
        d = make_float4(0.0f, 0.0f, 1.0f, -1.0f);  // tmax < tmin: no ray
        if (pixel_of_ray) pixel_of_ray[k] = 0xFFFFFFFFu;
    }
    store_ray(rays, k, o, d);
}

cudaError_t launch_raygen_primary(const CameraP& cam, uint32_t w, uint32_t h, rsh_ray* rays,
                                  uint32_t* pixel_of_ray, cudaStream_t s) {
    const uint32_t tx = (w + 7u) / 8u, ty = (h + 7u) / 8u;
    const uint32_t n = tx * ty * 64u;
    if (n == 0) return cudaSuccess;
    k_raygen_primary<<<(n + 255u) / 256u, 256, 0, s>>>(cam, w, h, tx, ty, n, rays, pixel_of_ray);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ shadow rays
// Soft-shadow sample k (0..15) around light position lp for the shadow direction d: the reference's 4x4
// grid without its centre row/column (RayTracer.cu:1550-1599): k = i + 4 j, a = i (+1 from i = 2),
// b = j (+1 from j = 2), position lp + axis0 (a - 2) / 8 + axis1 (b - 2) / 8, axis0 = cross(e, d) for the
// axis e the reference picks by min(|dx|, max(|dy|, |dz|)), axis1 = cross(d, axis0) (neither normalised).
RSH_DEV v3 soft_sample_pos(v3 lp, v3 d, uint32_t k) {
    const uint32_t i = k & 3u, j = k >> 2;
    const float ca = (float)((int)(i + (i >= 2u ? 1u : 0u)) - 2), cb = (float)((int)(j + (j >= 2u ? 1u : 0u)) - 2);
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    const float mn = fminf(ax, fmaxf(ay, az));
    const v3 e = (ax == mn) ? v3{1.f, 0.f, 0.f} : (ay == mn) ? v3{0.f, 1.f, 0.f} : v3{0.f, 0.f, 1.f};
    const v3 a0 = cross3(e, d);
    const v3 a1 = cross3(d, a0);
    return v3{(lp.x + (a0.x * ca) * 0.125f) + (a1.x * cb) * 0.125f, (lp.y + (a0.y * ca) * 0.125f) + (a1.y * cb) * 0.125f,
              (lp.z + (a0.z * ca) * 0.125f) + (a1.z * cb) * 0.125f};
}

// The batch keys of a block's slots (BatchKeyOut): each slot's key and prefilled result, and the block's
// count of rays in one atomic. Every thread of the block calls it (it synchronises the block).
RSH_DEV void batch_key_out(const BatchKeyOut& bk, uint32_t slot, bool in_range, bool valid, float4 o, float4 d) {
    __shared__ uint32_t s_cnt;
    if (threadIdx.x == 0) s_cnt = 0u;
    __syncthreads();
    if (in_range) {
        bk.keys[slot] = valid ? bk.tag | (ray_hash(o.x, o.y, o.z, d.x, d.y, d.z, bk.hp, 0u) >> bk.drop)
                              : RSH_KEY_NONE;
        if (bk.flags) bk.flags[slot] = 0u;
        else bk.hits[slot] = RSH_HIT_NONE;
    }
    const uint32_t b = __ballot_sync(0xffffffffu, in_range && valid);
    if (lane_id() == 0 && b) atomicAdd(&s_cnt, (uint32_t)__popc(b));
    __syncthreads();
    if (threadIdx.x == 0 && s_cnt) atomicAdd(bk.count, s_cnt);
}

// One thread per pixel: the pixel's surface point and normal are read and the normal normalised once,
// then its V = L x S slots are written (slot = x + W (v + V y), RayTracer.cu:700-702 with S samples per
// light), each with the same arithmetic as a thread per slot would use. The block's rays are counted once
// (BatchKeyOut). The light positions are copied to shared memory first: indexing the parameter bank with
// the light number is a constant load with a register index, which the SM issues through its narrow
// address-divergence pipe, and three of those per slot made that pipe the kernel's bound. 12 blocks per SM
// (at most 40 registers, no spills) keep enough warps in flight to cover the surface reads.
__global__ void __launch_bounds__(128, 12) k_raygen_shadow(const float4* __restrict__ spos,
                                                           const float4* __restrict__ snrm, uint32_t w, uint32_t h,
                                                           LightsP lights, float eps, HashP hp, rsh_ray* rays,
                                                           uint32_t* keys, BatchKeyOut bk) {
    __shared__ uint32_t s_cnt;
    __shared__ float s_lp[8 * 3];
    const uint32_t L = lights.count, S = lights.samples ? lights.samples : 1u, V = L * S;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = pix < w * h;
    const bool a32 = (reinterpret_cast<uintptr_t>(rays) & 31u) == 0u;
    uint32_t nvalid = 0;
    if (threadIdx.x == 0) s_cnt = 0u;
    if (threadIdx.x < 3u * L) s_lp[threadIdx.x] = (&lights.pos[0][0])[threadIdx.x];
    __syncthreads();
    if (in_range) {
        const uint32_t y = pix / w, x = pix - y * w;
        const float4 p4 = __ldg(spos + pix);
        const bool surface = p4.w != 0.0f;
        const v3 p = mk3(p4);
        const v3 nn = surface ? norm3(mk3(__ldg(snrm + pix))) : v3{0.f, 0.f, 0.f};
        for (uint32_t v = 0; v < V; ++v) {
            const uint32_t slot = x + w * (v + V * y);
            const uint32_t l = S == 1u ? v : v / S, sm = S == 1u ? 0u : v % S;
            bool valid = false;
            float4 ro = make_float4(0.f, 0.f, 0.f, 0.f), rd = make_float4(0.f, 0.f, 0.f, -1.f);
            uint32_t key = RSH_KEY_NONE;
            if (surface) {
                const v3 lp = mk3(s_lp[3u * l], s_lp[3u * l + 1u], s_lp[3u * l + 2u]);
                const v3 vl = p - lp;
                const float len = len3(vl);
                const v3 d = v3{vl.x / len, vl.y / len, vl.z / len};
                const float diffuse = dot3(d, -nn);
                const float tmax = len - 2.0f * eps;
                if (diffuse > 0.0f && tmax > eps) {
                    v3 src = lp, dir = d;
                    float tm = tmax;
                    bool ok = true;
                    if (S > 1) {  // a sample of the 4x4 grid: its own origin, direction and interval
                        src = soft_sample_pos(lp, d, sm);
                        const v3 vs = p - src;
                        const float ls = len3(vs);
                        dir = v3{vs.x / ls, vs.y / ls, vs.z / ls};
                        tm = ls - 2.0f * eps;
                        ok = tm > eps;
                    }
                    if (ok) {
                        const v3 o = src + dir * eps;
                        ro = make_float4(o.x, o.y, o.z, eps);
                        rd = make_float4(dir.x, dir.y, dir.z, tm);
                        key = keys ? ray_hash(o.x, o.y, o.z, dir.x, dir.y, dir.z, hp, v) : 0u;
                        valid = true;
                    }
                }
            }
            // an empty slot holds an explicit no-ray (tmax < tmin) for consumers without keys
            store_ray32(rays, slot, ro, rd, a32);
            if (keys) keys[slot] = key;
            if (bk.keys) {
                bk.keys[slot] = valid ? bk.tag | (ray_hash(ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, bk.hp, 0u) >> bk.drop)
                                      : RSH_KEY_NONE;
                if (bk.flags) bk.flags[slot] = 0u;
                else bk.hits[slot] = RSH_HIT_NONE;
            }
            nvalid += valid ? 1u : 0u;
        }
    }
    if (bk.keys) {
        const uint32_t c = __reduce_add_sync(0xffffffffu, nvalid);
        if (lane_id() == 0 && c) atomicAdd(&s_cnt, c);
        __syncthreads();
        if (threadIdx.x == 0 && s_cnt) atomicAdd(bk.count, s_cnt);
    }
}

cudaError_t launch_raygen_shadow(const float4* spos, const float4* snrm, uint32_t w, uint32_t h,
                                 const LightsP& lights, float eps, const HashP& hp, rsh_ray* rays,
                                 uint32_t* keys, cudaStream_t s, const BatchKeyOut& bk) {
    const uint32_t n = w * h;
    if (n == 0 || lights.count == 0) return cudaSuccess;
    k_raygen_shadow<<<(n + 127u) / 128u, 128, 0, s>>>(spos, snrm, w, h, lights, eps, hp, rays, keys, bk);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ reflection rays
// Integer hash of (seed, slot, bounce) -> 32 random bits (PCG output permutation on an LCG step).
RSH_DEV uint32_t rng_next(uint32_t& state) {
    state = state * 747796405u + 2891336453u;
    uint32_t w = ((state >> ((state >> 28) + 4u)) ^ state) * 277803737u;
    return (w >> 22) ^ w;
}
// Uniform point on the unit sphere by Marsaglia's (1972) rejection method: sqrt only.
RSH_DEV v3 sphere_sample(uint32_t seed, uint32_t slot, uint32_t bounce) {
    uint32_t st = seed ^ (slot * 0x9E3779B9u) ^ (bounce * 0x85EBCA6Bu);
    rng_next(st);
    for (int it = 0; it < 32; ++it) {
        const float x1 = (float)(rng_next(st) >> 9) * (1.0f / 4194304.0f) - 1.0f;
        const float x2 = (float)(rng_next(st) >> 9) * (1.0f / 4194304.0f) - 1.0f;
        const float q = x1 * x1 + x2 * x2;
        if (q < 1.0f && q > 0.0f) {
            const float t = 2.0f * sqrtf(1.0f - q);
            return v3{x1 * t, x2 * t, 1.0f - 2.0f * q};
        }
    }
    return v3{0.0f, 0.0f, 1.0f};
}

__global__ void k_raygen_reflect(const float4* __restrict__ spos, const float4* __restrict__ snrm,
                                 const rsh_ray* __restrict__ prev, v3 eye, uint32_t n, float eps,
                                 float jitter, uint32_t seed, uint32_t bounce, HashP hp,
                                 rsh_ray* rays, uint32_t* keys, BatchKeyOut bk) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = slot < n;
    const bool a32 = (reinterpret_cast<uintptr_t>(rays) & 31u) == 0u;
    bool valid = false;
    float4 ro = make_float4(0.f, 0.f, 0.f, 0.f), rd = make_float4(0.f, 0.f, 0.f, -1.f);
    if (in_range) {
        const float4 p4 = __ldg(spos + slot);
        uint32_t key = RSH_KEY_NONE;
        if (p4.w != 0.0f) {
            const v3 p = mk3(p4);
            const v3 nn = norm3(mk3(__ldg(snrm + slot)));
            v3 i;
            if (prev) {
                float4 po, pd;
                load_ray(prev, slot, po, pd);
                i = mk3(pd);
            } else {
                i = norm3(p - eye);
            }
            const float k2 = 2.0f * dot3(nn, i);
            v3 r = i - nn * k2;  // reflect(i, n)
            if (jitter > 0.0f) {
                const v3 u = sphere_sample(seed, slot, bounce);
                r = r + u * jitter;
                const float rn = dot3(r, nn);
                if (rn < 0.0f) r = r - nn * (2.0f * rn);
            }
            r = norm3(r);
            if (r.x == r.x && r.y == r.y && r.z == r.z) {  // drop degenerate (NaN) directions
                const v3 o = p + r * eps;
                ro = make_float4(o.x, o.y, o.z, eps);
                rd = make_float4(r.x, r.y, r.z, __int_as_float(0x7f800000));
                store_ray32(rays, slot, ro, rd, a32);
                key = keys ? ray_hash(o.x, o.y, o.z, r.x, r.y, r.z, hp, 0u) : 0u;
                valid = true;
            }
        }
        // no ray: stored as such, also for the next bounce, which reads this array as its incident rays
        if (!valid) store_ray32(rays, slot, ro, rd, a32);
        if (keys) keys[slot] = key;
    }
    if (bk.keys) batch_key_out(bk, slot, in_range, valid, ro, rd);
}

cudaError_t launch_raygen_reflect(const float4* spos, const float4* snrm, const rsh_ray* prev,
                                  const float eye[3], uint32_t w, uint32_t h, float eps,
                                  float jitter, uint32_t seed, uint32_t bounce, const HashP& hp,
                                  rsh_ray* rays, uint32_t* keys, cudaStream_t s, const BatchKeyOut& bk) {
    const uint32_t n = w * h;
    if (n == 0) return cudaSuccess;
    k_raygen_reflect<<<(n + 255u) / 256u, 256, 0, s>>>(spos, snrm, prev, v3{eye[0], eye[1], eye[2]}, n,
                                                     eps, jitter, seed, bounce, hp, rays, keys, bk);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ refraction rays
// CreateRefractionRays (RayTracer.cu:793-842): direction refract(i, n, eta) (GLSL's formula: k = 1 -
// eta^2 (1 - (n.i)^2), t = eta i - (eta n.i + sqrt k) n; no ray when k < 0, total internal reflection),
// i = normalize(p - eye) or the incident ray, the surface normal as stored; renormalised, origin offset by
// eps, interval (eps, inf). The reference creates these rays but never casts them.
__global__ void k_raygen_refract(const float4* __restrict__ spos, const float4* __restrict__ snrm,
                                 const rsh_ray* __restrict__ prev, v3 eye, uint32_t n, float eps, float eta,
                                 HashP hp, rsh_ray* rays, uint32_t* keys) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n) return;
    const float4 p4 = __ldg(spos + slot);
    uint32_t key = RSH_KEY_NONE;
    if (p4.w != 0.0f) {
        const v3 p = mk3(p4);
        const v3 nn = norm3(mk3(__ldg(snrm + slot)));
        v3 i;
        if (prev) {
            float4 po, pd;
            load_ray(prev, slot, po, pd);
            i = mk3(pd);
        } else {
            i = norm3(p - eye);
        }
        const float d = dot3(nn, i);
        const float k = 1.0f - eta * eta * (1.0f - d * d);
        if (k >= 0.0f) {
            const v3 t = norm3(i * eta - nn * (eta * d + sqrtf(k)));
            if (t.x == t.x && t.y == t.y && t.z == t.z) {
                const v3 o = p + t * eps;
                store_ray(rays, slot, make_float4(o.x, o.y, o.z, eps),
                          make_float4(t.x, t.y, t.z, __int_as_float(0x7f800000)));
                key = ray_hash(o.x, o.y, o.z, t.x, t.y, t.z, hp, 0u);
            }
        }
    }
    if (key == RSH_KEY_NONE)
        store_ray(rays, slot, make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, -1.f));
    keys[slot] = key;
}

cudaError_t launch_raygen_refract(const float4* spos, const float4* snrm, const rsh_ray* prev, const float eye[3],
                                  uint32_t w, uint32_t h, float eps, float eta, const HashP& hp, rsh_ray* rays,
                                  uint32_t* keys, cudaStream_t s) {
    const uint32_t n = w * h;
    if (n == 0) return cudaSuccess;
    k_raygen_refract<<<(n + 255u) / 256u, 256, 0, s>>>(spos, snrm, prev, v3{eye[0], eye[1], eye[2]}, n, eps, eta,
                                                     hp, rays, keys);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ hash of given rays
__global__ void k_hash(const rsh_ray* __restrict__ rays, uint32_t n, HashP hp, uint32_t tag,
                       uint32_t* keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 o, d;
    load_ray(rays, i, o, d);
    keys[i] = (d.w > o.w) ? ray_hash(o.x, o.y, o.z, d.x, d.y, d.z, hp, tag) : RSH_KEY_NONE;
}

cudaError_t launch_hash(const rsh_ray* rays, uint32_t n, const HashP& hp, uint32_t tag,
                        uint32_t* keys, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_hash<<<(n + 255u) / 256u, 256, 0, s>>>(rays, n, hp, tag, keys);
    note_launch();
    return cudaGetLastError();
}

// Segmented: binary search of the segment of ray i; the key's tag is the segment index placed at
// bit tag_shift (above every segment's hash bits).
__global__ void k_hash_segments(const rsh_ray* __restrict__ rays, uint32_t n,
                                const uint32_t* __restrict__ seg_start, uint32_t nseg,
                                const HashP* __restrict__ hps, uint32_t tag_shift, uint32_t* keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t lo = 0, hi = nseg;  // find last s with seg_start[s] <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(seg_start + mid) <= i) lo = mid; else hi = mid;
    }
    float4 o, d;
    load_ray(rays, i, o, d);
    uint32_t key = RSH_KEY_NONE;
    if (d.w > o.w) {
        const HashP hp = hps[lo];
        key = (lo << tag_shift) | ray_hash(o.x, o.y, o.z, d.x, d.y, d.z, hp, 0u);
    }
    keys[i] = key;
}

cudaError_t launch_hash_segments(const rsh_ray* rays, uint32_t n, const uint32_t* seg_start,
                                 uint32_t nseg, const HashP* hps_dev, uint32_t tag_shift,
                                 uint32_t* keys, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_hash_segments<<<(n + 255u) / 256u, 256, 0, s>>>(rays, n, seg_start, nseg, hps_dev, tag_shift,
                                                    keys);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ fills
__global__ void k_fill_u32(uint32_t* p, uint32_t v, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}
__global__ void k_fill_u64(unsigned long long* p, unsigned long long v, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}
cudaError_t launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    size_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_fill_u32<<<(unsigned)blocks, 256, 0, s>>>(p, v, n);
    note_launch();
    return cudaGetLastError();
}
cudaError_t launch_fill_u64(unsigned long long* p, unsigned long long v, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    size_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_fill_u64<<<(unsigned)blocks, 256, 0, s>>>(p, v, n);
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
