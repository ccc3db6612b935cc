// Shared device helpers for the sm_103a ray-space-hierarchy kernels.
//
// Numerics: the library is compiled with -fmad=false, so every a*b+c below is two rounded IEEE
// operations unless written as an explicit fmaf(). Hash keys, run heads, hierarchy nodes and
// intersection results are therefore reproducible bit for bit by a CPU restatement compiled with
// -ffp-contract=off. Division and square root use the IEEE-rounded defaults (-prec-div/-prec-sqrt).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rsh.h"

#define RSH_DEV __device__ __forceinline__

// ------------------------------------------------------------------ small vector math (own)
struct v3 {
    float x, y, z;
};
RSH_DEV v3 mk3(float x, float y, float z) { return v3{x, y, z}; }
RSH_DEV v3 mk3(float4 a) { return v3{a.x, a.y, a.z}; }
RSH_DEV v3 operator+(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
RSH_DEV v3 operator-(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
RSH_DEV v3 operator*(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
RSH_DEV v3 operator-(v3 a) { return v3{-a.x, -a.y, -a.z}; }
// dot as ((x*x + y*y) + z*z): the fixed evaluation order the CPU restatement uses
RSH_DEV float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
RSH_DEV v3 cross3(v3 a, v3 b) {
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
RSH_DEV float len3(v3 a) { return sqrtf(dot3(a, a)); }
// normalize by three IEEE divisions (not a reciprocal multiply), reproducible on the host
RSH_DEV v3 norm3(v3 a) {
    float l = len3(a);
    return v3{a.x / l, a.y / l, a.z / l};
}

// ------------------------------------------------------------------ ray storage
// rsh_ray is 32 bytes: two float4 halves, loaded with 128-bit accesses.
RSH_DEV void load_ray(const rsh_ray* rays, uint32_t i, float4& o, float4& d) {
    const float4* p = reinterpret_cast<const float4*>(rays) + 2ull * i;
    o = __ldg(p);
    d = __ldg(p + 1);
}
RSH_DEV void store_ray(rsh_ray* rays, uint32_t i, float4 o, float4 d) {
    float4* p = reinterpret_cast<float4*>(rays) + 2ull * i;
    p[0] = o;
    p[1] = d;
}
// The same ray as one 256-bit store (st.global.v8.f32, sm_100 and later): each lane writes its whole
// 32-byte sector in one instruction. Only for an array whose base is 32-byte aligned (a32, checked by the
// caller once per thread); otherwise the two 16-byte stores above.
RSH_DEV void store_ray32(rsh_ray* rays, uint32_t i, float4 o, float4 d, bool a32) {
    if (a32) {
        float* p = reinterpret_cast<float*>(rays) + 8ull * i;
        asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(o.x), "f"(o.y),
                     "f"(o.z), "f"(o.w), "f"(d.x), "f"(d.y), "f"(d.z), "f"(d.w)
                     : "memory");
    } else {
        store_ray(rays, i, o, d);
    }
}

// ------------------------------------------------------------------ device error word
// Bounded device waits and overflow checks report here (never __trap()); the host reads it back with
// rsh_check_device_errors. Bits: 1 = look-back timeout, 2 = overflow.
#ifndef RSH_DEVERR_TIMEOUT
#define RSH_DEVERR_TIMEOUT 1u
#define RSH_DEVERR_OVERFLOW 2u
#endif
#define RSH_SPIN_LIMIT (1u << 22)   // polls before a look-back wait gives up (~0.1-1 s)

RSH_DEV void raise_device_error(uint32_t* err, uint32_t bit) {
    if (err) atomicOr(err, bit);
}

RSH_DEV uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
RSH_DEV void st_release_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
RSH_DEV unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
RSH_DEV void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
RSH_DEV void st_relaxed_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
RSH_DEV uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
RSH_DEV unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

RSH_DEV uint32_t lane_id() { return threadIdx.x & 31u; }
RSH_DEV uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// device count helper: n = *d_count when given (clamped to n_max), else n_max
RSH_DEV uint32_t dev_count(const uint32_t* d_count, uint32_t n_max) {
    if (!d_count) return n_max;
    uint32_t n = *d_count;
    return n < n_max ? n : n_max;
}

// ------------------------------------------------------------------ Morton interleaving
RSH_DEV uint32_t spread3(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
RSH_DEV uint32_t spread2(uint32_t v) {  // 16 bits -> every second bit
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// ------------------------------------------------------------------ geometry access
// Scene triangles in cluster order: 3 float4 per triangle; w of vertex 0 carries the original id.
struct TriSoA {
    const float4* v;   // 3 per triangle
};
