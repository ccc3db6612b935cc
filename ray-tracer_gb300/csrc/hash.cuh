// The 32-bit ray hash (shared by ray generation and the batched form's segmented hash).
//   key = tag << (3g + 2b) | morton3(origin cell, g bits per axis) << 2b | morton2(octahedral bin, b bits)
// Only +, -, *, /, abs, min/max and truncation: a CPU restatement reproduces it bit for bit.
#pragma once
#include "common.cuh"
#include "kernels.h"

namespace rsh {

RSH_DEV uint32_t ray_hash(float ox, float oy, float oz, float dx, float dy, float dz, const HashP& hp,
                          uint32_t tag) {
    const float gmax = (float)((1u << hp.grid_bits) - 1u);
    float fx = (ox - hp.lo[0]) * hp.scale[0];
    float fy = (oy - hp.lo[1]) * hp.scale[1];
    float fz = (oz - hp.lo[2]) * hp.scale[2];
    fx = fminf(fmaxf(fx, 0.0f), gmax);
    fy = fminf(fmaxf(fy, 0.0f), gmax);
    fz = fminf(fmaxf(fz, 0.0f), gmax);
    const uint32_t cell = (spread3((uint32_t)fx) << 2) | (spread3((uint32_t)fy) << 1) |
                          spread3((uint32_t)fz);
    // octahedral map of the direction (L1-normalised; lower hemisphere folded)
    const float s = (fabsf(dx) + fabsf(dy)) + fabsf(dz);
    float px = dx / s;
    float py = dy / s;
    if (dz < 0.0f) {
        const float qx = 1.0f - fabsf(py);
        const float qy = 1.0f - fabsf(px);
        px = (px >= 0.0f) ? qx : -qx;
        py = (py >= 0.0f) ? qy : -qy;
    }
    const uint32_t B = 1u << hp.dir_log2;
    const float half_b = 0.5f * (float)B;
    const float bmax = (float)(B - 1u);
    float u = (px + 1.0f) * half_b;
    float v = (py + 1.0f) * half_b;
    u = fminf(fmaxf(u, 0.0f), bmax);
    v = fminf(fmaxf(v, 0.0f), bmax);
    const uint32_t dir = (spread2((uint32_t)u) << 1) | spread2((uint32_t)v);
    const uint32_t dbits = 2u * hp.dir_log2;
    const uint32_t hbits = 3u * hp.grid_bits + dbits;
    return (tag << hbits) | (cell << dbits) | dir;
}

}  // namespace rsh
