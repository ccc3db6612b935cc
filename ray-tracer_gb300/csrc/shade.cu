// Hit resolve (hit point + interpolated normal -> surface buffer) and Blinn-Phong shading.
//
// Reference: the resolve half of ColorReflectionRay / ColorAndCreateReflectionRay
// (RayTracer.cu:1806-1843: re-intersect the winning triangle, hit point, area-ratio barycentric
// normal) and the shading of ColorPrimaryShadowRay (:1616-1709) / ColorReflectionRay (:1845-1880):
// Blinn-Phong per unoccluded light with attenuation 1 / (0.75 + 0.0005 d + 0.00005 d^2) (:1667).
// The surface buffer replaces the GL G-buffer: position.w = 1 marks a surface, normal.w carries the
// material id bits.
#include "common.cuh"
#include "kernels.h"

namespace rsh {

__global__ void k_resolve(const float4* __restrict__ pos, const float4* __restrict__ nrm,
                          const uint32_t* __restrict__ mat_ids, const rsh_ray* __restrict__ rays,
                          const unsigned long long* __restrict__ hits,
                          const uint32_t* __restrict__ pixel_of_ray, uint32_t n, float4* spos,
                          float4* snrm) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t pix = pixel_of_ray ? __ldg(pixel_of_ray + k) : k;
    if (pix == 0xFFFFFFFFu) return;
    const unsigned long long h = __ldg(hits + k);
    if (h == RSH_HIT_NONE) {
        spos[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        snrm[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const uint32_t tri = (uint32_t)h;
    const float t = __uint_as_float((uint32_t)(h >> 32));
    float4 o, d;
    load_ray(rays, k, o, d);
    const v3 p = v3{o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
    const v3 a = mk3(__ldg(pos + 3ull * tri)), b = mk3(__ldg(pos + 3ull * tri + 1)),
             c = mk3(__ldg(pos + 3ull * tri + 2));
    const float abc = len3(cross3(b - a, c - a));
    const float pbc = len3(cross3(b - p, c - p));
    const float pca = len3(cross3(a - p, c - p));
    const float b0 = pbc / abc, b1 = pca / abc, b2 = (1.0f - b0) - b1;
    const v3 n0 = mk3(__ldg(nrm + 3ull * tri)), n1 = mk3(__ldg(nrm + 3ull * tri + 1)),
             n2 = mk3(__ldg(nrm + 3ull * tri + 2));
    const v3 nn = v3{(n0.x * b0 + n1.x * b1) + n2.x * b2, (n0.y * b0 + n1.y * b1) + n2.y * b2,
                     (n0.z * b0 + n1.z * b1) + n2.z * b2};
    const uint32_t mid = mat_ids ? __ldg(mat_ids + tri) : 0u;
    spos[pix] = make_float4(p.x, p.y, p.z, 1.0f);
    snrm[pix] = make_float4(nn.x, nn.y, nn.z, __uint_as_float(mid));
}

cudaError_t launch_resolve(const float4* tris_orig_pos, const float4* tris_orig_nrm,
                           const uint32_t* mat_ids, const rsh_ray* rays, const unsigned long long* hits,
                           const uint32_t* pixel_of_ray, uint32_t n, float4* spos, float4* snrm,
                           cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_resolve<<<(n + 255) / 256, 256, 0, s>>>(tris_orig_pos, tris_orig_nrm, mat_ids, rays, hits,
                                              pixel_of_ray, n, spos, snrm);
    note_launch();
    return cudaGetLastError();
}

// Soft-shadow weight of sample k (RayTracer.cu:1680-1690): inner four 0.55/16, corners 0.5375/16,
// edges 0.525/16.
RSH_DEV float soft_weight(uint32_t k) {
    if (k == 5 || k == 6 || k == 9 || k == 10) return 0.55f / 16.0f;
    if (k == 0 || k == 3 || k == 12 || k == 15) return 0.5375f / 16.0f;
    return 0.525f / 16.0f;
}

// The lights are copied to shared memory first: indexing the parameter bank with the light number would
// be a constant load with a register index per field, issued through the SM's narrow address-divergence
// pipe.
__global__ void k_shade(ShadeArgs a) {
    __shared__ rsh_light s_light[8];
    static_assert(sizeof(rsh_light) == 8 * sizeof(float), "rsh_light is 8 floats");
    if (threadIdx.x < 8u * a.lights)
        reinterpret_cast<float*>(s_light)[threadIdx.x] = reinterpret_cast<const float*>(a.light)[threadIdx.x];
    __syncthreads();
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= a.w * a.h) return;
    float4 acc = a.bounce == 0 ? make_float4(0.f, 0.f, 0.f, 1.f) : a.accum[pix];
    const float4 p4 = a.spos[pix];
    if (p4.w != 0.0f && acc.w > 0.0f) {
        const v3 p = mk3(p4);
        const float4 n4 = a.snrm[pix];
        const v3 n = norm3(mk3(n4));
        uint32_t mid = __float_as_uint(n4.w);
        if (mid >= a.material_count) mid = 0;
        const rsh_material m = a.materials[mid];
        v3 inc;
        if (a.incident) {
            float4 o, d;
            load_ray(a.incident, pix, o, d);
            inc = mk3(d);
        } else {
            inc = norm3(p - v3{a.eye[0], a.eye[1], a.eye[2]});
        }
        const uint32_t x = pix % a.w, y = pix / a.w;
        float cr = 0.f, cg = 0.f, cb = 0.f;
        const uint32_t S = a.samples ? a.samples : 1u;
        for (uint32_t l = 0; l < a.lights; ++l) {
            float factor = 1.0f;
            if (S == 1) {
                const uint32_t slot = x + a.w * (l + a.lights * y);
                if (a.shadow && a.shadow[slot] == RSH_OCCLUDED) continue;
            } else if (a.shadow) {
                // soft shadows (RayTracer.cu:1680-1696): weighted unoccluded samples, log2(1 + 2 sum)
                float sf = 0.0f;
                for (uint32_t k = 0; k < S; ++k)
                    if (a.shadow[x + a.w * ((l * S + k) + a.lights * S * y)] != RSH_OCCLUDED) sf += soft_weight(k);
                factor = log2f(1.0f + sf * 2.0f);
            }
            const rsh_light& L = s_light[l];
            v3 ld = v3{L.position[0], L.position[1], L.position[2]} - p;
            const float dist = len3(ld);
            ld = v3{ld.x / dist, ld.y / dist, ld.z / dist};
            const float att = 1.0f / (0.75f + dist * 0.0005f + dist * dist * 0.00005f);
            const float diff = fminf(fmaxf(dot3(ld, n), 0.0f), 1.0f);
            if (diff > 0.0f) {
                const v3 hv = norm3(ld - inc);
                const float sp = fminf(fmaxf(powf(fmaxf(dot3(hv, n), 0.0f), m.specular[3]), 0.0f), 1.0f);
                const float kd = diff * L.diffuse_intensity * att * factor, ks = sp * L.specular_intensity * att * factor;
                cr += (m.diffuse[0] * kd + m.specular[0] * ks) * L.color[0];
                cg += (m.diffuse[1] * kd + m.specular[1] * ks) * L.color[1];
                cb += (m.diffuse[2] * kd + m.specular[2] * ks) * L.color[2];
            }
        }
        acc.x += acc.w * cr;
        acc.y += acc.w * cg;
        acc.z += acc.w * cb;
        acc.w *= m.diffuse[3];  // reflectance carried to the next bounce
    } else if (a.bounce > 0) {
        acc.w = 0.0f;
    } else {
        acc.w = 0.0f;
    }
    a.accum[pix] = acc;
}

cudaError_t launch_shade(const ShadeArgs& a, cudaStream_t s) {
    const uint32_t n = a.w * a.h;
    if (n == 0) return cudaSuccess;
    k_shade<<<(n + 255) / 256, 256, 0, s>>>(a);
    note_launch();
    return cudaGetLastError();
}

__global__ void k_pack(const float4* __restrict__ acc, uint32_t n, uint32_t* rgba) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 c = acc[i];
    const uint32_t r = (uint32_t)fminf(fmaxf(c.x * 255.0f, 0.0f), 255.0f);
    const uint32_t g = (uint32_t)fminf(fmaxf(c.y * 255.0f, 0.0f), 255.0f);
    const uint32_t b = (uint32_t)fminf(fmaxf(c.z * 255.0f, 0.0f), 255.0f);
    rgba[i] = r | (g << 8) | (b << 16) | (255u << 24);
}

cudaError_t launch_pack_rgba(const float4* accum, uint32_t n, uint32_t* rgba, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_pack<<<(n + 255) / 256, 256, 0, s>>>(accum, n, rgba);
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
