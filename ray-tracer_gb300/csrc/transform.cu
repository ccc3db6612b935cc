// Per-frame object transforms: UpdateVertex (RayTracer.cu:448-511) and the bounds the hash and the object
// hierarchy are built over.
//
// Reference: every vertex is multiplied by its object's model matrix and every normal by its object's
// normal matrix (row-major 4x4, out[i] = sum_j M[4i + j] v[j], summed in j order), normals renormalised;
// the per-object bounding spheres follow (UpdateBoundingSphere, :513-570). Here the transform starts from
// the rest pose kept at upload (no error accumulates over frames), and the object-sphere hierarchy is
// rebuilt from the moved triangles instead of moving one sphere per object.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace rsh {

RSH_DEV float4 mat4_apply(const float* __restrict__ m, float4 v) {
    float o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float s = 0.0f;
        s += __ldg(m + 4 * i + 0) * v.x;
        s += __ldg(m + 4 * i + 1) * v.y;
        s += __ldg(m + 4 * i + 2) * v.z;
        s += __ldg(m + 4 * i + 3) * v.w;
        o[i] = s;
    }
    return make_float4(o[0], o[1], o[2], o[3]);
}

// One thread per vertex (3 per triangle). w of a position keeps its rest value; normals get w = 0.
__global__ void k_transform(const float4* __restrict__ pos_rest, const float4* __restrict__ nrm_rest,
                            const uint32_t* __restrict__ obj, uint32_t n_vertices, uint32_t n_objects,
                            const float* __restrict__ model, const float* __restrict__ normal,
                            float4* __restrict__ pos, float4* __restrict__ nrm) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n_vertices) return;
    uint32_t id = __ldg(obj + x / 3);
    if (id >= n_objects) id = 0;
    const float4 p = __ldg(pos_rest + x);
    const float4 q = mat4_apply(model + 16ull * id, p);
    pos[x] = make_float4(q.x, q.y, q.z, p.w);
    const float4 nr = __ldg(nrm_rest + x);
    const float4 m = mat4_apply((normal ? normal : model) + 16ull * id, make_float4(nr.x, nr.y, nr.z, nr.w));
    const v3 u = norm3(v3{m.x, m.y, m.z});
    nrm[x] = make_float4(u.x, u.y, u.z, 0.0f);
}

// Exact min / max of the vertex coordinates: per-block partials, then one block over them.
__global__ void k_bounds_partial(const float4* __restrict__ pos, uint32_t n_vertices, float* __restrict__ part) {
    __shared__ float s[6][256];
    const float inf = __int_as_float(0x7f800000);
    float mn[3] = {inf, inf, inf}, mx[3] = {-inf, -inf, -inf};
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n_vertices; x += gridDim.x * blockDim.x) {
        const float4 p = __ldg(pos + x);
        mn[0] = fminf(mn[0], p.x), mn[1] = fminf(mn[1], p.y), mn[2] = fminf(mn[2], p.z);
        mx[0] = fmaxf(mx[0], p.x), mx[1] = fmaxf(mx[1], p.y), mx[2] = fmaxf(mx[2], p.z);
    }
    for (int a = 0; a < 3; ++a) {
        s[a][threadIdx.x] = mn[a];
        s[3 + a][threadIdx.x] = mx[a];
    }
    __syncthreads();
    for (uint32_t st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st)
            for (int a = 0; a < 3; ++a) {
                s[a][threadIdx.x] = fminf(s[a][threadIdx.x], s[a][threadIdx.x + st]);
                s[3 + a][threadIdx.x] = fmaxf(s[3 + a][threadIdx.x], s[3 + a][threadIdx.x + st]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_bounds_final(const float* __restrict__ part, uint32_t blocks, float* __restrict__ out) {
    if (threadIdx.x >= 6) return;
    const bool is_min = threadIdx.x < 3;
    float v = part[threadIdx.x];
    for (uint32_t b = 1; b < blocks; ++b) {
        const float q = part[6 * b + threadIdx.x];
        v = is_min ? fminf(v, q) : fmaxf(v, q);
    }
    out[threadIdx.x] = v;
}

cudaError_t launch_transform(const float4* pos_rest, const float4* nrm_rest, const uint32_t* obj, uint32_t tri_count,
                             uint32_t n_objects, const float* model, const float* normal, float4* pos, float4* nrm,
                             cudaStream_t s) {
    const uint32_t nv = 3 * tri_count;
    if (nv == 0) return cudaSuccess;
    k_transform<<<(nv + 255) / 256, 256, 0, s>>>(pos_rest, nrm_rest, obj, nv, n_objects, model, normal, pos, nrm);
    note_launch();
    return cudaGetLastError();
}

size_t bounds_scratch_bytes() { return 6 * 4 * 608 + 64; }

cudaError_t launch_bounds(const float4* pos, uint32_t tri_count, void* scratch, float* out6, cudaStream_t s) {
    const uint32_t nv = 3 * tri_count;
    const uint32_t blocks = std::min<uint32_t>(608u, (nv + 255) / 256 > 0 ? (nv + 255) / 256 : 1u);
    float* part = static_cast<float*>(scratch);
    k_bounds_partial<<<blocks, 256, 0, s>>>(pos, nv, part);
    note_launch();
    k_bounds_final<<<1, 32, 0, s>>>(part, blocks, out6);
    note_launch();
    return cudaGetLastError();
}

}  // namespace rsh
