// Packet-node vs sphere test and the watertight ray/triangle test, shared by the traversal, the
// intersection kernels and the fused persistent kernel.
#pragma once
#include "common.cuh"

namespace rsh {

// A ray-hierarchy node held in registers.
struct NodeR {
    float cx, cy, cz, r;
    float ax, ay, az, cs;
    float sn, reach;
    uint32_t first, count;
};
RSH_DEV NodeR load_node(const rsh_node* nodes, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    NodeR n;
    n.cx = a.x;
    n.cy = a.y;
    n.cz = a.z;
    n.r = a.w;
    n.ax = b.x;
    n.ay = b.y;
    n.az = b.z;
    n.cs = b.w;
    n.sn = c.x;
    n.reach = c.y;
    n.first = __float_as_uint(c.z);
    n.count = __float_as_uint(c.w);
    return n;
}

// Can any ray of node `p` reach sphere s = (centre, radius)? Conservative: the rays' origins lie in
// the node sphere and their directions in the cone, so every reachable point lies in the node sphere
// swept along the cone (Minkowski sum of the sphere with the infinite cone at its centre) and within
// `reach` of the centre. The line distance perp*cos - t*sin from the sphere centre to the cone
// boundary never exceeds the true distance to the cone (RayTracer.cu:283-298 uses the same bound
// without the reach term). A relative slack of 1e-5 absorbs FP32 rounding.
RSH_DEV bool node_hits_sphere(const NodeR& p, float4 s) {
    const float vx = s.x - p.cx, vy = s.y - p.cy, vz = s.z - p.cz;
    const float dd = (vx * vx + vy * vy) + vz * vz;
    const float dist = sqrtf(dd);
    const float rr = p.r + s.w;
    const float slack = (dist + rr) * 1e-5f;
    if (dist - s.w > p.reach + slack) return false;
    if (p.cs > 0.0f) {
        const float t = (vx * p.ax + vy * p.ay) + vz * p.az;
        const float wx = vy * p.az - vz * p.ay;
        const float wy = vz * p.ax - vx * p.az;
        const float wz = vx * p.ay - vy * p.ax;
        const float perp = sqrtf((wx * wx + wy * wy) + wz * wz);
        if (perp * p.cs - t * p.sn > rr + slack) return false;
    }
    return true;
}

// Can ray (o, d, [tmin, tmax]) touch sphere s? Conservative per-ray test: the squared distance from the
// sphere centre to the ray line (through a cross product) against the squared inflated radius, and the
// sphere's parameter interval along the ray against [tmin, tmax]. The inflation is 1e-5 of the L1 distance
// plus radius (an upper bound of the Euclidean one), which absorbs FP32 rounding and |d| = 1 +- 1e-7.
// No square roots. A miss here implies every triangle inside the sphere is missed.
RSH_DEV bool ray_hits_sphere(float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float tmax,
                             float4 s) {
    const float vx = s.x - ox, vy = s.y - oy, vz = s.z - oz;
    const float t = (vx * dx + vy * dy) + vz * dz;
    const float wx = vy * dz - vz * dy;
    const float wy = vz * dx - vx * dz;
    const float wz = vx * dy - vy * dx;
    const float perp2 = (wx * wx + wy * wy) + wz * wz;
    const float slack = (((fabsf(vx) + fabsf(vy)) + fabsf(vz)) + s.w) * 1e-5f;
    const float r = s.w + slack;
    if (perp2 > r * r) return false;
    if (t + r < tmin) return false;
    if (t - r > tmax) return false;
    return true;
}

// ---------------------------------------------------------------- watertight ray/triangle test
// Woop, Benthin & Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013: shear the triangle
// into the ray's frame (largest |d| axis becomes z), evaluate the 2-D edge functions, fall back to
// double precision when one is exactly zero. Hit iff tmin < t < tmax with t = T / det (IEEE divide).
struct RayWT {
    float ox, oy, oz;
    float sx, sy, sz;
    int kx, ky, kz;
    float tmin, tmax;
};
RSH_DEV float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

RSH_DEV RayWT wt_setup(float4 o, float4 d) {
    RayWT r;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dz = comp(d.x, d.y, d.z, kz);
    if (dz < 0.0f) {
        const int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.sx = comp(d.x, d.y, d.z, kx) / dz;
    r.sy = comp(d.x, d.y, d.z, ky) / dz;
    r.sz = 1.0f / dz;
    r.ox = o.x;
    r.oy = o.y;
    r.oz = o.z;
    r.tmin = o.w;
    r.tmax = d.w;
    return r;
}

RSH_DEV bool wt_hit(const RayWT& r, float4 p0, float4 p1, float4 p2, float& t_out) {
    const float A0 = p0.x - r.ox, A1 = p0.y - r.oy, A2 = p0.z - r.oz;
    const float B0 = p1.x - r.ox, B1 = p1.y - r.oy, B2 = p1.z - r.oz;
    const float C0 = p2.x - r.ox, C1 = p2.y - r.oy, C2 = p2.z - r.oz;
    const float Akz = comp(A0, A1, A2, r.kz), Bkz = comp(B0, B1, B2, r.kz), Ckz = comp(C0, C1, C2, r.kz);
    const float Ax = comp(A0, A1, A2, r.kx) - r.sx * Akz;
    const float Ay = comp(A0, A1, A2, r.ky) - r.sy * Akz;
    const float Bx = comp(B0, B1, B2, r.kx) - r.sx * Bkz;
    const float By = comp(B0, B1, B2, r.ky) - r.sy * Bkz;
    const float Cx = comp(C0, C1, C2, r.kx) - r.sx * Ckz;
    const float Cy = comp(C0, C1, C2, r.ky) - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
    const float T = (U * Az + V * Bz) + W * Cz;
    const float t = T / det;
    t_out = t;
    return t > r.tmin && t < r.tmax;
}

RSH_DEV unsigned long long hit_key(float t, uint32_t tri) {
    return ((unsigned long long)__float_as_uint(t) << 32) | (unsigned long long)tri;
}

// ---------------------------------------------------------------- object-tree child ranges
// Children of object node (L, idx) at level L-1: [first, first + cnt). L == levels is the virtual root
// over the top level. Level l's child-range starts sit at kids[lvl_off[l] + l].
RSH_DEV void node_children(const uint32_t* __restrict__ kids, const uint32_t* lvl_off, const uint32_t* lvl_size,
                           uint32_t levels, uint32_t L, uint32_t idx, uint32_t& first, uint32_t& cnt) {
    if (L == levels) {
        first = 0u;
        cnt = lvl_size[L - 1];
        return;
    }
    const uint32_t* k = kids + lvl_off[L] + L + idx;
    first = __ldg(k);
    cnt = __ldg(k + 1) - first;
}
// Triangles of cluster c: [t0, t1).
RSH_DEV void cluster_tris(const uint32_t* __restrict__ kids, uint32_t c, uint32_t& t0, uint32_t& t1) {
    t0 = __ldg(kids + c);
    t1 = __ldg(kids + c + 1);
}

}  // namespace rsh
