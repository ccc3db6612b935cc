/*
 * rsh_oracle.cpp — CPU ORACLE for the ray-space-hierarchy secondary-ray path. TEST INFRASTRUCTURE ONLY:
 * imported by tests/, by __graft_entry__.smoke() as the checker, and by bench.py's cpu_baseline /
 * reference legs. The product library never links or calls it.
 *
 * Parity: the reference (nuno-tiago-reis/ray-tracer, projects/CUDA-Engine) cannot be built here (CUDA 6.5
 * headers, texture references, Win32/GL) and ships no CPU path, no golden vectors and no known-answer
 * tests for this path. This file restates the reference's algorithm stage by stage, citing the lines it
 * follows, with the arithmetic the GPU port defines where the reference is replaced (hash, conservative
 * nodes, watertight test, 64-bit hit key). The brute-force any/closest hit (as CUDA-Naive-Engine,
 * RayTracer.cu:276-291 and :344-360) is the independent end-to-end check. Parity against the reference's
 * own outputs is UNPINNED: only order-of-magnitude sanity ranges exist (output/tests/configuration-n8).
 *
 * Numerics: compile with -ffp-contract=off (no FMA contraction); every expression below uses the same
 * operation order as the GPU kernels so that keys, run heads, permutations, nodes, candidates and hit
 * records are reproduced bit for bit.
 */
#include <omp.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace {

const uint32_t KEY_NONE = 0xFFFFFFFFu;
const uint64_t HIT_NONE = 0xFFFFFFFFFFFFFFFFull;
const uint32_t OCCLUDED = 0xFFFFFFFFu;
const float INF = std::numeric_limits<float>::infinity();

struct V3 {
    float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) {
    const float l = length(a);
    return V3{a.x / l, a.y / l, a.z / l};
}

struct Ray {  // same 32-byte layout as rsh_ray
    float o[3];
    float tmin;
    float d[3];
    float tmax;
};
struct Node {  // same 48-byte layout as rsh_node
    float c[3];
    float radius;
    float axis[3];
    float cos_spread;
    float sin_spread;
    float reach;
    uint32_t first;
    uint32_t count;
};
struct HashP {
    float lo[3], scale[3];
    uint32_t g, b;
};

inline uint32_t spread3(uint32_t v) {
    uint32_t r = 0;
    for (int i = 0; i < 10; ++i) r |= ((v >> i) & 1u) << (3 * i);
    return r;
}
inline uint32_t spread2(uint32_t v) {
    uint32_t r = 0;
    for (int i = 0; i < 16; ++i) r |= ((v >> i) & 1u) << (2 * i);
    return r;
}

// 32-bit ray hash: tag | morton3(origin cell) | morton2(octahedral direction bin). Replaces
// CreateShadowRayIndex / CreateReflectionRayIndex (RayTracer.cu:147-198), whose atan2(x, x) is constant.
uint32_t ray_hash(const float o[3], const float d[3], const HashP& hp, uint32_t tag) {
    const float gmax = (float)((1u << hp.g) - 1u);
    uint32_t c[3];
    for (int i = 0; i < 3; ++i) {
        float f = (o[i] - hp.lo[i]) * hp.scale[i];
        f = std::fmin(std::fmax(f, 0.0f), gmax);
        c[i] = (uint32_t)f;
    }
    const uint32_t cell = (spread3(c[0]) << 2) | (spread3(c[1]) << 1) | spread3(c[2]);
    const float s = (std::fabs(d[0]) + std::fabs(d[1])) + std::fabs(d[2]);
    float px = d[0] / s, py = d[1] / s;
    if (d[2] < 0.0f) {
        const float qx = 1.0f - std::fabs(py), qy = 1.0f - std::fabs(px);
        px = (px >= 0.0f) ? qx : -qx;
        py = (py >= 0.0f) ? qy : -qy;
    }
    const uint32_t B = 1u << hp.b;
    const float half_b = 0.5f * (float)B, bmax = (float)(B - 1u);
    float u = (px + 1.0f) * half_b, v = (py + 1.0f) * half_b;
    u = std::fmin(std::fmax(u, 0.0f), bmax);
    v = std::fmin(std::fmax(v, 0.0f), bmax);
    const uint32_t dir = (spread2((uint32_t)u) << 1) | spread2((uint32_t)v);
    const uint32_t dbits = 2u * hp.b, hbits = 3u * hp.g + dbits;
    return (tag << hbits) | (cell << dbits) | dir;
}

HashP mkhp(const float* lo, const float* scale, uint32_t g, uint32_t b) {
    HashP h;
    for (int i = 0; i < 3; ++i) {
        h.lo[i] = lo[i];
        h.scale[i] = scale[i];
    }
    h.g = g;
    h.b = b;
    return h;
}

// ------------------------------------------------------------- watertight test (Woop et al. 2013)
struct RayWT {
    float o[3], s[3];
    int kx, ky, kz;
    float tmin, tmax;
};
inline RayWT wt_setup(const Ray& r) {
    RayWT w;
    const float ax = std::fabs(r.d[0]), ay = std::fabs(r.d[1]), az = std::fabs(r.d[2]);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dz = r.d[kz];
    if (dz < 0.0f) std::swap(kx, ky);
    w.kx = kx;
    w.ky = ky;
    w.kz = kz;
    w.s[0] = r.d[kx] / dz;
    w.s[1] = r.d[ky] / dz;
    w.s[2] = 1.0f / dz;
    for (int i = 0; i < 3; ++i) w.o[i] = r.o[i];
    w.tmin = r.tmin;
    w.tmax = r.tmax;
    return w;
}
inline bool wt_hit(const RayWT& r, const float* p0, const float* p1, const float* p2, float& t_out) {
    const float A[3] = {p0[0] - r.o[0], p0[1] - r.o[1], p0[2] - r.o[2]};
    const float B[3] = {p1[0] - r.o[0], p1[1] - r.o[1], p1[2] - r.o[2]};
    const float C[3] = {p2[0] - r.o[0], p2[1] - r.o[1], p2[2] - r.o[2]};
    const float Ax = A[r.kx] - r.s[0] * A[r.kz], Ay = A[r.ky] - r.s[1] * A[r.kz];
    const float Bx = B[r.kx] - r.s[0] * B[r.kz], By = B[r.ky] - r.s[1] * B[r.kz];
    const float Cx = C[r.kx] - r.s[0] * C[r.kz], Cy = C[r.ky] - r.s[1] * C[r.kz];
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = r.s[2] * A[r.kz], Bz = r.s[2] * B[r.kz], Cz = r.s[2] * C[r.kz];
    const float T = (U * Az + V * Bz) + W * Cz;
    const float t = T / det;
    t_out = t;
    return t > r.tmin && t < r.tmax;
}
inline uint64_t hit_key(float t, uint32_t tri) {
    uint32_t b;
    std::memcpy(&b, &t, 4);
    return ((uint64_t)b << 32) | tri;
}
inline float u2f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline uint32_t f2u(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// Per-ray test of a sphere (same arithmetic as the GPU): squared line distance against the squared radius
// inflated by 1e-5 of the L1 distance plus radius, and the sphere's interval along the ray.
inline bool ray_hits_sphere(const Ray& r, const float* s) {
    const float vx = s[0] - r.o[0], vy = s[1] - r.o[1], vz = s[2] - r.o[2];
    const float t = (vx * r.d[0] + vy * r.d[1]) + vz * r.d[2];
    const float wx = vy * r.d[2] - vz * r.d[1];
    const float wy = vz * r.d[0] - vx * r.d[2];
    const float wz = vx * r.d[1] - vy * r.d[0];
    const float perp2 = (wx * wx + wy * wy) + wz * wz;
    const float slack = (((std::fabs(vx) + std::fabs(vy)) + std::fabs(vz)) + s[3]) * 1e-5f;
    const float rr = s[3] + slack;
    if (perp2 > rr * rr) return false;
    if (t + rr < r.tmin) return false;
    if (t - rr > r.tmax) return false;
    return true;
}

// ------------------------------------------------------------- node test (RayTracer.cu:283-298 + reach)
inline bool node_hits_sphere(const Node& p, const float* s) {
    const float vx = s[0] - p.c[0], vy = s[1] - p.c[1], vz = s[2] - p.c[2];
    const float dd = (vx * vx + vy * vy) + vz * vz;
    const float dist = std::sqrt(dd);
    const float rr = p.radius + s[3];
    const float slack = (dist + rr) * 1e-5f;
    if (dist - s[3] > p.reach + slack) return false;
    if (p.cos_spread > 0.0f) {
        const float t = (vx * p.axis[0] + vy * p.axis[1]) + vz * p.axis[2];
        const float wx = vy * p.axis[2] - vz * p.axis[1];
        const float wy = vz * p.axis[0] - vx * p.axis[2];
        const float wz = vx * p.axis[1] - vy * p.axis[0];
        const float perp = std::sqrt((wx * wx + wy * wy) + wz * wz);
        if (perp * p.cos_spread - t * p.sin_spread > rr + slack) return false;
    }
    return true;
}

const float kRadSlack = 1.0f + 1.0f / 1048576.0f;
const float kCosMargin = 4e-6f;

// pairwise tree sum in index order with zero padding to a power of two (= the GPU xor butterfly)
float tree_sum(std::vector<float> v) {
    size_t n = 1;
    while (n < v.size()) n <<= 1;
    v.resize(n, 0.0f);
    for (size_t s = 1; s < n; s <<= 1)
        for (size_t i = 0; i + s < n; i += 2 * s) v[i] = v[i] + v[i + s];
    return v[0];
}

// Leaf of the ray hierarchy (CreateHierarchyLevel0, RayTracer.cu:1061-1108, made conservative).
Node make_leaf(const Ray* rays, const uint32_t* ids, uint32_t n, uint32_t k0, uint32_t P) {
    std::vector<Ray> r;
    std::vector<char> act;
    for (uint32_t j = 0; j < P; ++j) {
        const uint32_t k = k0 + j;
        Ray x{};
        bool a = k < n;
        if (a) {
            x = rays[ids ? ids[k] : k];
            a = x.tmax > x.tmin;
        }
        r.push_back(x);
        act.push_back(a);
    }
    float mn[3] = {INF, INF, INF}, mx[3] = {-INF, -INF, -INF};
    std::vector<float> sx(P), sy(P), sz(P);
    uint32_t cnt = 0;
    for (uint32_t j = 0; j < P; ++j) {
        if (act[j]) {
            ++cnt;
            for (int i = 0; i < 3; ++i) {
                mn[i] = std::fmin(mn[i], r[j].o[i]);
                mx[i] = std::fmax(mx[i], r[j].o[i]);
            }
        }
        sx[j] = act[j] ? r[j].d[0] : 0.0f;
        sy[j] = act[j] ? r[j].d[1] : 0.0f;
        sz[j] = act[j] ? r[j].d[2] : 0.0f;
    }
    const float Sx = tree_sum(sx), Sy = tree_sum(sy), Sz = tree_sum(sz);
    const V3 c = V3{(mn[0] + mx[0]) * 0.5f, (mn[1] + mx[1]) * 0.5f, (mn[2] + mx[2]) * 0.5f};
    const float sl = std::sqrt((Sx * Sx + Sy * Sy) + Sz * Sz);
    bool full = !(sl > 1e-20f);
    const V3 a = full ? V3{0.f, 0.f, 1.f} : V3{Sx / sl, Sy / sl, Sz / sl};
    float mr2 = 0.0f, dt = INF, rc = 0.0f;
    for (uint32_t j = 0; j < P; ++j) {
        if (!act[j]) continue;
        const V3 oc = V3{r[j].o[0] - c.x, r[j].o[1] - c.y, r[j].o[2] - c.z};
        const float r2 = dot(oc, oc);
        mr2 = std::fmax(mr2, r2);
        dt = std::fmin(dt, dot(a, V3{r[j].d[0], r[j].d[1], r[j].d[2]}));
        rc = std::fmax(rc, std::sqrt(r2) + r[j].tmax);
    }
    const float cs = dt - kCosMargin;
    if (!(cs > 0.0f)) full = true;
    Node nd{};
    nd.c[0] = c.x;
    nd.c[1] = c.y;
    nd.c[2] = c.z;
    nd.radius = std::sqrt(mr2) * kRadSlack;
    nd.axis[0] = a.x;
    nd.axis[1] = a.y;
    nd.axis[2] = a.z;
    nd.cos_spread = full ? -1.0f : cs;
    nd.sin_spread = full ? 0.0f : std::sqrt((1.0f - cs) * (1.0f + cs));
    nd.reach = rc * kRadSlack;
    nd.first = k0;
    nd.count = cnt;
    return nd;
}

// Upper level (CreateHierarchyLevelN, RayTracer.cu:1110-1150, made conservative).
Node merge_nodes(const Node* ch, uint32_t m) {
    float mn[3] = {INF, INF, INF}, mx[3] = {-INF, -INF, -INF};
    uint32_t count = 0;
    bool full = false;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (uint32_t i = 0; i < m; ++i) {
        const Node& q = ch[i];
        if (q.count == 0) continue;
        count += q.count;
        for (int k = 0; k < 3; ++k) {
            mn[k] = std::fmin(mn[k], q.c[k] - q.radius);
            mx[k] = std::fmax(mx[k], q.c[k] + q.radius);
        }
        if (!(q.cos_spread > 0.f)) full = true;
        const float w = (float)q.count;
        sx = sx + q.axis[0] * w;
        sy = sy + q.axis[1] * w;
        sz = sz + q.axis[2] * w;
    }
    Node nd{};
    nd.first = ch[0].first;
    nd.count = count;
    const V3 c = V3{(mn[0] + mx[0]) * 0.5f, (mn[1] + mx[1]) * 0.5f, (mn[2] + mx[2]) * 0.5f};
    const float sl = std::sqrt((sx * sx + sy * sy) + sz * sz);
    if (!(sl > 1e-20f)) full = true;
    const V3 a = full ? V3{0.f, 0.f, 1.f} : V3{sx / sl, sy / sl, sz / sl};
    float rad = 0.f, reach = 0.f, cs = 1.f;
    for (uint32_t i = 0; i < m; ++i) {
        const Node& q = ch[i];
        if (q.count == 0) continue;
        const V3 dc = V3{q.c[0] - c.x, q.c[1] - c.y, q.c[2] - c.z};
        const float dl = length(dc);
        rad = std::fmax(rad, dl + q.radius);
        reach = std::fmax(reach, dl + q.reach);
        if (!full) {
            float ca = dot(a, V3{q.axis[0], q.axis[1], q.axis[2]});
            ca = std::fmin(std::fmax(ca, -1.f), 1.f);
            const float sa = std::sqrt((1.f - ca) * (1.f + ca));
            cs = std::fmin(cs, ca * q.cos_spread - sa * q.sin_spread);
        }
    }
    cs = cs - kCosMargin;
    if (!(cs > 0.f)) full = true;
    nd.c[0] = c.x;
    nd.c[1] = c.y;
    nd.c[2] = c.z;
    nd.radius = rad * kRadSlack;
    nd.axis[0] = a.x;
    nd.axis[1] = a.y;
    nd.axis[2] = a.z;
    nd.cos_spread = full ? -1.f : cs;
    nd.sin_spread = full ? 0.f : std::sqrt((1.f - cs) * (1.f + cs));
    nd.reach = reach * kRadSlack;
    if (count == 0) {
        nd.c[0] = nd.c[1] = nd.c[2] = 0.f;
        nd.radius = 0.f;
        nd.reach = 0.f;
    }
    return nd;
}

struct ObjH {
    uint32_t T = 0, cluster = 8, levels = 0;
    uint32_t off[16] = {}, size[16] = {};
    uint32_t koff[16] = {};      // level l's child-range array starts at kid[koff[l]] (size[l] + 1 entries)
    std::vector<float> sph;      // 4 per node
    std::vector<uint32_t> kid;   // node j of level l: children [kid[koff[l]+j], kid[koff[l]+j+1]) of level l-1
                                 // (level 0: the cluster's triangles)
    std::vector<float> tris;     // 12 per triangle, cluster order, w of vertex 0 = original id bits
    std::vector<uint32_t> order;
    // per node (absolute index off[l] + j): padded box lo xyz, link, hi xyz, count (8 floats), link and
    // count as raw u32 bits. A cluster's link is its first triangle; a node's (level l >= 1) is its whole
    // single-ray stack entry, l << 27 | (children - 1) << 24 | absolute node index of its first child
    std::vector<float> box;
    // the single-ray box tree (wide.cu): 8 floats per slot laid out as `box`, a cluster's count with the
    // top bit set; its triangles in its own depth-first order; the root's stack entry
    std::vector<float> wbox;
    std::vector<float> wtris;
    uint32_t wroot = 0;
};

// children of node (L, idx) at level L-1 (L == levels: the virtual root over the top level)
inline void children(const ObjH& h, uint32_t L, uint32_t idx, uint32_t& first, uint32_t& cnt) {
    if (L == h.levels) {
        first = 0;
        cnt = h.size[L - 1];
        return;
    }
    const uint32_t* k = &h.kid[h.koff[L] + idx];
    first = k[0];
    cnt = k[1] - k[0];
}
// triangles of cluster c
inline void cluster_tris(const ObjH& h, uint32_t c, uint32_t& t0, uint32_t& t1) {
    t0 = h.kid[h.koff[0] + c];
    t1 = h.kid[h.koff[0] + c + 1];
}

void traverse_packet(const Node& p, const ObjH& h, uint32_t L, uint32_t idx, std::vector<uint32_t>& clusters,
                     uint64_t& tests) {
    // children of (L, idx): level L-1 nodes [8 idx, ...) or the top level for the virtual root
    const uint32_t cl = L - 1;
    uint32_t first, cnt;
    children(h, L, idx, first, cnt);
    for (uint32_t c = 0; c < cnt; ++c) {
        const float* s = &h.sph[4ull * (h.off[cl] + first + c)];
        ++tests;
        if (!node_hits_sphere(p, s)) continue;
        if (cl == 0) clusters.push_back(first + c);
        else traverse_packet(p, h, cl, first + c, clusters, tests);
    }
}

// Per-ray descent of the object subtree below (L0, idx0): nearest child first, spheres culled against
// the ray's running closest-hit distance, triangle tests with the ray's own interval (the batched form's
// per-ray phase). Returns true if occluded (any hit); updates best (closest hit).
bool ray_descend(const ObjH& h, const Ray& r, const RayWT& w, uint32_t L0, uint32_t idx0, bool any, uint64_t& best,
                 uint64_t& ntests, uint64_t& ttests) {
    float tcur = r.tmax;
    if (best != HIT_NONE) tcur = std::fmin(tcur, u2f((uint32_t)(best >> 32)));
    Ray rc = r;
    uint32_t stk[96];
    int sp = 0;
    stk[sp++] = (L0 << 24) | idx0;
    while (sp > 0) {
        const uint32_t e = stk[--sp];
        const uint32_t L = e >> 24, idx = e & 0xFFFFFFu;
        const uint32_t cl = L - 1;
        uint32_t first, cnt;
        children(h, L, idx, first, cnt);
        rc.tmax = tcur;
        if (cl == 0) {
            for (uint32_t c = 0; c < cnt; ++c) {
                ++ntests;
                rc.tmax = tcur;
                if (!ray_hits_sphere(rc, &h.sph[4ull * (h.off[0] + first + c)])) continue;
                uint32_t t0, t1;
                cluster_tris(h, first + c, t0, t1);
                for (uint32_t t = t0; t < t1; ++t) {
                    const float* v = &h.tris[12ull * t];
                    float th;
                    ++ttests;
                    if (wt_hit(w, v, v + 4, v + 8, th)) {
                        if (any) return true;
                        const uint64_t key = hit_key(th, f2u(v[3]));
                        if (key < best) {
                            best = key;
                            tcur = std::fmin(tcur, th);
                        }
                    }
                }
            }
        } else {
            float te[8];
            uint32_t ci[8];
            uint32_t nh = 0;
            for (uint32_t c = 0; c < cnt; ++c) {
                const float* q = &h.sph[4ull * (h.off[cl] + first + c)];
                ++ntests;
                if (!ray_hits_sphere(rc, q)) continue;
                const float tc = ((q[0] - r.o[0]) * r.d[0] + (q[1] - r.o[1]) * r.d[1]) + (q[2] - r.o[2]) * r.d[2] - q[3];
                uint32_t k = nh++;
                while (k > 0 && te[k - 1] < tc) {
                    te[k] = te[k - 1];
                    ci[k] = ci[k - 1];
                    --k;
                }
                te[k] = tc;
                ci[k] = first + c;
            }
            for (uint32_t k = 0; k < nh && sp < 96; ++k) stk[sp++] = (cl << 24) | ci[k];
        }
    }
    return false;
}

// Ray vs a padded node box over [tmin, tmax] (fused.cu box_hit_fma): per plane t = fma(b, inv, -(o * inv))
// with inv the IEEE reciprocal of the direction component, components below 1e-20 in magnitude replaced by
// +-1e-20; entry distance tn = max(tmin, per-axis minima), exit = min(tmax, per-axis maxima). tn is the
// nearest-first order key.
inline float safe_rcp(float d) {
    const float m = 1e-20f;
    return 1.0f / (std::fabs(d) < m ? std::copysign(m, d) : d);
}
inline bool box_hit(const float* b, const float inv[3], const float oi[3], float tmin, float tmax, float& tn) {
    const float ax = std::fma(b[0], inv[0], -oi[0]), bx = std::fma(b[4], inv[0], -oi[0]);
    const float ay = std::fma(b[1], inv[1], -oi[1]), by = std::fma(b[5], inv[1], -oi[1]);
    const float az = std::fma(b[2], inv[2], -oi[2]), bz = std::fma(b[6], inv[2], -oi[2]);
    tn = std::fmax(std::fmax(std::fmax(tmin, std::fmin(ax, bx)), std::fmin(ay, by)), std::fmin(az, bz));
    const float tf = std::fmin(std::fmin(std::fmin(tmax, std::fmax(ax, bx)), std::fmax(ay, by)), std::fmax(az, bz));
    return tn <= tf;
}

// One ray from the root of the single-ray box tree (wide.cu): the batched form's rays-only traversal
// (fused.cu k_fused_rays). A stack entry is a node's entry word (its box's lo.w: 1 << 27 | (children - 1)
// << 24 | first child slot) or a cluster's slot, with the distance at which the ray enters its box (from
// the parent's test; the root's is -inf). A closest-hit ray drops an entry whose entry distance lies beyond
// its current best unread: no box inside it (children lie inside their parent's box) can be entered
// earlier, and for a cluster this is exactly the outcome of testing its box again against the current
// best. An any-hit ray's interval never shrinks, so it never drops one. A node step tests every child's box
// against [tmin, current best] and pushes the hits: any hit in child order (the last child pops first),
// closest hit farthest first (the nearest pops first; among equal entry distances the lower child). A
// cluster step tests its triangles. Counts node tests (every child of a node that is stepped) and triangle
// tests. Returns false on a stack overflow (more than 96 entries).
bool ray_descend_box(const ObjH& h, const Ray& r, bool any, bool& occluded, uint64_t& best, uint64_t& ntests,
                     uint64_t& ttests) {
    occluded = false;
    best = HIT_NONE;
    if (!(r.tmax > r.tmin) || h.levels == 0) return true;
    const RayWT w = wt_setup(r);
    const float inv[3] = {safe_rcp(r.d[0]), safe_rcp(r.d[1]), safe_rcp(r.d[2])};
    const float oi[3] = {r.o[0] * inv[0], r.o[1] * inv[1], r.o[2] * inv[2]};
    float tcur = r.tmax;
    uint32_t stk[96];
    float stt[96];
    int sp = 0;
    stk[sp] = h.wroot;
    stt[sp++] = -INF;
    while (sp > 0) {
        --sp;
        const uint32_t e = stk[sp];
        if (stt[sp] > tcur) continue;
        const uint32_t L = e >> 27, idx = e & 0xFFFFFFu;
        if (L == 0) {
            const float* b = &h.wbox[8ull * idx];
            const uint32_t t0 = f2u(b[3]), t1 = t0 + (f2u(b[7]) & 0x7FFFFFFFu);
            for (uint32_t t = t0; t < t1; ++t) {
                const float* v = &h.wtris[12ull * t];
                float th;
                ++ttests;
                if (wt_hit(w, v, v + 4, v + 8, th)) {
                    if (any) {
                        occluded = true;
                        return true;
                    }
                    const uint64_t key = hit_key(th, f2u(v[3]));
                    if (key < best) {
                        best = key;
                        tcur = std::fmin(tcur, th);
                    }
                }
            }
            continue;
        }
        const uint32_t cnt = ((e >> 24) & 7u) + 1u;
        ntests += cnt;
        if (sp + (int)cnt > 96) return false;
        float tcs[8];
        uint32_t hm = 0;
        for (uint32_t c = 0; c < cnt; ++c) {
            float tc;
            tcs[c] = 0.0f;
            if (box_hit(&h.wbox[8ull * (idx + c)], inv, oi, r.tmin, tcur, tc)) {
                hm |= 1u << c;
                tcs[c] = tc;
            }
        }
        while (hm) {
            uint32_t bc = 0;
            if (!any) {
                float bt = -INF;
                for (uint32_t c = 0; c < 8; ++c)
                    if (((hm >> c) & 1u) && tcs[c] >= bt) {
                        bt = tcs[c];
                        bc = c;
                    }
            } else {
                bc = (uint32_t)__builtin_ctz(hm);
            }
            hm &= ~(1u << bc);
            const float* cb = &h.wbox[8ull * (idx + bc)];
            stk[sp] = (f2u(cb[7]) & 0x80000000u) ? idx + bc : f2u(cb[3]);
            stt[sp++] = tcs[bc];
        }
    }
    return true;
}

}  // namespace

extern "C" {

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

// ---------------------------------------------------------------- hashing / raygen
void orc_hash_params(const float lo[3], const float hi[3], uint32_t g, float scale_out[3]) {
    const float G = (float)(1u << g);
    for (int i = 0; i < 3; ++i) {
        const float ext = hi[i] - lo[i];
        scale_out[i] = ext > 0.0f ? G / ext : 0.0f;
    }
}

void orc_hash(const float* rays, uint32_t n, const float lo[3], const float scale[3], uint32_t g, uint32_t b,
              uint32_t tag, uint32_t* keys) {
    const HashP hp = mkhp(lo, scale, g, b);
    const Ray* r = reinterpret_cast<const Ray*>(rays);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i)
        keys[i] = (r[i].tmax > r[i].tmin) ? ray_hash(r[i].o, r[i].d, hp, tag) : KEY_NONE;
}

// Camera basis of Camera::loadView (E/Camera.cpp:108-133): direction = unit(target - eye) * dist,
// right = unit(direction x up) * halfW, up = unit(right x direction) * halfH with halfH = 2 dist tan(fov/2)
// and halfW = halfH * W / H. Evaluated in double and rounded once to float (cam: eye, dir, right, up).
// Returns 0 for a degenerate camera (eye == target, zero size).
int orc_camera_look_at(const float eye[3], const float target[3], const float up[3], float fov_degrees,
                       uint32_t W, uint32_t H, float* cam) {
    if (W == 0 || H == 0) return 0;
    double dir[3] = {target[0] - (double)eye[0], target[1] - (double)eye[1], target[2] - (double)eye[2]};
    const double dist = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (!(dist > 0)) return 0;
    const double half_h = 2.0 * dist * std::tan(0.5 * fov_degrees * 3.14159265358979323846 / 180.0);
    const double half_w = half_h * (double)W / (double)H;
    auto unit = [](double* v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (l > 0) for (int i = 0; i < 3; ++i) v[i] /= l;
    };
    double f[3] = {dir[0] / dist, dir[1] / dist, dir[2] / dist};
    double r[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    unit(r);
    double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    unit(u);
    for (int i = 0; i < 3; ++i) {
        cam[i] = eye[i];
        cam[3 + i] = (float)(f[i] * dist);
        cam[6 + i] = (float)(r[i] * half_w);
        cam[9 + i] = (float)(u[i] * half_h);
    }
    return 1;
}

// Camera ray (CUDA-Naive-Ray-Tracer RayTracer.cu:606-607; RayTracer.cu:666-667) in 8x8 tile order.
void orc_raygen_primary(const float* cam /*eye,dir,right,up*/, uint32_t W, uint32_t H, float* rays_out,
                        uint32_t* pix_out) {
    const uint32_t tx = (W + 7) / 8, ty = (H + 7) / 8, n = tx * ty * 64;
    Ray* rays = reinterpret_cast<Ray*>(rays_out);
#pragma omp parallel for schedule(static)
    for (int64_t kk = 0; kk < (int64_t)n; ++kk) {
        const uint32_t k = (uint32_t)kk;
        const uint32_t tile = k >> 6, within = k & 63u;
        // tile rows from the image's middle outwards (raygen.cu tile_row)
        const uint32_t tr = tile / tx, m = ty >> 1, row = (tr & 1u) ? m - ((tr + 1u) >> 1) : m + (tr >> 1);
        const uint32_t x = (tile % tx) * 8 + (within & 7u), y = row * 8 + (within >> 3);
        Ray r{};
        r.o[0] = cam[0];
        r.o[1] = cam[1];
        r.o[2] = cam[2];
        r.tmin = 0.0f;
        if (x < W && y < H) {
            const float a = (float)x / (float)W - 0.5f, b = (float)y / (float)H - 0.5f;
            const V3 q = V3{(cam[3] + cam[6] * a) + cam[9] * b, (cam[4] + cam[7] * a) + cam[10] * b,
                            (cam[5] + cam[8] * a) + cam[11] * b};
            const V3 d = normalize(q);
            r.d[0] = d.x;
            r.d[1] = d.y;
            r.d[2] = d.z;
            r.tmax = INF;
            if (pix_out) pix_out[k] = y * W + x;
        } else {
            r.d[0] = 0.f;
            r.d[1] = 0.f;
            r.d[2] = 1.f;
            r.tmax = -1.0f;
            if (pix_out) pix_out[k] = 0xFFFFFFFFu;
        }
        rays[k] = r;
    }
}

// CreateShadowRays (RayTracer.cu:682-740): origin at the light, direction to the surface point, kept iff
// N.(-d) > 0; the test interval is (eps, |light - p| - 2 eps) from the eps-offset origin (:1607-1611).
// Soft-shadow sample k (0..15) of a shadow ray with direction d from light position lp: the reference's
// 4x4 grid around the light without its centre row/column (RayTracer.cu:1550-1599): k = i + 4 j,
// a = i (+1 from i = 2), b = j (+1 from j = 2), position lp + axis0 (a - 2) / 8 + axis1 (b - 2) / 8 with
// axis0 = cross(e, d) for the axis e picked by min(|dx|, max(|dy|, |dz|)), axis1 = cross(d, axis0).
static V3 soft_sample_pos(V3 lp, V3 d, uint32_t k) {
    const uint32_t i = k & 3u, j = k >> 2;
    const float ca = (float)((int)(i + (i >= 2u ? 1u : 0u)) - 2), cb = (float)((int)(j + (j >= 2u ? 1u : 0u)) - 2);
    const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    const float mn = std::fmin(ax, std::fmax(ay, az));
    const V3 e = (ax == mn) ? V3{1.f, 0.f, 0.f} : (ay == mn) ? V3{0.f, 1.f, 0.f} : V3{0.f, 0.f, 1.f};
    const V3 a0 = cross(e, d);
    const V3 a1 = cross(d, a0);
    return V3{(lp.x + (a0.x * ca) * 0.125f) + (a1.x * cb) * 0.125f, (lp.y + (a0.y * ca) * 0.125f) + (a1.y * cb) * 0.125f,
              (lp.z + (a0.z * ca) * 0.125f) + (a1.z * cb) * 0.125f};
}

// CreateShadowRays (RayTracer.cu:682-740): S = 1, or S = 16 soft-shadow samples per light. Slot of
// (pixel x, y, light l, sample s) = x + W (v + L S y), v = l S + s; the hash tag is v.
void orc_raygen_shadow_samples(const float* spos, const float* snrm, uint32_t W, uint32_t H, const float* light_pos,
                               uint32_t L, uint32_t S, float eps, const float lo[3], const float scale[3], uint32_t g,
                               uint32_t b, float* rays_out, uint32_t* keys) {
    const HashP hp = mkhp(lo, scale, g, b);
    Ray* rays = reinterpret_cast<Ray*>(rays_out);
    const uint32_t V = L * S;
    const uint64_t n = (uint64_t)W * H * V;
#pragma omp parallel for schedule(static)
    for (int64_t si = 0; si < (int64_t)n; ++si) {
        const uint32_t slot = (uint32_t)si;
        const uint32_t x = slot % W, v = (slot / W) % V, y = slot / (W * V);
        const uint32_t l = v / S, s = v % S;
        const uint32_t pix = y * W + x;
        uint32_t key = KEY_NONE;
        if (spos[4ull * pix + 3] != 0.0f) {
            const V3 p = V3{spos[4ull * pix], spos[4ull * pix + 1], spos[4ull * pix + 2]};
            const V3 nn = normalize(V3{snrm[4ull * pix], snrm[4ull * pix + 1], snrm[4ull * pix + 2]});
            const V3 lp = V3{light_pos[3 * l], light_pos[3 * l + 1], light_pos[3 * l + 2]};
            const V3 vv = sub(p, lp);
            const float len = length(vv);
            const V3 d = V3{vv.x / len, vv.y / len, vv.z / len};
            const float diffuse = dot(d, V3{-nn.x, -nn.y, -nn.z});
            const float tmax = len - 2.0f * eps;
            if (diffuse > 0.0f && tmax > eps) {
                V3 src = lp, dir = d;
                float tm = tmax;
                bool ok = true;
                if (S > 1) {
                    src = soft_sample_pos(lp, d, s);
                    const V3 vs = sub(p, src);
                    const float ls = length(vs);
                    dir = V3{vs.x / ls, vs.y / ls, vs.z / ls};
                    tm = ls - 2.0f * eps;
                    ok = tm > eps;
                }
                if (ok) {
                    const V3 o = add(src, mul(dir, eps));
                    Ray r;
                    r.o[0] = o.x;
                    r.o[1] = o.y;
                    r.o[2] = o.z;
                    r.tmin = eps;
                    r.d[0] = dir.x;
                    r.d[1] = dir.y;
                    r.d[2] = dir.z;
                    r.tmax = tm;
                    rays[slot] = r;
                    key = ray_hash(r.o, r.d, hp, v);
                }
            }
        }
        if (key == KEY_NONE) rays[slot] = Ray{{0.f, 0.f, 0.f}, 0.f, {0.f, 0.f, 0.f}, -1.f};
        keys[slot] = key;
    }
}
void orc_raygen_shadow(const float* spos, const float* snrm, uint32_t W, uint32_t H, const float* light_pos,
                       uint32_t L, float eps, const float lo[3], const float scale[3], uint32_t g, uint32_t b,
                       float* rays_out, uint32_t* keys) {
    orc_raygen_shadow_samples(spos, snrm, W, H, light_pos, L, 1, eps, lo, scale, g, b, rays_out, keys);
}

// Soft-shadow weight of sample k (RayTracer.cu:1680-1690): inner four 0.55/16, corners 0.5375/16, edges
// 0.525/16, summed over the unoccluded samples; the light's term is scaled by log2(1 + 2 sum).
static float soft_weight(uint32_t k) {
    if (k == 5 || k == 6 || k == 9 || k == 10) return 0.55f / 16.0f;
    if (k == 0 || k == 3 || k == 12 || k == 15) return 0.5375f / 16.0f;
    return 0.525f / 16.0f;
}

// Blinn-Phong shading of one surface buffer into the accumulators (ColorPrimaryShadowRay
// RayTracer.cu:1616-1709, ColorReflectionRay :1776-1882): lights = L x {position[3], color[3], diffuse,
// specular}, materials = M x {diffuse[4] (w = reflectance), specular[4] (w = shininess)}, shadow flags per
// (pixel, light, sample) slot or NULL (unshadowed), accum = W*H x {rgb, carried reflectance}.
// incident == NULL: the incident direction is p - eye.
void orc_shade(const float* spos, const float* snrm, const float* materials, uint32_t nmat, const uint32_t* shadow,
               float* accum, uint32_t W, uint32_t H, const float* lights, uint32_t L, uint32_t S, const float eye[3],
               uint32_t bounce, const float* incident) {
    const uint64_t npix = (uint64_t)W * H;
#pragma omp parallel for schedule(static)
    for (int64_t pi = 0; pi < (int64_t)npix; ++pi) {
        const uint32_t pix = (uint32_t)pi;
        float acc[4] = {0.f, 0.f, 0.f, 1.f};
        if (bounce != 0)
            for (int i = 0; i < 4; ++i) acc[i] = accum[4ull * pix + i];
        const float* p4 = spos + 4ull * pix;
        if (p4[3] != 0.0f && acc[3] > 0.0f) {
            const V3 p = V3{p4[0], p4[1], p4[2]};
            const float* n4 = snrm + 4ull * pix;
            const V3 n = normalize(V3{n4[0], n4[1], n4[2]});
            uint32_t mid = f2u(n4[3]);
            if (mid >= nmat) mid = 0;
            const float* md = materials + 8ull * mid;
            const float* ms = md + 4;
            V3 inc;
            if (incident) {
                const float* r = incident + 8ull * pix;
                inc = V3{r[4], r[5], r[6]};
            } else {
                inc = normalize(sub(p, V3{eye[0], eye[1], eye[2]}));
            }
            const uint32_t x = pix % W, y = pix / W;
            float cr = 0.f, cg = 0.f, cb = 0.f;
            for (uint32_t l = 0; l < L; ++l) {
                float factor = 1.0f;
                if (S == 1) {
                    if (shadow && shadow[x + W * (l + L * y)] == OCCLUDED) continue;
                } else if (shadow) {
                    float sf = 0.0f;
                    for (uint32_t k = 0; k < S; ++k)
                        if (shadow[x + W * ((l * S + k) + L * S * y)] != OCCLUDED) sf += soft_weight(k);
                    factor = std::log2(1.0f + sf * 2.0f);
                }
                const float* Lt = lights + 8ull * l;
                V3 ld = sub(V3{Lt[0], Lt[1], Lt[2]}, p);
                const float dist = length(ld);
                ld = V3{ld.x / dist, ld.y / dist, ld.z / dist};
                const float att = 1.0f / (0.75f + dist * 0.0005f + dist * dist * 0.00005f);
                const float diff = std::fmin(std::fmax(dot(ld, n), 0.0f), 1.0f);
                if (diff > 0.0f) {
                    const V3 hv = normalize(sub(ld, inc));
                    const float sp = std::fmin(std::fmax(std::pow(std::fmax(dot(hv, n), 0.0f), ms[3]), 0.0f), 1.0f);
                    const float kd = diff * Lt[6] * att * factor, ks = sp * Lt[7] * att * factor;
                    cr += (md[0] * kd + ms[0] * ks) * Lt[3];
                    cg += (md[1] * kd + ms[1] * ks) * Lt[4];
                    cb += (md[2] * kd + ms[2] * ks) * Lt[5];
                }
            }
            acc[0] += acc[3] * cr;
            acc[1] += acc[3] * cg;
            acc[2] += acc[3] * cb;
            acc[3] *= md[3];
        } else {
            acc[3] = 0.0f;
        }
        for (int i = 0; i < 4; ++i) accum[4ull * pix + i] = acc[i];
    }
}

// RgbToInt (RayTracer.cu:1702): clamp(c * 255) per channel, alpha 255.
void orc_pack(const float* accum, uint32_t n, uint32_t* rgba) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* c = accum + 4ull * i;
        const uint32_t r = (uint32_t)std::fmin(std::fmax(c[0] * 255.0f, 0.0f), 255.0f);
        const uint32_t g = (uint32_t)std::fmin(std::fmax(c[1] * 255.0f, 0.0f), 255.0f);
        const uint32_t b = (uint32_t)std::fmin(std::fmax(c[2] * 255.0f, 0.0f), 255.0f);
        rgba[i] = r | (g << 8) | (b << 16) | (255u << 24);
    }
}

static uint32_t rng_next(uint32_t& state) {
    state = state * 747796405u + 2891336453u;
    const uint32_t w = ((state >> ((state >> 28) + 4u)) ^ state) * 277803737u;
    return (w >> 22) ^ w;
}
// Marsaglia (1972): uniform point on the unit sphere by rejection (sqrt only).
static V3 sphere_sample(uint32_t seed, uint32_t slot, uint32_t bounce) {
    uint32_t st = seed ^ (slot * 0x9E3779B9u) ^ (bounce * 0x85EBCA6Bu);
    rng_next(st);
    for (int it = 0; it < 32; ++it) {
        const float x1 = (float)(rng_next(st) >> 9) * (1.0f / 4194304.0f) - 1.0f;
        const float x2 = (float)(rng_next(st) >> 9) * (1.0f / 4194304.0f) - 1.0f;
        const float q = x1 * x1 + x2 * x2;
        if (q < 1.0f && q > 0.0f) {
            const float t = 2.0f * std::sqrt(1.0f - q);
            return V3{x1 * t, x2 * t, 1.0f - 2.0f * q};
        }
    }
    return V3{0.f, 0.f, 1.f};
}

// CreateReflectionRays (RayTracer.cu:742-791) / ColorAndCreateReflectionRay (:1995-2016):
// d = reflect(incident, n), origin offset by eps (:1765), optional cosine-lobe perturbation.
// CreateRefractionRays (RayTracer.cu:793-842): refract(i, n, eta) by GLSL's formula, no ray on total
// internal reflection, renormalised, origin offset by eps, interval (eps, inf); hash as every other ray.
void orc_raygen_refract(const float* spos, const float* snrm, const float* prev_rays, const float eye[3], uint32_t W,
                        uint32_t H, float eps, float eta, const float lo[3], const float scale[3], uint32_t g,
                        uint32_t b, float* rays_out, uint32_t* keys) {
    const HashP hp = mkhp(lo, scale, g, b);
    Ray* rays = reinterpret_cast<Ray*>(rays_out);
    const Ray* prev = reinterpret_cast<const Ray*>(prev_rays);
    const uint64_t n = (uint64_t)W * H;
#pragma omp parallel for schedule(static)
    for (int64_t si = 0; si < (int64_t)n; ++si) {
        const uint32_t slot = (uint32_t)si;
        uint32_t key = KEY_NONE;
        if (spos[4ull * slot + 3] != 0.0f) {
            const V3 p = V3{spos[4ull * slot], spos[4ull * slot + 1], spos[4ull * slot + 2]};
            const V3 nn = normalize(V3{snrm[4ull * slot], snrm[4ull * slot + 1], snrm[4ull * slot + 2]});
            const V3 i = prev ? V3{prev[slot].d[0], prev[slot].d[1], prev[slot].d[2]}
                              : normalize(sub(p, V3{eye[0], eye[1], eye[2]}));
            const float d = dot(nn, i);
            const float k = 1.0f - eta * eta * (1.0f - d * d);
            if (k >= 0.0f) {
                const V3 tr = normalize(sub(mul(i, eta), mul(nn, eta * d + std::sqrt(k))));
                if (tr.x == tr.x && tr.y == tr.y && tr.z == tr.z) {
                    const V3 o = add(p, mul(tr, eps));
                    Ray r;
                    r.o[0] = o.x;
                    r.o[1] = o.y;
                    r.o[2] = o.z;
                    r.tmin = eps;
                    r.d[0] = tr.x;
                    r.d[1] = tr.y;
                    r.d[2] = tr.z;
                    r.tmax = std::numeric_limits<float>::infinity();
                    rays[slot] = r;
                    key = ray_hash(r.o, r.d, hp, 0u);
                }
            }
        }
        if (key == KEY_NONE) rays[slot] = Ray{{0.f, 0.f, 0.f}, 0.f, {0.f, 0.f, 0.f}, -1.f};
        keys[slot] = key;
    }
}

void orc_raygen_reflect(const float* spos, const float* snrm, const float* prev_rays, const float eye[3],
                        uint32_t W, uint32_t H, float eps, float jitter, uint32_t seed, uint32_t bounce,
                        const float lo[3], const float scale[3], uint32_t g, uint32_t b, float* rays_out,
                        uint32_t* keys) {
    const HashP hp = mkhp(lo, scale, g, b);
    Ray* rays = reinterpret_cast<Ray*>(rays_out);
    const Ray* prev = reinterpret_cast<const Ray*>(prev_rays);
    const uint64_t n = (uint64_t)W * H;
#pragma omp parallel for schedule(static)
    for (int64_t si = 0; si < (int64_t)n; ++si) {
        const uint32_t slot = (uint32_t)si;
        uint32_t key = KEY_NONE;
        if (spos[4ull * slot + 3] != 0.0f) {
            const V3 p = V3{spos[4ull * slot], spos[4ull * slot + 1], spos[4ull * slot + 2]};
            const V3 nn = normalize(V3{snrm[4ull * slot], snrm[4ull * slot + 1], snrm[4ull * slot + 2]});
            V3 i;
            if (prev) i = V3{prev[slot].d[0], prev[slot].d[1], prev[slot].d[2]};
            else i = normalize(sub(p, V3{eye[0], eye[1], eye[2]}));
            const float k2 = 2.0f * dot(nn, i);
            V3 r = sub(i, mul(nn, k2));
            if (jitter > 0.0f) {
                const V3 u = sphere_sample(seed, slot, bounce);
                r = add(r, mul(u, jitter));
                const float rn = dot(r, nn);
                if (rn < 0.0f) r = sub(r, mul(nn, 2.0f * rn));
            }
            r = normalize(r);
            if (r.x == r.x && r.y == r.y && r.z == r.z) {
                const V3 o = add(p, mul(r, eps));
                Ray ry;
                ry.o[0] = o.x;
                ry.o[1] = o.y;
                ry.o[2] = o.z;
                ry.tmin = eps;
                ry.d[0] = r.x;
                ry.d[1] = r.y;
                ry.d[2] = r.z;
                ry.tmax = INF;
                rays[slot] = ry;
                key = ray_hash(ry.o, ry.d, hp, 0u);
            }
        }
        if (key == KEY_NONE) rays[slot] = Ray{{0.f, 0.f, 0.f}, 0.f, {0.f, 0.f, 0.f}, -1.f};
        keys[slot] = key;
    }
}

// ---------------------------------------------------------------- trim / compress / sort / decompress
// CreateTrimmedRays (RayTracer.cu:844-884) + CreateChunkFlags/Bases/Sizes (:886-991).
void orc_compress(const uint32_t* keys, uint32_t n, uint32_t* trimmed, uint32_t* ckeys, uint32_t* cbases,
                  uint32_t* csizes, uint32_t* counts) {
    uint32_t R = 0, C = 0;
    uint32_t last = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t k = keys[i];
        if (k == KEY_NONE) continue;
        if (R == 0 || k != last) {
            ckeys[C] = k;
            cbases[C] = R;
            ++C;
        }
        trimmed[R++] = i;
        last = k;
    }
    cbases[C] = R;
    if (csizes)
        for (uint32_t c = 0; c < C; ++c) csizes[c] = cbases[c + 1] - cbases[c];
    counts[0] = R;
    counts[1] = C;
}

// Stable sort by the low key_bits (cub::DeviceRadixSort::SortPairs semantics, RayTracer.cu:2400-2404).
void orc_sort_pairs(const uint32_t* keys, const uint32_t* vals, uint32_t n, uint32_t key_bits, uint32_t* ko,
                    uint32_t* vo) {
    const uint32_t mask = key_bits >= 32 ? 0xFFFFFFFFu : ((1u << key_bits) - 1u);
    const uint32_t passes = key_bits == 0 ? 1 : (key_bits + 7) / 8;
    const uint32_t smask = passes >= 4 ? 0xFFFFFFFFu : ((1u << (8 * passes)) - 1u);
    (void)mask;
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](uint32_t a, uint32_t b) { return (keys[a] & smask) < (keys[b] & smask); });
    for (uint32_t i = 0; i < n; ++i) {
        ko[i] = keys[idx[i]];
        vo[i] = vals ? vals[idx[i]] : idx[i];
    }
}

// CreateSortedRaySkeleton + ExclusiveSum + CreateSortedRays (RayTracer.cu:993-1059, :2445-2462).
void orc_decompress(const uint32_t* skeys, const uint32_t* svals, const uint32_t* cbases, const uint32_t* trimmed,
                    uint32_t R, uint32_t C, uint32_t* sorted_keys, uint32_t* sorted_ids) {
    (void)R;
    uint32_t k = 0;
    for (uint32_t x = 0; x < C; ++x) {
        const uint32_t c = svals[x];
        const uint32_t base = cbases[c], size = cbases[c + 1] - cbases[c];
        for (uint32_t j = 0; j < size; ++j) {
            sorted_ids[k] = trimmed[base + j];
            if (sorted_keys) sorted_keys[k] = skeys ? skeys[x] : 0u;
            ++k;
        }
    }
}

// ---------------------------------------------------------------- ray hierarchy
uint32_t orc_hierarchy_offsets(uint32_t max_rays, uint32_t P, uint32_t off[4]) {
    const uint32_t n0 = (max_rays + P - 1) / P, n1 = (n0 + 7) / 8, n2 = (n1 + 7) / 8;
    off[0] = 0;
    off[1] = n0;
    off[2] = n0 + n1;
    off[3] = n0 + n1 + n2;
    return off[3];
}

// HierarchyCreationWrapper (RayTracer.cu:2469-2535). Nodes written at the offsets of max_rays.
void orc_build_rsh(const float* rays_in, const uint32_t* ids, uint32_t n, uint32_t max_rays, uint32_t P,
                   void* nodes_out) {
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
    Node* nodes = static_cast<Node*>(nodes_out);
    uint32_t off[4];
    orc_hierarchy_offsets(max_rays, P, off);
    const uint32_t n0 = (n + P - 1) / P, n1 = (n0 + 7) / 8, n2 = (n1 + 7) / 8;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < (int64_t)n0; ++j) nodes[off[0] + j] = make_leaf(rays, ids, n, (uint32_t)j * P, P);
    const uint32_t sizes[3] = {n0, n1, n2};
    for (int lvl = 1; lvl <= 2; ++lvl) {
        const uint32_t nc = sizes[lvl - 1], np = sizes[lvl];
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < (int64_t)np; ++j) {
            const uint32_t c0 = 8 * (uint32_t)j, c1 = std::min(c0 + 8, nc);
            nodes[off[lvl] + j] = merge_nodes(&nodes[off[lvl - 1] + c0], c1 - c0);
        }
    }
}

// ---------------------------------------------------------------- object hierarchy
// Restates the GPU build (objh.cu): Morton order of the triangle centroids; boundary strength before
// sorted triangle k = highest differing bit of the 64-bit keys (code << 32 | k); level 0 groups triangles
// into clusters of at most `cluster`, higher levels group the level below into nodes of at most 8, cutting
// boundary j iff the range it splits (between the nearest stronger boundaries) holds more than G items
// (fixed groups of G when a level would shrink less than 2x for clusters or 4x above); spheres from every
// vertex of a node's triangle range; up to the first level of at most 8 nodes.
static ObjH* g_last_objh = nullptr;

static void build_box_tree(ObjH& h, float pad);
static void build_objh(const float* pos, uint32_t T, uint32_t cluster, const float lo[3], const float hi[3],
                       ObjH& h) {
    h.T = T;
    h.cluster = cluster;
    std::vector<uint32_t> codes(T);
    float ext = hi[0] - lo[0];
    if (hi[1] - lo[1] > ext) ext = hi[1] - lo[1];
    if (hi[2] - lo[2] > ext) ext = hi[2] - lo[2];
    const float sc1 = (ext > 0.0f) ? 1024.0f / ext : 0.0f;
    const float sc[3] = {sc1, sc1, sc1};
    for (uint32_t t = 0; t < T; ++t) {
        const float* a = pos + 12ull * t;
        uint32_t cc[3];
        for (int i = 0; i < 3; ++i) {
            const float c = ((a[i] + a[4 + i]) + a[8 + i]) / 3.0f;
            float f = std::fmin(std::fmax((c - lo[i]) * sc[i], 0.f), 1023.f);
            cc[i] = (uint32_t)f;
        }
        codes[t] = (spread3(cc[0]) << 2) | (spread3(cc[1]) << 1) | spread3(cc[2]);
    }
    h.order.resize(T);
    std::iota(h.order.begin(), h.order.end(), 0u);
    std::stable_sort(h.order.begin(), h.order.end(), [&](uint32_t a, uint32_t b) { return codes[a] < codes[b]; });
    h.tris.resize(12ull * T);
    std::vector<uint32_t> scode(T);
    for (uint32_t k = 0; k < T; ++k) {
        const uint32_t t = h.order[k];
        std::memcpy(&h.tris[12ull * k], pos + 12ull * t, 48);
        h.tris[12ull * k + 3] = u2f(t);
        scode[k] = codes[t];
    }
    h.levels = 0;
    h.sph.clear();
    h.kid.clear();
    if (T == 0) return;
    // boundary strength before sorted triangle k: highest differing bit of the 64-bit keys
    // (code << 32 | k) of triangles k-1 and k; 64 at both ends
    auto dtri = [&](uint32_t k) -> uint32_t {
        if (k == 0 || k >= T) return 64u;
        const uint32_t a = scode[k - 1], b = scode[k];
        if (a != b) return 32u + (31u - (uint32_t)__builtin_clz(a ^ b));
        return 31u - (uint32_t)__builtin_clz((k - 1) ^ k);
    };
    // items of the level being grouped: start[j] = first triangle of item j (start[n] = T)
    std::vector<uint32_t> start(T + 1);
    std::iota(start.begin(), start.end(), 0u);
    uint32_t n = T;
    uint32_t total_nodes = 0, total_kids = 0;
    std::vector<std::vector<uint32_t>> lvl_first;  // per level: child-range starts (+ sentinel)
    std::vector<std::vector<uint32_t>> lvl_tri;    // per level: triangle-range starts (+ sentinel)
    while (true) {
        const uint32_t l = h.levels;
        const uint32_t G = (l == 0) ? cluster : 8u;
        auto delta = [&](uint32_t j) -> uint32_t { return (j == 0 || j >= n) ? 64u : dtri(start[j]); };
        std::vector<uint32_t> firsts;
        for (uint32_t j = 0; j < n; ++j) {
            bool cut = (j == 0);
            if (!cut) {
                const uint32_t d = delta(j);
                int64_t lo = -1, hi = -1;
                for (int64_t q = (int64_t)j - 1; q >= 0 && q >= (int64_t)j - (int64_t)G; --q)
                    if (delta((uint32_t)q) > d) {
                        lo = q;
                        break;
                    }
                for (uint64_t q = (uint64_t)j + 1; q <= n && q <= (uint64_t)j + G; ++q)
                    if (delta((uint32_t)q) > d) {
                        hi = (int64_t)q;
                        break;
                    }
                cut = lo < 0 || hi < 0 || (hi - lo) > (int64_t)G;
            }
            if (cut) firsts.push_back(j);
        }
        uint64_t nn = firsts.size();
        // fixed groups of G when the Morton groups reduce too little (>= 2x for clusters, >= 4x above)
        if ((l == 0 && nn * 2 > (uint64_t)n + 1) || (l > 0 && nn * 4 > (uint64_t)n + 3)) {
            firsts.clear();
            for (uint32_t j = 0; j < n; j += G) firsts.push_back(j);
            nn = firsts.size();
        }
        firsts.push_back(n);
        std::vector<uint32_t> tstart(nn + 1);
        for (uint64_t g = 0; g <= nn; ++g) tstart[g] = start[firsts[g]];
        h.off[l] = total_nodes;
        h.size[l] = (uint32_t)nn;
        h.koff[l] = total_kids;
        total_nodes += (uint32_t)nn;
        total_kids += (uint32_t)nn + 1;
        lvl_first.push_back(firsts);
        lvl_tri.push_back(tstart);
        h.levels = l + 1;
        start.assign(tstart.begin(), tstart.end());
        n = (uint32_t)nn;
        if (n <= 8 || h.levels >= 16) break;
    }
    h.sph.assign(4ull * total_nodes, 0.0f);
    h.box.assign(8ull * total_nodes, 0.0f);
    // boxes are widened by 1e-5 of the scene's largest coordinate magnitude (objh.cu)
    float smax = 0.0f;
    for (int a = 0; a < 3; ++a) smax = std::fmax(smax, std::fmax(std::fabs(lo[a]), std::fabs(hi[a])));
    const float pad = 1e-5f * smax + 1e-30f;
    h.kid.assign(total_kids, 0u);
    for (uint32_t l = 0; l < h.levels; ++l) {
        // level 0 stores the clusters' triangle ranges, higher levels their child ranges
        const std::vector<uint32_t>& k = (l == 0) ? lvl_tri[0] : lvl_first[l];
        std::memcpy(&h.kid[h.koff[l]], k.data(), 4ull * (h.size[l] + 1));
        // spheres: midpoint of the vertex box, radius = max vertex distance (x (1 + 2^-20)), over every
        // vertex of the node's triangle range
        for (uint32_t j = 0; j < h.size[l]; ++j) {
            const uint64_t t0 = lvl_tri[l][j], t1 = lvl_tri[l][j + 1];
            float mn[3] = {INF, INF, INF}, mx[3] = {-INF, -INF, -INF};
            for (uint64_t v = 3 * t0; v < 3 * t1; ++v)
                for (int i = 0; i < 3; ++i) {
                    mn[i] = std::fmin(mn[i], h.tris[4 * v + i]);
                    mx[i] = std::fmax(mx[i], h.tris[4 * v + i]);
                }
            const V3 c = V3{(mn[0] + mx[0]) * 0.5f, (mn[1] + mx[1]) * 0.5f, (mn[2] + mx[2]) * 0.5f};
            float r2 = 0.f;
            for (uint64_t v = 3 * t0; v < 3 * t1; ++v) {
                const float* p = &h.tris[4 * v];
                const V3 d = V3{p[0] - c.x, p[1] - c.y, p[2] - c.z};
                r2 = std::fmax(r2, dot(d, d));
            }
            float* s = &h.sph[4ull * (h.off[l] + j)];
            s[0] = c.x;
            s[1] = c.y;
            s[2] = c.z;
            s[3] = std::sqrt(r2) * kRadSlack;
            // the padded box and child link (objh.cu k_level_spheres)
            const uint32_t* k = &h.kid[h.koff[l] + j];
            const uint32_t child_off = (l == 0) ? 0u : h.off[l - 1];
            float* bx = &h.box[8ull * (h.off[l] + j)];
            for (int i = 0; i < 3; ++i) {
                bx[i] = mn[i] - pad;
                bx[4 + i] = mx[i] + pad;
            }
            // level 0: the first triangle; above: the node's whole single-ray stack entry
            bx[3] = u2f(l == 0 ? k[0] : (l << 27) | ((k[1] - k[0] - 1u) << 24) | ((child_off + k[0]) & 0xFFFFFFu));
            bx[7] = u2f(k[1] - k[0]);
        }
    }
    build_box_tree(h, pad);
}

// The single-ray box tree (wide.cu), restated: PLOC (Meister & Bittner 2018) over the Morton-ordered
// triangles h.tris with search radius 8 -- each pass every cluster's nearest neighbour by merged-box area
// (x y + y z) + x z (ties: the lower position), mutual pairs merge into a node at the lower position,
// merged nodes numbered in position order -- then the triangles in depth-first order (left first), then the
// collapse to 8-wide nodes chosen by dynamic programming on the traversal cost (f(x, 1) = min(A (8 +
// triangles) for a cluster of at most `cluster`, min over j of A (16 + j) + f(x, j)); f(x, k >= 2) = min
// over i of f(left, i) + f(right, k - i); FP32, ties to the cluster, the smaller j, the smaller i), laid
// out breadth first, every node's decomposition (left parts first) in consecutive slots from slot 1.
namespace {
struct PBox {
    float lo[3], hi[3];
    uint32_t cnt;
};
inline float parea(const float* a, const float* b) {
    const float x = b[0] - a[0], y = b[1] - a[1], z = b[2] - a[2];
    return (x * y + y * z) + x * z;
}
inline float pmerged(const PBox& p, const PBox& q) {
    float a[3], b[3];
    for (int i = 0; i < 3; ++i) {
        a[i] = std::fmin(p.lo[i], q.lo[i]);
        b[i] = std::fmax(p.hi[i], q.hi[i]);
    }
    return parea(a, b);
}
}  // namespace

static void build_box_tree(ObjH& h, float pad) {
    const uint32_t n = h.T;
    h.wbox.clear();
    h.wtris.clear();
    h.wroot = 0;
    if (n == 0) return;
    std::vector<PBox> nodes(n);
    std::vector<std::pair<int32_t, int32_t>> ch(n);
    std::vector<int32_t> cur(n);
    for (uint32_t k = 0; k < n; ++k) {
        const float* v = &h.tris[12ull * k];
        PBox b;
        for (int i = 0; i < 3; ++i) {
            b.lo[i] = std::fmin(std::fmin(v[i], v[4 + i]), v[8 + i]);
            b.hi[i] = std::fmax(std::fmax(v[i], v[4 + i]), v[8 + i]);
        }
        b.cnt = 1;
        nodes[k] = b;
        ch[k] = {-(int32_t)k - 1, 0};
        cur[k] = (int32_t)k;
    }
    const int64_t R = 8;
    while (cur.size() > 1) {
        const int64_t m = (int64_t)cur.size();
        std::vector<int64_t> nn(m);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < m; ++i) {
            float best = INF;
            int64_t bj = -1;
            for (int64_t j = std::max<int64_t>(0, i - R); j <= std::min<int64_t>(m - 1, i + R); ++j) {
                if (j == i) continue;
                const float a = pmerged(nodes[cur[i]], nodes[cur[j]]);
                if (a < best) {
                    best = a;
                    bj = j;
                }
            }
            nn[i] = bj;
        }
        std::vector<int32_t> nxt;
        nxt.reserve(m);
        for (int64_t i = 0; i < m; ++i) {
            const int64_t j = nn[i];
            const bool mutual = j >= 0 && nn[j] == i;
            if (mutual && i > j) continue;
            if (mutual) {
                const PBox& p = nodes[cur[i]];
                const PBox& q = nodes[cur[j]];
                PBox b;
                for (int a = 0; a < 3; ++a) {
                    b.lo[a] = std::fmin(p.lo[a], q.lo[a]);
                    b.hi[a] = std::fmax(p.hi[a], q.hi[a]);
                }
                b.cnt = p.cnt + q.cnt;
                nodes.push_back(b);
                ch.push_back({cur[i], cur[j]});
                nxt.push_back((int32_t)nodes.size() - 1);
            } else {
                nxt.push_back(cur[i]);
            }
        }
        cur.swap(nxt);
    }
    const int32_t root = cur[0];
    // depth-first triangle order: a node's children always have lower ids, so ids descending visit every
    // parent before its children
    std::vector<uint32_t> first(nodes.size(), 0);
    for (int64_t x = (int64_t)nodes.size() - 1; x >= (int64_t)n; --x) {
        first[ch[x].first] = first[x];
        first[ch[x].second] = first[x] + nodes[ch[x].first].cnt;
    }
    h.wtris.resize(12ull * n);
    for (uint32_t k = 0; k < n; ++k) std::memcpy(&h.wtris[12ull * first[k]], &h.tris[12ull * k], 48);
    // collapse costs (wide.cu): f(x, 1..8) and choices, children before parents (ids ascending)
    const uint32_t G = h.cluster;
    const size_t N = nodes.size();
    const float FINF = INF;
    std::vector<float> fc(8 * N, FINF);
    std::vector<uint32_t> choice(N, 0u);
    const uint32_t CH_CLUSTER = 1u << 24;
    for (size_t x = 0; x < N; ++x) {
        float* f = &fc[8 * x];
        uint32_t chw = 0;
        if (x >= n) {
            const float* fl = &fc[8ull * ch[x].first];
            const float* fr = &fc[8ull * ch[x].second];
            for (uint32_t k = 2; k <= 8; ++k) {
                float best = FINF;
                uint32_t bi = 1;
                for (uint32_t i = 1; i < k; ++i) {
                    const float c = fl[i - 1] + fr[k - i - 1];
                    if (c < best) {
                        best = c;
                        bi = i;
                    }
                }
                f[k - 1] = best;
                chw |= bi << (3u * (k - 2u));
            }
        }
        const float A = parea(nodes[x].lo, nodes[x].hi);
        float best = FINF;
        uint32_t bj = 0;
        for (uint32_t j = 2; j <= 8; ++j) {
            const float c = A * (16.0f + (float)j) + f[j - 1];
            if (c < best) {
                best = c;
                bj = j;
            }
        }
        const float ccl = nodes[x].cnt <= G ? A * (8.0f + (float)nodes[x].cnt) : FINF;
        if (ccl <= best) {
            f[0] = ccl;
            chw |= CH_CLUSTER;
        } else {
            f[0] = best;
            chw |= (bj - 2u) << 21;
        }
        choice[x] = chw;
    }
    // a node's children: the slots of its decomposition, left parts first; at the root a cluster is its
    // own single child
    auto expand = [&](int32_t x, bool at_root, std::vector<int32_t>& c) {
        c.clear();
        if (choice[x] & CH_CLUSTER) {
            if (at_root) c.push_back(x);
            return;
        }
        std::vector<std::pair<int32_t, uint32_t>> st{{x, ((choice[x] >> 21) & 7u) + 2u}};
        while (!st.empty()) {
            const auto [y, k] = st.back();
            st.pop_back();
            if (k == 1u) {
                c.push_back(y);
                continue;
            }
            const uint32_t si = (choice[y] >> (3u * (k - 2u))) & 7u;
            st.push_back({ch[y].second, k - si});
            st.push_back({ch[y].first, si});
        }
    };
    h.wbox.assign(8, 0.0f);  // slot 0: unused (the root has no slot)
    std::vector<std::pair<int32_t, uint32_t>> level{{root, 0u}}, next;
    std::vector<int32_t> c;
    uint32_t slots = 1;
    bool at_root = true;
    while (!level.empty()) {
        next.clear();
        for (const auto& it : level) {
            expand(it.first, at_root, c);
            const uint32_t f = slots;
            uint32_t lw, hw;
            if (c.empty()) {
                lw = first[it.first];
                hw = 0x80000000u | nodes[it.first].cnt;
            } else {
                lw = (1u << 27) | (((uint32_t)c.size() - 1u) << 24) | (f & 0xFFFFFFu);
                hw = (uint32_t)c.size();
                for (size_t q = 0; q < c.size(); ++q) next.push_back({c[q], f + (uint32_t)q});
                slots += (uint32_t)c.size();
            }
            if (at_root) {
                h.wroot = lw;
                continue;
            }
            const PBox& b = nodes[it.first];
            float* bx = &h.wbox[8ull * it.second];
            for (int i = 0; i < 3; ++i) {
                bx[i] = b.lo[i] - pad;
                bx[4 + i] = b.hi[i] + pad;
            }
            bx[3] = u2f(lw);
            bx[7] = u2f(hw);
        }
        h.wbox.resize(8ull * slots, 0.0f);
        level.swap(next);
        at_root = false;
    }
}

// UpdateVertex (RayTracer.cu:448-511): per vertex of triangle t, the object obj[t]'s row-major model
// matrix on the position (w kept) and normal matrix (NULL: the model matrix) on the normal, summed in j
// order from 0, the normal renormalised with w = 0.
void orc_transform(const float* pos_rest, const float* nrm_rest, const uint32_t* obj, uint32_t T, uint32_t nobj,
                   const float* model, const float* normal, float* pos, float* nrm) {
    auto apply = [](const float* m, const float* v, float* o) {
        for (int i = 0; i < 4; ++i) {
            float s = 0.0f;
            s += m[4 * i + 0] * v[0];
            s += m[4 * i + 1] * v[1];
            s += m[4 * i + 2] * v[2];
            s += m[4 * i + 3] * v[3];
            o[i] = s;
        }
    };
    for (uint64_t x = 0; x < 3ull * T; ++x) {
        uint32_t id = obj[x / 3];
        if (id >= nobj) id = 0;
        float q[4];
        apply(model + 16ull * id, pos_rest + 4 * x, q);
        pos[4 * x] = q[0];
        pos[4 * x + 1] = q[1];
        pos[4 * x + 2] = q[2];
        pos[4 * x + 3] = pos_rest[4 * x + 3];
        apply((normal ? normal : model) + 16ull * id, nrm_rest + 4 * x, q);
        const V3 u = normalize(V3{q[0], q[1], q[2]});
        nrm[4 * x] = u.x;
        nrm[4 * x + 1] = u.y;
        nrm[4 * x + 2] = u.z;
        nrm[4 * x + 3] = 0.0f;
    }
}

// Builds the object-sphere hierarchy; returns a handle used by the traversal / intersection calls.
void* orc_objh_build(const float* pos, uint32_t T, uint32_t cluster, const float lo[3], const float hi[3]) {
    ObjH* h = new ObjH();
    build_objh(pos, T, cluster, lo, hi, *h);
    g_last_objh = h;
    return h;
}
void orc_objh_free(void* hp) { delete static_cast<ObjH*>(hp); }
void orc_objh_boxes(void* hp, float* out) {
    const ObjH& h = *static_cast<ObjH*>(hp);
    std::memcpy(out, h.box.data(), 4ull * h.box.size());
}
// the single-ray box tree: number of slots (slot 0 unused) and the root's entry; boxes (8 floats per slot)
// and triangles (12 floats each, its depth-first order) when the pointers are not NULL
uint32_t orc_objh_box_tree(void* hp, uint32_t* root, float* boxes, float* tris) {
    const ObjH& h = *static_cast<ObjH*>(hp);
    if (root) *root = h.wroot;
    if (boxes) std::memcpy(boxes, h.wbox.data(), 4ull * h.wbox.size());
    if (tris) std::memcpy(tris, h.wtris.data(), 4ull * h.wtris.size());
    return (uint32_t)(h.wbox.size() / 8);
}
uint32_t orc_objh_levels(void* hp) { return static_cast<ObjH*>(hp)->levels; }
uint32_t orc_objh_level_size(void* hp, uint32_t l) { return static_cast<ObjH*>(hp)->size[l]; }
// child ranges of every level, level after level (size[l] + 1 entries each; level 0: triangle ranges)
uint32_t orc_objh_kid_count(void* hp) { return (uint32_t)static_cast<ObjH*>(hp)->kid.size(); }
void orc_objh_kids(void* hp, uint32_t* out) {
    const ObjH* h = static_cast<ObjH*>(hp);
    std::memcpy(out, h->kid.data(), 4ull * h->kid.size());
}
void orc_objh_get(void* hp, uint32_t* order, float* tris, float* spheres) {
    const ObjH* h = static_cast<ObjH*>(hp);
    if (order) std::memcpy(order, h->order.data(), 4ull * h->T);
    if (tris) std::memcpy(tris, h->tris.data(), 48ull * h->T);
    if (spheres) std::memcpy(spheres, h->sph.data(), 4ull * h->sph.size());
}

// ---------------------------------------------------------------- traversal + intersection
// Candidate set of the hierarchy-vs-hierarchy traversal (RayTracer.cu:1152-1496 semantics: a packet
// reaches a triangle cluster iff it passes the node test at the cluster and at all its ancestors).
// Written sorted ascending; returns the count (capped by cap). node_tests_out may be NULL.
uint64_t orc_traverse(void* hp, const void* nodes_in, uint32_t n, uint32_t max_rays, uint32_t P, uint64_t* cand,
                      uint64_t cap, uint64_t* node_tests_out) {
    const ObjH& h = *static_cast<ObjH*>(hp);
    const Node* nodes = static_cast<const Node*>(nodes_in);
    uint32_t off[4];
    orc_hierarchy_offsets(max_rays, P, off);
    const uint32_t n0 = (n + P - 1) / P;
    std::vector<std::vector<uint64_t>> per(n0);
    uint64_t tests = 0;
    if (h.levels == 0) return 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : tests)
    for (int64_t p = 0; p < (int64_t)n0; ++p) {
        const Node& nd = nodes[off[0] + p];
        if (nd.count == 0) continue;
        std::vector<uint32_t> cl;
        uint64_t t = 0;
        traverse_packet(nd, h, h.levels, 0, cl, t);
        tests += t;
        for (uint32_t c : cl) per[p].push_back(((uint64_t)p << 32) | c);
    }
    std::vector<uint64_t> all;
    for (auto& v : per) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end());
    const uint64_t m = std::min<uint64_t>(all.size(), cap);
    if (cand) std::memcpy(cand, all.data(), 8 * m);
    if (node_tests_out) *node_tests_out = tests;
    return all.size();
}

// CalculateShadowRayIntersections / CalculateReflectionRayIntersections (RayTracer.cu:1498-1774) over
// the candidates. Outputs indexed by ray slot; caller initialises flags (0) / hits (HIT_NONE).
void orc_intersect(void* hp, const float* rays_in, const uint32_t* ids, uint32_t n, uint32_t P,
                   const uint64_t* cand, uint64_t ncand, int any, uint32_t* flags, uint64_t* hits) {
    const ObjH& h = *static_cast<ObjH*>(hp);
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
    for (uint64_t c = 0; c < ncand; ++c) {
        const uint32_t packet = (uint32_t)(cand[c] >> 32), cluster = (uint32_t)cand[c];
        for (uint32_t j = 0; j < P; ++j) {
            const uint32_t k = packet * P + j;
            if (k >= n) break;
            const uint32_t id = ids ? ids[k] : k;
            const Ray& r = rays[id];
            if (!(r.tmax > r.tmin)) continue;
            if (!ray_hits_sphere(r, &h.sph[4ull * cluster])) continue;
            const RayWT w = wt_setup(r);
            uint32_t t0, t1;
            cluster_tris(h, cluster, t0, t1);
            for (uint32_t t = t0; t < t1; ++t) {
                const float* v = &h.tris[12ull * t];
                float th;
                if (wt_hit(w, v, v + 4, v + 8, th)) {
                    if (any) {
                        flags[id] = OCCLUDED;
                        break;
                    }
                    const uint64_t key = hit_key(th, f2u(v[3]));
                    if (key < hits[id]) hits[id] = key;
                }
            }
        }
    }
}

// Traces rays by per-ray box descent from the root (the batched form's rays-only traversal, fused.cu
// k_fused_rays) on all host threads. Outputs per ray: flags (any) or hits (closest); per_ray (nullable)
// gets node tests and triangle tests per ray (2 x u32). counters = total node tests, triangle tests.
// Returns 0 on a job-stack overflow (the GPU raises RSH_DEVERR_OVERFLOW there), else 1.
int orc_trace_rays_box(void* hp, const float* rays_in, uint32_t n, int any, uint32_t* flags, uint64_t* hits,
                       uint32_t* per_ray, uint64_t* counters) {
    const ObjH& h = *static_cast<ObjH*>(hp);
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
    uint64_t nt = 0, tt = 0;
    int ok = 1;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : nt, tt) reduction(& : ok)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        bool occ = false;
        uint64_t best = HIT_NONE, a = 0, b = 0;
        if (!ray_descend_box(h, rays[i], any != 0, occ, best, a, b)) ok = 0;
        if (any) flags[i] = occ ? OCCLUDED : 0u;
        else hits[i] = best;
        if (per_ray) {
            per_ray[2 * i] = (uint32_t)a;
            per_ray[2 * i + 1] = (uint32_t)b;
        }
        nt += a;
        tt += b;
    }
    if (counters) {
        counters[0] = nt;
        counters[1] = tt;
    }
    return ok;
}

// Brute force over all triangles (CUDA-Naive-Engine RayTracer.cu:276-291 any-hit, :344-360 closest),
// one triangle after the other with the scalar watertight test. Kept as the plain statement of the
// semantics; orc_brute gives the same results faster.
void orc_brute_scalar(const float* pos, uint32_t T, const float* rays_in, uint32_t n, int any, uint32_t* flags,
                      uint64_t* hits) {
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const Ray& r = rays[i];
        if (any) flags[i] = 0;
        else hits[i] = HIT_NONE;
        if (!(r.tmax > r.tmin)) continue;
        const RayWT w = wt_setup(r);
        uint64_t best = HIT_NONE;
        for (uint32_t t = 0; t < T; ++t) {
            const float* v = pos + 12ull * t;
            float th;
            if (wt_hit(w, v, v + 4, v + 8, th)) {
                if (any) {
                    flags[i] = OCCLUDED;
                    break;
                }
                const uint64_t key = hit_key(th, t);
                if (key < best) best = key;
            }
        }
        if (!any) hits[i] = best;
    }
}

// Brute force over all triangles, same results as orc_brute_scalar (every ray against every triangle), in
// two steps. (1) For a tile of rays and a block of triangles, the watertight test's 2-D edge functions U,
// V, W are computed in FP32 exactly as wt_hit computes them (same operations, same order, no contraction)
// over a structure-of-arrays copy of the triangles, in a loop the compiler vectorises; a triangle stays a
// candidate unless wt_hit would reject it at its sign test with no edge function exactly zero (a zero sends
// wt_hit to its double-precision fallback, so such a triangle stays a candidate too). (2) Every candidate
// goes through wt_hit itself. A ray's line crosses few triangles, so (2) is cheap and (1) is the whole
// cost. pos: original order, 12 floats per triangle. Fills flags (any) or hits (closest) for every ray.
void orc_brute(const float* pos, uint32_t T, const float* rays_in, uint32_t n, int any, uint32_t* flags,
               uint64_t* hits) {
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
    constexpr uint32_t TB = 2048;  // triangles per block: 72 KB of the SoA copy, reused by a tile of rays
    constexpr uint32_t RT = 32;    // rays per tile
    std::vector<float> soa(9ull * T);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < (int64_t)T; ++t)
        for (int v = 0; v < 3; ++v)
            for (int c = 0; c < 3; ++c) soa[(3ull * v + c) * T + t] = pos[12ull * t + 4 * v + c];
    const int64_t tiles = ((int64_t)n + RT - 1) / RT;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t tile = 0; tile < tiles; ++tile) {
        const uint32_t r0 = (uint32_t)tile * RT, r1 = std::min<uint32_t>(n, r0 + RT);
        RayWT w[RT];
        uint64_t best[RT];
        bool live[RT];
        for (uint32_t i = r0; i < r1; ++i) {
            const Ray& r = rays[i];
            live[i - r0] = r.tmax > r.tmin;
            if (live[i - r0]) w[i - r0] = wt_setup(r);
            best[i - r0] = HIT_NONE;
        }
        alignas(64) uint8_t cand[TB];
        for (uint32_t b0 = 0; b0 < T; b0 += TB) {
            const uint32_t nb = std::min<uint32_t>(TB, T - b0);
            for (uint32_t j = 0; j < r1 - r0; ++j) {
                if (!live[j]) continue;
                const RayWT& q = w[j];
                const float* ax = &soa[(0ull + q.kx) * T + b0];
                const float* ay = &soa[(0ull + q.ky) * T + b0];
                const float* az = &soa[(0ull + q.kz) * T + b0];
                const float* bx = &soa[(3ull + q.kx) * T + b0];
                const float* by = &soa[(3ull + q.ky) * T + b0];
                const float* bz = &soa[(3ull + q.kz) * T + b0];
                const float* cx = &soa[(6ull + q.kx) * T + b0];
                const float* cy = &soa[(6ull + q.ky) * T + b0];
                const float* cz = &soa[(6ull + q.kz) * T + b0];
                const float ox = q.o[q.kx], oy = q.o[q.ky], oz = q.o[q.kz];
                const float sx = q.s[0], sy = q.s[1];
                uint32_t any_c = 0;
#pragma omp simd reduction(| : any_c)
                for (uint32_t t = 0; t < nb; ++t) {
                    const float Akz = az[t] - oz, Bkz = bz[t] - oz, Ckz = cz[t] - oz;
                    const float Ax = (ax[t] - ox) - sx * Akz, Ay = (ay[t] - oy) - sy * Akz;
                    const float Bx = (bx[t] - ox) - sx * Bkz, By = (by[t] - oy) - sy * Bkz;
                    const float Cx = (cx[t] - ox) - sx * Ckz, Cy = (cy[t] - oy) - sy * Ckz;
                    const float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
                    const uint32_t neg = (U < 0.0f) | (V < 0.0f) | (W < 0.0f);
                    const uint32_t pos_ = (U > 0.0f) | (V > 0.0f) | (W > 0.0f);
                    const uint32_t zero = (U == 0.0f) | (V == 0.0f) | (W == 0.0f);
                    const uint32_t c = (1u - (neg & pos_)) | zero;
                    cand[t] = (uint8_t)c;
                    any_c |= c;
                }
                if (!any_c) continue;
                for (uint32_t t = 0; t < nb; ++t) {
                    if (!cand[t]) continue;
                    const float* v = pos + 12ull * (b0 + t);
                    float th;
                    if (wt_hit(q, v, v + 4, v + 8, th)) {
                        if (any) {
                            live[j] = false;
                            best[j] = 0;  // occluded
                            break;
                        }
                        const uint64_t key = hit_key(th, b0 + t);
                        if (key < best[j]) best[j] = key;
                    }
                }
            }
        }
        for (uint32_t i = r0; i < r1; ++i) {
            if (any) flags[i] = best[i - r0] == 0 ? OCCLUDED : 0u;
            else hits[i] = best[i - r0];
        }
    }
}

// Second-nearest hit distance per ray (for the near-tie exception of the hit-ID comparison).
void orc_brute_second(const float* pos, uint32_t T, const float* rays_in, uint32_t n, float* t1, float* t2) {
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const Ray& r = rays[i];
        float a = INF, b = INF;
        if (r.tmax > r.tmin) {
            const RayWT w = wt_setup(r);
            for (uint32_t t = 0; t < T; ++t) {
                const float* v = pos + 12ull * t;
                float th;
                if (wt_hit(w, v, v + 4, v + 8, th)) {
                    if (th < a) {
                        b = a;
                        a = th;
                    } else if (th < b) {
                        b = th;
                    }
                }
            }
        }
        t1[i] = a;
        t2[i] = b;
    }
}

// Hit resolve (RayTracer.cu:1806-1843): hit point and area-ratio barycentric normal.
void orc_resolve(const float* pos, const float* nrm, const uint32_t* mat, const float* rays_in,
                 const uint64_t* hits, const uint32_t* pix, uint32_t n, float* spos, float* snrm) {
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
#pragma omp parallel for schedule(static)
    for (int64_t kk = 0; kk < (int64_t)n; ++kk) {
        const uint32_t k = (uint32_t)kk;
        const uint32_t px = pix ? pix[k] : k;
        if (px == 0xFFFFFFFFu) continue;
        const uint64_t hk = hits[k];
        float* sp = spos + 4ull * px;
        float* sn = snrm + 4ull * px;
        if (hk == HIT_NONE) {
            for (int i = 0; i < 4; ++i) sp[i] = sn[i] = 0.f;
            continue;
        }
        const uint32_t tri = (uint32_t)hk;
        const float t = u2f((uint32_t)(hk >> 32));
        const Ray& r = rays[k];
        const V3 p = V3{r.o[0] + r.d[0] * t, r.o[1] + r.d[1] * t, r.o[2] + r.d[2] * t};
        const float* v = pos + 12ull * tri;
        const V3 a = V3{v[0], v[1], v[2]}, b = V3{v[4], v[5], v[6]}, c = V3{v[8], v[9], v[10]};
        const float abc = length(cross(sub(b, a), sub(c, a)));
        const float pbc = length(cross(sub(b, p), sub(c, p)));
        const float pca = length(cross(sub(a, p), sub(c, p)));
        const float b0 = pbc / abc, b1 = pca / abc, b2 = (1.0f - b0) - b1;
        const float* q = nrm + 12ull * tri;
        sp[0] = p.x;
        sp[1] = p.y;
        sp[2] = p.z;
        sp[3] = 1.0f;
        for (int i = 0; i < 3; ++i) sn[i] = (q[i] * b0 + q[4 + i] * b1) + q[8 + i] * b2;
        sn[3] = u2f(mat ? mat[tri] : 0u);
    }
}

// ---------------------------------------------------------------- the whole algorithm on the CPU
// One keyed batch through compress -> sort -> decompress -> build -> traverse+intersect (per packet, all
// host threads), with the same hybrid traversal as the GPU's batched form: packet tests above
// `ray_level`, per-ray descent below. Used as the CPU baseline; returns the number of traced rays.
// stage_ms (8 floats) gets per-stage wall times: compress, sort, decompress, build, traverse+intersect.
uint32_t orc_trace_keyed(void* hp, const float* rays_in, const uint32_t* keys, uint32_t n_slots, uint32_t key_bits,
                         uint32_t P, int any, uint32_t* flags, uint64_t* hits, float* stage_ms,
                         uint64_t* counters /* node tests, tri tests */, uint32_t ray_level) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return std::chrono::duration<float, std::milli>(b - a).count();
    };
    const ObjH& h = *static_cast<ObjH*>(hp);
    const Ray* rays = reinterpret_cast<const Ray*>(rays_in);
    std::vector<uint32_t> trimmed(n_slots), ckeys(n_slots + 1), cbases(n_slots + 1);
    uint32_t counts[2];
    auto t0 = clk::now();
    orc_compress(keys, n_slots, trimmed.data(), ckeys.data(), cbases.data(), nullptr, counts);
    const uint32_t R = counts[0], C = counts[1];
    auto t1 = clk::now();
    std::vector<uint32_t> sk(C), sv(C);
    orc_sort_pairs(ckeys.data(), nullptr, C, key_bits, sk.data(), sv.data());
    auto t2 = clk::now();
    std::vector<uint32_t> sorted(R);
    orc_decompress(sk.data(), sv.data(), cbases.data(), trimmed.data(), R, C, nullptr, sorted.data());
    auto t3 = clk::now();
    uint32_t off[4];
    const uint32_t cap = orc_hierarchy_offsets(R, P, off);
    std::vector<Node> nodes(cap ? cap : 1);
    orc_build_rsh(rays_in, sorted.data(), R, R, P, nodes.data());
    auto t4 = clk::now();
    const uint32_t n0 = (R + P - 1) / P;
    uint64_t ntests = 0, ttests = 0;
    if (h.levels) {
        // per packet: packet tests above ray_level (and not at all for full cones), then each ray descends
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : ntests, ttests)
        for (int64_t p = 0; p < (int64_t)n0; ++p) {
            Node nd = nodes[off[0] + p];
            if (nd.count == 0) continue;
            uint32_t ids[64];
            RayWT ws[64];
            uint64_t best[64];
            bool occl[64];
            uint32_t nr = 0;
            for (uint32_t j = 0; j < P; ++j) {
                const uint32_t k = (uint32_t)p * P + j;
                if (k >= R) break;
                const uint32_t id = sorted[k];
                if (!(rays[id].tmax > rays[id].tmin)) continue;
                ids[nr] = id;
                ws[nr] = wt_setup(rays[id]);
                best[nr] = HIT_NONE;
                occl[nr] = false;
                ++nr;
            }
            auto descend_all = [&](uint32_t L, uint32_t idx) {
                for (uint32_t j = 0; j < nr; ++j)
                    if (!occl[j]) occl[j] = ray_descend(h, rays[ids[j]], ws[j], L, idx, any != 0, best[j], ntests, ttests);
            };
            if (!(nd.cos_spread > 0.0f) || h.levels <= ray_level) {
                descend_all(h.levels, 0);
            } else {
                uint32_t stk[96];
                int sp = 0;
                stk[sp++] = h.levels << 24;
                while (sp > 0) {
                    const uint32_t e = stk[--sp];
                    const uint32_t L = e >> 24, idx = e & 0xFFFFFFu;
                    if (L <= ray_level) {
                        descend_all(L, idx);
                        if (any) {
                            bool all = true;
                            for (uint32_t j = 0; j < nr; ++j) all = all && occl[j];
                            if (all) break;
                        }
                        continue;
                    }
                    const uint32_t cl = L - 1;
                    uint32_t first, cnt;
                    children(h, L, idx, first, cnt);
                    float te[8];
                    uint32_t ci[8];
                    uint32_t nh = 0;
                    for (uint32_t c = 0; c < cnt; ++c) {
                        const float* q = &h.sph[4ull * (h.off[cl] + first + c)];
                        ++ntests;
                        if (!node_hits_sphere(nd, q)) continue;
                        const V3 dc = V3{q[0] - nd.c[0], q[1] - nd.c[1], q[2] - nd.c[2]};
                        const float tc = length(dc) - q[3];
                        uint32_t k = nh++;
                        while (k > 0 && te[k - 1] < tc) {
                            te[k] = te[k - 1];
                            ci[k] = ci[k - 1];
                            --k;
                        }
                        te[k] = tc;
                        ci[k] = first + c;
                    }
                    if (cl == 0) {  // ray_level 0: packets reach the clusters; rays filter and test them
                        for (uint32_t k = nh; k-- > 0;) {
                            const uint32_t c = ci[k];
                            for (uint32_t j = 0; j < nr; ++j) {
                                if (occl[j]) continue;
                                const Ray& ry = rays[ids[j]];
                                if (!ray_hits_sphere(ry, &h.sph[4ull * (h.off[0] + c)])) continue;
                                uint32_t a0, a1;
                                cluster_tris(h, c, a0, a1);
                                for (uint32_t t2i = a0; t2i < a1; ++t2i) {
                                    const float* v = &h.tris[12ull * t2i];
                                    float th;
                                    ++ttests;
                                    if (wt_hit(ws[j], v, v + 4, v + 8, th)) {
                                        if (any) {
                                            occl[j] = true;
                                            break;
                                        }
                                        const uint64_t key = hit_key(th, f2u(v[3]));
                                        if (key < best[j]) best[j] = key;
                                    }
                                }
                            }
                        }
                    } else {
                        for (uint32_t k = 0; k < nh && sp < 96; ++k) stk[sp++] = (cl << 24) | ci[k];
                    }
                    if (!any) {  // shrink the packet's reach to its rays' current closest hits
                        float rm = 0.0f;
                        for (uint32_t j = 0; j < nr; ++j) {
                            const Ray& ry = rays[ids[j]];
                            const float tb = best[j] == HIT_NONE ? ry.tmax : u2f((uint32_t)(best[j] >> 32));
                            const V3 oc = V3{ry.o[0] - nd.c[0], ry.o[1] - nd.c[1], ry.o[2] - nd.c[2]};
                            rm = std::fmax(rm, length(oc) + tb);
                        }
                        nd.reach = std::fmin(nd.reach, rm * kRadSlack);
                    }
                }
            }
            for (uint32_t j = 0; j < nr; ++j) {
                if (any) {
                    if (occl[j]) flags[ids[j]] = OCCLUDED;
                } else if (best[j] < hits[ids[j]]) {
                    hits[ids[j]] = best[j];
                }
            }
        }
    }
    auto t5 = clk::now();
    if (stage_ms) {
        stage_ms[0] = ms(t0, t1);
        stage_ms[1] = ms(t1, t2);
        stage_ms[2] = ms(t2, t3);
        stage_ms[3] = ms(t3, t4);
        stage_ms[4] = ms(t4, t5);
    }
    if (counters) {
        counters[0] = ntests;
        counters[1] = ttests;
    }
    return R;
}

}  // extern "C"
