// Host-side launchers of the sm_103a kernels (one translation unit per stage). Internal to the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rsh.h"

// Device error word bits (bounded waits that gave up, buffer overflows).
#ifndef RSH_DEVERR_TIMEOUT
#define RSH_DEVERR_TIMEOUT 1u
#define RSH_DEVERR_OVERFLOW 2u
#endif

namespace rsh {

// Counts this library's kernel launches (rsh_kernel_launches).
void note_launch(unsigned n = 1);

struct HashP {
    float lo[3];
    float scale[3];
    uint32_t grid_bits, dir_log2, tag_bits, key_bits;
};
inline HashP to_hashp(const rsh_hash_params& h) {
    HashP p;
    for (int i = 0; i < 3; ++i) {
        p.lo[i] = h.lo[i];
        p.scale[i] = h.scale[i];
    }
    p.grid_bits = h.grid_bits;
    p.dir_log2 = h.dir_log2;
    p.tag_bits = h.tag_bits;
    p.key_bits = h.key_bits;
    return p;
}

struct LightsP {
    uint32_t count;
    uint32_t samples;  // shadow rays per light: 1, or 16 (soft shadows)
    float pos[8][3];
};

struct CameraP {
    float eye[3], dir[3], right[3], up[3];
};

// ---- raygen + hash (raygen.cu)
cudaError_t launch_raygen_primary(const CameraP& cam, uint32_t w, uint32_t h, rsh_ray* rays,
                                  uint32_t* pixel_of_ray, cudaStream_t s);
// Keys of a batched call written by ray generation itself (the batched form of a frame): key = tag |
// (ray hash >> drop) or RSH_KEY_NONE, the segment's ray count (one atomic per block into *count), and the
// segment's results prefilled (flags 0 for an any-hit segment, hits RSH_HIT_NONE otherwise), so the batch
// need not read the rays back to hash them.
struct BatchKeyOut {
    uint32_t* keys = nullptr;      // the batch's key array at the segment's first slot; null: not used
    uint32_t tag = 0;
    uint32_t drop = 0;
    HashP hp{};                    // the segment scene's hash (tag 0)
    uint32_t* count = nullptr;
    uint32_t* flags = nullptr;
    unsigned long long* hits = nullptr;
};
cudaError_t launch_raygen_shadow(const float4* spos, const float4* snrm, uint32_t w, uint32_t h,
                                 const LightsP& lights, float eps, const HashP& hp, rsh_ray* rays,
                                 uint32_t* keys, cudaStream_t s, const BatchKeyOut& bk = BatchKeyOut());
cudaError_t launch_raygen_reflect(const float4* spos, const float4* snrm, const rsh_ray* prev,
                                  const float eye[3], uint32_t w, uint32_t h, float eps,
                                  float jitter, uint32_t seed, uint32_t bounce, const HashP& hp,
                                  rsh_ray* rays, uint32_t* keys, cudaStream_t s,
                                  const BatchKeyOut& bk = BatchKeyOut());
cudaError_t launch_raygen_refract(const float4* spos, const float4* snrm, const rsh_ray* prev, const float eye[3],
                                  uint32_t w, uint32_t h, float eps, float eta, const HashP& hp, rsh_ray* rays,
                                  uint32_t* keys, cudaStream_t s);
cudaError_t launch_hash(const rsh_ray* rays, uint32_t n, const HashP& hp, uint32_t tag,
                        uint32_t* keys, cudaStream_t s);
// Segmented hash for the batched form: segment s covers rays [seg_start[s], seg_start[s+1]) of the
// concatenated ray array; tag = segment index; hash params per segment (scene bounds).
cudaError_t launch_hash_segments(const rsh_ray* rays, uint32_t n, const uint32_t* seg_start,
                                 uint32_t nseg, const HashP* hps_dev, uint32_t tag_shift,
                                 uint32_t* keys, cudaStream_t s);

// ---- trim + compress (compress.cu)
size_t compress_scratch_bytes(uint32_t n_slots);
cudaError_t launch_compress(const uint32_t* keys, uint32_t n_slots, uint32_t* trimmed_ids,
                            uint32_t* chunk_keys, uint32_t* chunk_bases, uint32_t* counts,
                            void* scratch, uint32_t* err, cudaStream_t s);
cudaError_t launch_chunk_sizes(const uint32_t* chunk_bases, const uint32_t* counts, uint32_t max_chunks,
                               uint32_t* chunk_sizes, cudaStream_t s);

// ---- onesweep radix sort (sort.cu)
size_t sort_scratch_bytes(uint32_t n_max, uint32_t key_bits);
size_t sort_selftest_scratch_bytes();
cudaError_t sort_selftest_timeout(void* scratch, uint32_t* err, uint32_t spin_limit, cudaStream_t s);
cudaError_t launch_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                              uint32_t* vals_out, uint32_t n_max, const uint32_t* d_count,
                              uint32_t key_bits, void* scratch, uint32_t* err, cudaStream_t s);

// ---- decompress (decompress.cu)
size_t decompress_scratch_bytes(uint32_t max_chunks);
// Batched layout target of decompression: ray k of the sorted order (segment tag = key >> tag_shift)
// is written to padded[k + seg_delta[tag]] instead of sorted_ids[k].
struct PaddedOut {
    const uint32_t* seg_delta;
    uint32_t tag_shift;
    uint32_t max_padded;
    uint32_t* padded;
};
cudaError_t launch_decompress(const uint32_t* sorted_chunk_keys, const uint32_t* sorted_chunk_vals,
                              const uint32_t* chunk_bases, const uint32_t* trimmed_ids,
                              const uint32_t* counts, uint32_t max_rays, uint32_t* sorted_keys,
                              uint32_t* sorted_ids, void* scratch, uint32_t* err, cudaStream_t s,
                              const PaddedOut* padded_out = nullptr);

// ---- ray-space hierarchy build (build.cu)
uint32_t hierarchy_capacity(uint32_t max_rays, uint32_t packet, uint32_t offsets[4]);
cudaError_t launch_build_rsh(const rsh_ray* rays, const uint32_t* sorted_ids, uint32_t max_rays,
                             const uint32_t* d_count, uint32_t packet, rsh_node* nodes,
                             cudaStream_t s);

// ---- object-sphere hierarchy (objh.cu)
struct ObjHierarchy {
    uint32_t tri_count = 0;
    uint32_t cluster = 8;
    uint32_t levels = 0;           // level 0 = clusters; levels-1 = top (<= 8 nodes)
    uint32_t level_off[16] = {};   // offsets into spheres
    uint32_t level_size[16] = {};
    float4* spheres = nullptr;     // all levels
    uint32_t* kids = nullptr;      // per level l (at level_off[l] + l): level_size[l] + 1 child-range starts
    float4* tris = nullptr;        // cluster order, 3 per triangle, v0.w = original id bits
    uint32_t* order = nullptr;     // cluster slot -> original triangle id
    float4* boxes = nullptr;       // per node, all levels like spheres: padded box lo, hi; lo.w / hi.w: child link
    // the single-ray box tree (wide.cu): 8-wide, mixed depth, 2 float4 per slot; triangles in its own
    // depth-first order (v0.w = original id bits); wroot = the root's stack entry
    float4* wboxes = nullptr;
    float4* wtris = nullptr;
    uint32_t wroot = 0;
    uint32_t wslots = 0;
    // the same tree as traversal records (14 float4 per node: child boxes plane by plane, child entries)
    float4* wnodes = nullptr;
    uint32_t wnode_count = 0;
    uint32_t wnroot = 0;           // the root's entry in record form
};
// A traversal record of the box tree: REC_F4 float4 (the eight children's box planes lo x, hi x, lo y, hi y,
// lo z, hi z, 8 floats each, then their eight stack entries); a node's entry is REC_NODE | (children - 1)
// << 28 | record index, a cluster's its first triangle | (triangles - 1) << 23.
constexpr uint32_t REC_F4 = 14;
constexpr uint32_t REC_NODE = 0x80000000u;
// Builds the single-ray box tree from h.tris (Morton order) and h.cluster; boxes widened by `pad`.
cudaError_t build_box_tree(ObjHierarchy& h, float pad, cudaStream_t s);
cudaError_t build_object_hierarchy(const float4* positions_dev, uint32_t tri_count, uint32_t cluster,
                                   const float lo[3], const float hi[3], ObjHierarchy& h,
                                   void* scratch, size_t scratch_bytes, uint32_t* err, cudaStream_t s);
size_t objh_scratch_bytes(uint32_t tri_count);

// ---- traversal (traverse.cu)
struct TravArgs {
    const rsh_node* nodes;
    uint32_t node_off[4];       // level offsets of the ray hierarchy (from max_rays)
    uint32_t max_rays;
    const uint32_t* d_count;
    uint32_t packet;
    const float4* spheres;
    const uint32_t* kids;        // object-tree child ranges (level l at lvl_off[l] + l)
    uint32_t lvl_off[16];
    uint32_t lvl_size[16];
    uint32_t levels;
    unsigned long long* cand;
    unsigned long long capacity;
    unsigned long long* cand_count;
    uint32_t* work;              // [0] = next unit, [1] = resume unit (min failed)
    uint32_t unit_end;           // units >= unit_end are left for a later pass
    uint32_t ray_level;          // >= 1: rays descend individually at and below this object-tree level and
                                 // emit per-ray candidates (sorted ray index << 32 | 1 << 31 | cluster)
    const rsh_ray* rays;         // per-ray mode: the rays (by slot) and the sorted order
    const uint32_t* sorted_ids;
    unsigned long long* node_tests;
    uint32_t* err;
};
cudaError_t launch_traverse(const TravArgs& a, cudaStream_t s);

// ---- intersection (intersect.cu)
struct IsectArgs {
    const float4* spheres;       // cluster spheres (object-hierarchy level 0)
    const uint32_t* kids;        // level 0 child ranges: cluster c holds triangles [kids[c], kids[c + 1])
    const float4* tris;
    uint32_t tri_count;
    uint32_t cluster;
    const rsh_ray* rays;
    const uint32_t* sorted_ids;
    uint32_t max_rays;
    const uint32_t* d_count;
    uint32_t packet;
    const unsigned long long* cand;
    const unsigned long long* cand_count;
    unsigned long long capacity;
    uint32_t* flags;
    unsigned long long* hits;
    unsigned long long* tri_tests;
    uint32_t per_ray;            // candidates are per ray (sorted ray index << 32 | 1 << 31 | cluster)
};
cudaError_t launch_intersect(const IsectArgs& a, bool any_hit, cudaStream_t s);

// ---- fused persistent traversal + intersection (fused.cu)
struct FusedSeg {
    const float4* spheres;
    const uint32_t* kids;          // object-tree child ranges (level l at lvl_off[l] + l)
    const float4* tris;
    const float4* boxes;           // per node (like spheres): padded box lo, hi; lo.w / hi.w: child link
    const float4* wboxes;          // the single-ray box tree (wide.cu): slots (cluster boxes), triangles,
    const float4* wtris;           // traversal records and the root's record entry
    const float4* wnodes;
    uint32_t wnroot;
    uint32_t tri_count;
    uint32_t cluster;
    uint32_t levels;
    uint32_t lvl_off[16];
    uint32_t lvl_size[16];
    uint32_t ray_begin, ray_end;   // sorted ray range of this segment
    uint32_t unit_begin;           // first work unit (level-1 node) of this segment
    uint32_t any_hit;
    uint32_t ray_level;            // object-tree level at and below which rays descend individually
    const rsh_ray* rays;           // the segment's own rays (slot - slot_base); read in place by the rays-only kernel
    uint32_t* flags;               // indexed by slot - slot_base
    unsigned long long* hits;
    uint32_t slot_base;
};
struct FusedArgs {
    const rsh_node* nodes;
    uint32_t node_off[4];
    uint32_t packet;
    const rsh_ray* rays;
    const uint32_t* sorted_ids;    // null (rays-only kernel): rays in their own order, ordered_n of them
    uint32_t ordered_n;
    const FusedSeg* segs;          // device
    uint32_t nseg;
    const uint32_t* unit_seg;      // device: work unit -> segment (size = units)
    uint32_t units_max;
    const uint32_t* d_units;       // device count of units
    uint32_t* work;
    uint32_t rays_only;            // every segment's switch level >= its tree depth: no packet phase
    uint32_t blocks_per_sm;        // CTAs per SM of the launch (0: as many as fit)
    uint32_t share_tail;           // rays-only kernel: a drained warp shares its last rays among its lanes
    unsigned long long* node_tests;
    unsigned long long* tri_tests;
    uint32_t* err;
};
cudaError_t launch_fused(const FusedArgs& a, cudaStream_t s);
// rays per work unit of the rays-only kernel (a multiple of 64, at most 256: job words hold 8 bits)
#ifndef RSH_RAYS_UNIT
#define RSH_RAYS_UNIT 64
#endif

// ---- resolve + shade (shade.cu)
cudaError_t launch_resolve(const float4* tris_orig_pos, const float4* tris_orig_nrm,
                           const uint32_t* mat_ids, const rsh_ray* rays, const unsigned long long* hits,
                           const uint32_t* pixel_of_ray, uint32_t n, float4* spos, float4* snrm,
                           cudaStream_t s);
struct ShadeArgs {
    const float4* spos;
    const float4* snrm;
    const rsh_material* materials;
    uint32_t material_count;
    const uint32_t* shadow;   // W*H*L*samples slots
    float4* accum;            // W*H rgb accumulators + weight in w
    uint32_t w, h;
    uint32_t lights;
    uint32_t samples;         // shadow samples per light (1, or 16 for soft shadows)
    rsh_light light[8];
    float eye[3];
    uint32_t bounce;
    const rsh_ray* incident;  // reflection rays that produced the surface (bounce>0), else null
};
cudaError_t launch_shade(const ShadeArgs& a, cudaStream_t s);
cudaError_t launch_pack_rgba(const float4* accum, uint32_t n, uint32_t* rgba, cudaStream_t s);

// ---- object transforms and bounds (transform.cu)
cudaError_t launch_transform(const float4* pos_rest, const float4* nrm_rest, const uint32_t* obj, uint32_t tri_count,
                             uint32_t n_objects, const float* model, const float* normal, float4* pos, float4* nrm,
                             cudaStream_t s);
size_t bounds_scratch_bytes();
cudaError_t launch_bounds(const float4* pos, uint32_t tri_count, void* scratch, float* out6, cudaStream_t s);

// ---- misc (util kernels in raygen.cu)
cudaError_t launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t s);
cudaError_t launch_fill_u64(unsigned long long* p, unsigned long long v, size_t n, cudaStream_t s);
cudaError_t launch_mark_hit_counts(const uint32_t* counts, unsigned long long* acc, cudaStream_t s);

}  // namespace rsh
