"""ctypes binding of the CPU oracle (oracle/rsh_oracle.cpp). TEST INFRASTRUCTURE ONLY.

Used by tests/, by __graft_entry__.smoke() as the checker and by bench.py's cpu_baseline / reference
legs; the product (ray-tracer_gb300/) never imports it. `build()` compiles liboracle.so with g++.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "rsh_oracle.cpp"
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared"]

KEY_NONE = 0xFFFFFFFF
HIT_NONE = 0xFFFFFFFFFFFFFFFF
OCCLUDED = 0xFFFFFFFF

# The GPU path's default configuration (rsh_config_default): origin-grid bits, direction bits (2 per
# octahedral axis), packet size, cluster size, and the plain path's switch level from packets to rays.
# The CPU baseline follows the same configuration; a CPU test checks these against the library's.
DEFAULTS = {"grid_bits": 4, "dir_log2": 6, "packet_size": 8, "cluster_size": 6, "plain_ray_level": 4,
            "ray_level": 15, "epsilon": 0.01}

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
NODE_DTYPE = np.dtype([("c", "<f4", 3), ("radius", "<f4"), ("axis", "<f4", 3), ("cos_spread", "<f4"),
                       ("sin_spread", "<f4"), ("reach", "<f4"), ("first", "<u4"), ("count", "<u4")])


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run([cxx, *CXXFLAGS, "-o", str(tmp), str(SRC)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        P, U32, U64, F, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
        sig = {
            "orc_num_threads": (C.c_int, []),
            "orc_set_threads": (None, [C.c_int]),
            "orc_hash_params": (None, [P, P, U32, P]),
            "orc_hash": (None, [P, U32, P, P, U32, U32, U32, P]),
            "orc_raygen_primary": (None, [P, U32, U32, P, P]),
            "orc_camera_look_at": (I, [P, P, P, F, U32, U32, P]),
            "orc_raygen_shadow": (None, [P, P, U32, U32, P, U32, F, P, P, U32, U32, P, P]),
            "orc_raygen_shadow_samples": (None, [P, P, U32, U32, P, U32, U32, F, P, P, U32, U32, P, P]),
            "orc_shade": (None, [P, P, P, U32, P, P, U32, U32, P, U32, U32, P, U32, P]),
            "orc_pack": (None, [P, U32, P]),
            "orc_raygen_reflect": (None, [P, P, P, P, U32, U32, F, F, U32, U32, P, P, U32, U32, P, P]),
            "orc_raygen_refract": (None, [P, P, P, P, U32, U32, F, F, P, P, U32, U32, P, P]),
            "orc_compress": (None, [P, U32, P, P, P, P, P]),
            "orc_sort_pairs": (None, [P, P, U32, U32, P, P]),
            "orc_decompress": (None, [P, P, P, P, U32, U32, P, P]),
            "orc_hierarchy_offsets": (U32, [U32, U32, P]),
            "orc_build_rsh": (None, [P, P, U32, U32, U32, P]),
            "orc_objh_build": (P, [P, U32, U32, P, P]),
            "orc_transform": (None, [P, P, P, U32, U32, P, P, P, P]),
            "orc_objh_free": (None, [P]),
            "orc_objh_levels": (U32, [P]),
            "orc_objh_level_size": (U32, [P, U32]),
            "orc_objh_get": (None, [P, P, P, P]),
            "orc_objh_kid_count": (U32, [P]),
            "orc_objh_kids": (None, [P, P]),
            "orc_traverse": (U64, [P, P, U32, U32, U32, P, U64, P]),
            "orc_intersect": (None, [P, P, P, U32, U32, P, U64, I, P, P]),
            "orc_brute": (None, [P, U32, P, U32, I, P, P]),
            "orc_trace_rays_box": (I, [P, P, U32, I, P, P, P, P]),
            "orc_objh_boxes": (None, [P, P]),
            "orc_objh_box_tree": (U32, [P, P, P, P]),
            "orc_brute_scalar": (None, [P, U32, P, U32, I, P, P]),
            "orc_brute_second": (None, [P, U32, P, U32, P, P]),
            "orc_resolve": (None, [P, P, P, P, P, P, U32, P, P]),
            "orc_trace_keyed": (U32, [P, P, P, U32, U32, U32, I, P, P, P, P, U32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(a):
    # a ctypes pointer that keeps the array alive for the call (the array may be a temporary conversion)
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _u32(a):
    return np.ascontiguousarray(a, np.uint32)


def threads() -> int:
    return lib().orc_num_threads()


def hash_scale(lo, hi, grid_bits: int) -> np.ndarray:
    out = np.zeros(3, np.float32)
    lib().orc_hash_params(_p(_f32(lo)), _p(_f32(hi)), grid_bits, _p(out))
    return out


def hash_rays(rays, lo, scale, g, b, tag=0):
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    keys = np.empty(len(rays), np.uint32)
    lib().orc_hash(_p(rays), len(rays), _p(_f32(lo)), _p(_f32(scale)), g, b, tag, _p(keys))
    return keys


def camera_look_at(eye, target, up, fov_degrees, W, H) -> np.ndarray:
    """Camera::loadView's basis as 12 floats (eye, direction, right, up), the layout of rsh_camera."""
    cam = np.zeros(12, np.float32)
    e, t, u = _f32(eye), _f32(target), _f32(up)
    ok = lib().orc_camera_look_at(_p(e), _p(t), _p(u), float(fov_degrees), W, H, _p(cam))
    if not ok:
        raise ValueError("degenerate camera")
    return cam


def raygen_primary(cam: np.ndarray, W: int, H: int):
    n = ((W + 7) // 8) * ((H + 7) // 8) * 64
    rays = np.zeros(n, RAY_DTYPE)
    pix = np.zeros(n, np.uint32)
    lib().orc_raygen_primary(_p(_f32(cam)), W, H, _p(rays), _p(pix))
    return rays, pix


def raygen_shadow(spos, snrm, W, H, light_pos, eps, lo, scale, g, b, samples=1):
    """Shadow rays; samples = 16: the soft-shadow grid around each light (slot x + W (l*16 + s + L*16 y))."""
    light_pos = _f32(np.asarray(light_pos).reshape(-1, 3))
    L = light_pos.shape[0]
    n = W * H * L * samples
    rays = np.zeros(n, RAY_DTYPE)
    keys = np.empty(n, np.uint32)
    sp, sn, lo_, sc_ = _f32(spos), _f32(snrm), _f32(lo), _f32(scale)
    lib().orc_raygen_shadow_samples(_p(sp), _p(sn), W, H, _p(light_pos), L, samples, float(eps), _p(lo_), _p(sc_),
                                    g, b, _p(rays), _p(keys))
    return rays, keys


def shade(spos, snrm, materials, shadow, accum, W, H, lights, eye, bounce, incident=None, samples=1):
    """One surface buffer of Blinn-Phong shading into accum (W*H x 4 float32, updated in place).
    lights: list of dicts {position, color, diffuse, specular}; materials: (M, 8) float32."""
    lt = _f32(np.array([[*l["position"], *l.get("color", (1.0, 1.0, 1.0)), l.get("diffuse", 1.0),
                         l.get("specular", 1.0)] for l in lights], np.float32))
    mats = _f32(np.asarray(materials, np.float32).reshape(-1, 8))
    inc = None if incident is None else np.ascontiguousarray(incident, RAY_DTYPE)
    sp, sn, e3 = _f32(spos), _f32(snrm), _f32(np.asarray(eye, np.float32).reshape(3))
    sh = None if shadow is None else _u32(shadow)
    assert accum.dtype == np.float32 and accum.flags.c_contiguous
    lib().orc_shade(_p(sp), _p(sn), _p(mats), mats.shape[0], _p(sh), _p(accum), W, H, _p(lt), len(lights), samples,
                    _p(e3), bounce, _p(inc))


def pack(accum):
    n = accum.shape[0]
    out = np.empty(n, np.uint32)
    lib().orc_pack(_p(accum), n, _p(out))
    return out


def raygen_reflect(spos, snrm, prev, eye, W, H, eps, jitter, seed, bounce, lo, scale, g, b):
    rays = np.zeros(W * H, RAY_DTYPE)
    keys = np.empty(W * H, np.uint32)
    prev = None if prev is None else np.ascontiguousarray(prev, RAY_DTYPE)
    lib().orc_raygen_reflect(_p(_f32(spos)), _p(_f32(snrm)), _p(prev), _p(_f32(eye)), W, H, float(eps), float(jitter),
                             seed, bounce, _p(_f32(lo)), _p(_f32(scale)), g, b, _p(rays), _p(keys))
    return rays, keys


def raygen_refract(spos, snrm, prev, eye, W, H, eps, eta, lo, scale, g, b):
    rays = np.zeros(W * H, RAY_DTYPE)
    keys = np.empty(W * H, np.uint32)
    prev = None if prev is None else np.ascontiguousarray(prev, RAY_DTYPE)
    sp, sn, lo_, sc_ = _f32(spos), _f32(snrm), _f32(lo), _f32(scale)
    e3 = None if eye is None else _f32(np.asarray(eye, np.float32).reshape(3))
    lib().orc_raygen_refract(_p(sp), _p(sn), _p(prev), _p(e3), W, H, float(eps), float(eta), _p(lo_), _p(sc_), g, b,
                             _p(rays), _p(keys))
    return rays, keys


def compress(keys):
    keys = _u32(keys)
    n = len(keys)
    trimmed = np.zeros(max(n, 1), np.uint32)
    ck = np.zeros(n + 1, np.uint32)
    cb = np.zeros(n + 1, np.uint32)
    cs = np.zeros(n + 1, np.uint32)
    counts = np.zeros(2, np.uint32)
    lib().orc_compress(_p(keys), n, _p(trimmed), _p(ck), _p(cb), _p(cs), _p(counts))
    R, Cc = int(counts[0]), int(counts[1])
    return trimmed[:R], ck[:Cc], cb[:Cc + 1], cs[:Cc]


def sort_pairs(keys, vals, key_bits):
    keys = _u32(keys)
    n = len(keys)
    ko = np.empty(n, np.uint32)
    vo = np.empty(n, np.uint32)
    lib().orc_sort_pairs(_p(keys), _p(None if vals is None else _u32(vals)), n, key_bits, _p(ko), _p(vo))
    return ko, vo


def decompress(skeys, svals, cbases, trimmed):
    R = len(trimmed)
    Cc = len(svals)
    sk = np.empty(R, np.uint32)
    si = np.empty(R, np.uint32)
    lib().orc_decompress(_p(_u32(skeys)), _p(_u32(svals)), _p(_u32(cbases)), _p(_u32(trimmed)), R, Cc, _p(sk), _p(si))
    return sk, si


def build_rsh(rays, ids, n, P, max_rays=None):
    max_rays = n if max_rays is None else max_rays
    off = np.zeros(4, np.uint32)
    cap = lib().orc_hierarchy_offsets(max_rays, P, _p(off))
    nodes = np.zeros(max(cap, 1), NODE_DTYPE)
    lib().orc_build_rsh(_p(np.ascontiguousarray(rays, RAY_DTYPE)), _p(None if ids is None else _u32(ids)), n,
                        max_rays, P, _p(nodes))
    return nodes, off


def transform(positions, normals, object_ids, model, normal=None):
    """UpdateVertex restated: positions / normals [T,3,4] moved by per-object row-major 4x4 matrices."""
    pr = _f32(positions).reshape(-1, 3, 4)
    nr = _f32(normals).reshape(-1, 3, 4)
    T = pr.shape[0]
    ob = _u32(object_ids)
    md = _f32(np.asarray(model, np.float32).reshape(-1, 16))
    nm = None if normal is None else _f32(np.asarray(normal, np.float32).reshape(-1, 16))
    pos = np.empty_like(pr)
    nrm = np.empty_like(nr)
    lib().orc_transform(_p(pr), _p(nr), _p(ob), T, md.shape[0], _p(md), _p(nm), _p(pos), _p(nrm))
    return pos, nrm


class ObjH:
    def __init__(self, positions, cluster, lo, hi):
        self.positions = _f32(positions).reshape(-1, 12)
        self.T = self.positions.shape[0]
        self.h = lib().orc_objh_build(_p(self.positions), self.T, cluster, _p(_f32(lo)), _p(_f32(hi)))
        self.cluster = cluster

    def levels(self):
        return [lib().orc_objh_level_size(self.h, l) for l in range(lib().orc_objh_levels(self.h))]

    def arrays(self):
        total = sum(self.levels())
        order = np.empty(self.T, np.uint32)
        tris = np.empty((self.T, 12), np.float32)
        sph = np.empty((max(total, 1), 4), np.float32)
        lib().orc_objh_get(self.h, _p(order), _p(tris), _p(sph))
        return order, tris, sph[:total]

    def kids(self) -> list[np.ndarray]:
        """Per level: child-range starts (size + 1 entries; level 0: the clusters' triangle ranges)."""
        flat = np.empty(max(lib().orc_objh_kid_count(self.h), 1), np.uint32)
        lib().orc_objh_kids(self.h, _p(flat))
        out, o = [], 0
        for n in self.levels():
            out.append(flat[o:o + n + 1].copy())
            o += n + 1
        return out

    def traverse(self, nodes, n, P, max_rays=None, cap=1 << 28):
        max_rays = n if max_rays is None else max_rays
        tests = np.zeros(1, np.uint64)
        cnt = lib().orc_traverse(self.h, _p(nodes), n, max_rays, P, None, 0, _p(tests))
        cand = np.empty(max(int(cnt), 1), np.uint64)
        lib().orc_traverse(self.h, _p(nodes), n, max_rays, P, _p(cand), cnt, None)
        return cand[:cnt], int(tests[0])

    def intersect(self, rays, ids, n, P, cand, any_hit, n_slots):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        flags = np.zeros(n_slots, np.uint32)
        hits = np.full(n_slots, HIT_NONE, np.uint64)
        cand = np.ascontiguousarray(cand, np.uint64)
        lib().orc_intersect(self.h, _p(rays), _p(None if ids is None else _u32(ids)), n, P, _p(cand), len(cand),
                            int(any_hit), _p(flags), _p(hits))
        return flags if any_hit else hits

    def trace_keyed(self, rays, keys, key_bits, P, any_hit, ray_level=4):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        keys = _u32(keys)
        n = len(keys)
        flags = np.zeros(n, np.uint32)
        hits = np.full(n, HIT_NONE, np.uint64)
        ms = np.zeros(8, np.float32)
        ctr = np.zeros(2, np.uint64)
        R = lib().orc_trace_keyed(self.h, _p(rays), _p(keys), n, key_bits, P, int(any_hit), _p(flags), _p(hits),
                                  _p(ms), _p(ctr), ray_level)
        return (flags if any_hit else hits), int(R), ms, ctr

    def boxes(self) -> np.ndarray:
        """Per node (levels concatenated): padded box lo xyz, link, hi xyz, count; link and count as u32 bits."""
        out = np.empty((max(sum(self.levels()), 1), 8), np.float32)
        lib().orc_objh_boxes(self.h, _p(out))
        return out[: sum(self.levels())]

    def box_tree(self):
        """The single-ray box tree: (root entry, boxes [slots, 8] float32 with u32 words in columns 3 and 7,
        triangles [T, 12] in its depth-first order)."""
        root = np.zeros(1, np.uint32)
        n = lib().orc_objh_box_tree(self.h, _p(root), None, None)
        boxes = np.empty((max(n, 1), 8), np.float32)
        tris = np.empty((max(self.T, 1), 12), np.float32)
        lib().orc_objh_box_tree(self.h, None, _p(boxes), _p(tris))
        return int(root[0]), boxes[:n], tris[: self.T]

    def trace_box(self, rays, any_hit, per_ray=False):
        """Per-ray descent of the single-ray box tree (the batched form's rays-only traversal): flags or hits, the
        (node tests, triangle tests) totals and, with per_ray, the counts of every ray ([n, 2] u32)."""
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(rays)
        flags = np.zeros(n, np.uint32)
        hits = np.full(n, HIT_NONE, np.uint64)
        pr = np.zeros((n, 2), np.uint32) if per_ray else None
        ctr = np.zeros(2, np.uint64)
        ok = lib().orc_trace_rays_box(self.h, _p(rays), n, int(any_hit), _p(flags), _p(hits), _p(pr), _p(ctr))
        if not ok:
            raise OverflowError("job stack overflow")
        out = flags if any_hit else hits
        return (out, (int(ctr[0]), int(ctr[1])), pr) if per_ray else (out, (int(ctr[0]), int(ctr[1])))

    def __del__(self):
        try:
            lib().orc_objh_free(self.h)
        except Exception:
            pass


def brute(positions, rays, any_hit, scalar=False):
    """Every ray against every triangle: shadow flags (any_hit) or closest-hit records. scalar=True runs the
    plain one-triangle-at-a-time loop (same results, slower)."""
    pos = _f32(positions).reshape(-1, 12)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(rays)
    flags = np.zeros(n, np.uint32)
    hits = np.full(n, HIT_NONE, np.uint64)
    fn = lib().orc_brute_scalar if scalar else lib().orc_brute
    fn(_p(pos), pos.shape[0], _p(rays), n, int(any_hit), _p(flags), _p(hits))
    return flags if any_hit else hits


def brute_two_nearest(positions, rays):
    pos = _f32(positions).reshape(-1, 12)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(rays)
    t1 = np.empty(n, np.float32)
    t2 = np.empty(n, np.float32)
    lib().orc_brute_second(_p(pos), pos.shape[0], _p(rays), n, _p(t1), _p(t2))
    return t1, t2


def resolve(positions, normals, mat, rays, hits, pix, npix):
    spos = np.zeros((npix, 4), np.float32)
    snrm = np.zeros((npix, 4), np.float32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    lib().orc_resolve(_p(_f32(positions)), _p(_f32(normals)), _p(None if mat is None else _u32(mat)), _p(rays),
                      _p(np.ascontiguousarray(hits, np.uint64)), _p(None if pix is None else _u32(pix)), len(rays),
                      _p(spos), _p(snrm))
    return spos, snrm
