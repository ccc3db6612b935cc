"""Python mirror of the rsh C ABI (include/rsh.h) over ctypes.

The engine interface mirrors the reference's CUDA-Engine host side: a scene of triangle soups with
materials (main.cpp:2374-2470), point lights (main.cpp:2596-2656), an orbit/pinhole camera
(Camera.cpp:91-133), and per-stage wrappers for the secondary-ray pipeline (RayTracer.cu:2042-3301).
All compute runs in `librsh.so` (hand-written sm_103a kernels); importing this module without the built
library raises immediately — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "librsh.so"

RSH_OK, RSH_ERR_OOM, RSH_ERR_OVERFLOW, RSH_ERR_TIMEOUT, RSH_ERR_INVALID, RSH_ERR_CUDA = range(6)
STATUS_NAMES = {0: "RSH_OK", 1: "RSH_ERR_OOM", 2: "RSH_ERR_OVERFLOW", 3: "RSH_ERR_TIMEOUT",
                4: "RSH_ERR_INVALID", 5: "RSH_ERR_CUDA"}
KEY_NONE = 0xFFFFFFFF
HIT_NONE = 0xFFFFFFFFFFFFFFFF
OCCLUDED = 0xFFFFFFFF
FLAG_STAGE_TIMERS = 1
FLAG_FUSED = 2
FLAG_RAH = 4
FLAG_SOFT_SHADOWS = 8
FLAG_NO_COMPRESS = 16
FLAG_SEQUENTIAL_RAYS = 32

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
NODE_DTYPE = np.dtype([("c", "<f4", 3), ("radius", "<f4"), ("axis", "<f4", 3), ("cos_spread", "<f4"),
                       ("sin_spread", "<f4"), ("reach", "<f4"), ("first", "<u4"), ("count", "<u4")])
OBJNODE_DTYPE = np.dtype([("c", "<f4", 3), ("radius", "<f4"), ("first_tri", "<u4"), ("tri_count", "<u4"),
                          ("first_child", "<u4"), ("child_count", "<u4")])


class RshError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str = ""):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {msg}".strip())
        self.status = status


# ---------------------------------------------------------------- ctypes structures
class Config(C.Structure):
    _fields_ = [("grid_bits", C.c_uint32), ("dir_log2", C.c_uint32), ("packet_size", C.c_uint32),
                ("cluster_size", C.c_uint32), ("epsilon", C.c_float), ("hbm_budget", C.c_uint64),
                ("candidate_capacity", C.c_uint64), ("flags", C.c_uint32), ("reflect_jitter", C.c_float),
                ("seed", C.c_uint32), ("ray_level", C.c_uint32), ("plain_ray_level", C.c_uint32),
                ("fused_blocks", C.c_uint32)]


class HashParams(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("scale", C.c_float * 3), ("grid_bits", C.c_uint32),
                ("dir_log2", C.c_uint32), ("tag_bits", C.c_uint32), ("key_bits", C.c_uint32)]


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("color", C.c_float * 3), ("diffuse_intensity", C.c_float),
                ("specular_intensity", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("direction", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3)]

    def as_array(self) -> np.ndarray:
        return np.array([*self.eye, *self.direction, *self.right, *self.up], dtype=np.float32)


class Material(C.Structure):
    _fields_ = [("diffuse", C.c_float * 4), ("specular", C.c_float * 4)]


class SceneDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("material_ids", C.c_void_p),
                ("object_ids", C.c_void_p), ("materials", C.c_void_p), ("triangle_count", C.c_uint32),
                ("material_count", C.c_uint32)]


class ObjData(C.Structure):
    _fields_ = [("desc", SceneDesc), ("object_count", C.c_uint32), ("owner", C.c_void_p)]


class FrameStats(C.Structure):
    _fields_ = [("primary_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("reflection_rays", C.c_uint64),
                ("chunks", C.c_uint64), ("candidates", C.c_uint64), ("node_tests", C.c_uint64),
                ("tri_tests", C.c_uint64), ("secondary_ms", C.c_float), ("frame_ms", C.c_float),
                ("stage_ms", C.c_float * 12), ("overflow_passes", C.c_uint32)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "stage_ms"}
        d["stage_ms"] = list(self.stage_ms)
        return d


class BatchSegment(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("rays", C.c_void_p), ("n", C.c_uint32), ("any_hit", C.c_int),
                ("hits", C.c_void_p), ("flags", C.c_void_p)]


TUNE_DEFAULT = 0xFFFFFFFF


class SceneTuning(C.Structure):
    _fields_ = [("grid_bits", C.c_uint32), ("dir_log2", C.c_uint32), ("ray_level", C.c_uint32)]


class TuneSpace(C.Structure):
    _fields_ = [("grid_bits", C.c_void_p), ("n_grid", C.c_uint32), ("dir_log2", C.c_void_p), ("n_dir", C.c_uint32),
                ("ray_levels", C.c_void_p), ("n_ray_level", C.c_uint32), ("packet_sizes", C.c_void_p),
                ("n_packet", C.c_uint32), ("reps", C.c_uint32), ("fused_blocks", C.c_void_p),
                ("n_fused_blocks", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene_index", C.c_uint32), ("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("depth", C.c_uint32), ("light_count", C.c_uint32), ("lights", Light * 8)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("submit_ms", C.c_double), ("start_ms", C.c_double),
                ("finish_ms", C.c_double), ("rays", C.c_uint64)]


# ---------------------------------------------------------------- library loading
_lib = None

# name -> (restype, argtypes); every entry point declared in include/rsh.h
_P = C.c_void_p
_U32 = C.c_uint32
_U64 = C.c_uint64
_I32 = C.c_int32
_F = C.c_float
SIGNATURES = {
    "rsh_config_default": (None, [_P]),
    "rsh_create": (C.c_int, [_P, _P]),
    "rsh_destroy": (C.c_int, [_P]),
    "rsh_get_config": (C.c_int, [_P, _P]),
    "rsh_set_config": (C.c_int, [_P, _P]),
    "rsh_last_error_string": (C.c_char_p, []),
    "rsh_check_device_errors": (C.c_int, [_P, _P]),
    "rsh_selftest_wait_timeout": (C.c_int, [_P, _U32, _P]),
    "rsh_bytes_allocated": (_U64, [_P]),
    "rsh_malloc": (C.c_int, [_P, C.c_size_t]),
    "rsh_free": (C.c_int, [_P]),
    "rsh_malloc_host": (C.c_int, [_P, C.c_size_t]),
    "rsh_free_host": (C.c_int, [_P]),
    "rsh_memcpy_h2d": (C.c_int, [_P, _P, C.c_size_t, _P]),
    "rsh_memcpy_d2h": (C.c_int, [_P, _P, C.c_size_t, _P]),
    "rsh_memset": (C.c_int, [_P, C.c_int, C.c_size_t, _P]),
    "rsh_stream_create": (C.c_int, [_P]),
    "rsh_stream_destroy": (C.c_int, [_P]),
    "rsh_stream_synchronize": (C.c_int, [_P]),
    "rsh_device_synchronize": (C.c_int, []),
    "rsh_event_create": (C.c_int, [_P]),
    "rsh_event_destroy": (C.c_int, [_P]),
    "rsh_event_record": (C.c_int, [_P, _P]),
    "rsh_event_elapsed": (C.c_int, [_P, _P, _P]),
    "rsh_device_count": (C.c_int, []),
    "rsh_sm_count": (C.c_int, []),
    "rsh_test_counters": (C.c_int, [_P, _P, _P, _I32, _P]),
    "rsh_device_memory": (C.c_int, [_P, _P]),
    "rsh_kernel_launches": (_U64, []),
    "rsh_scene_upload": (C.c_int, [_P, _P, _P]),
    "rsh_scene_set_transforms": (C.c_int, [_P, _P, _P, _P, _U32, _P]),
    "rsh_build_object_hierarchy": (C.c_int, [_P, _P, _P]),
    "rsh_obj_load": (C.c_int, [C.c_char_p, _P]),
    "rsh_obj_free": (None, [_P]),
    "rsh_scene_destroy": (C.c_int, [_P, _P]),
    "rsh_scene_bounds": (C.c_int, [_P, _P, _P]),
    "rsh_scene_triangle_count": (_U32, [_P]),
    "rsh_scene_levels": (_U32, [_P]),
    "rsh_scene_box_tree": (_U32, [_P, _P, _P, _P]),
    "rsh_scene_level_size": (_U32, [_P, _U32]),
    "rsh_scene_get_level": (C.c_int, [_P, _U32, _P]),
    "rsh_scene_get_order": (C.c_int, [_P, _P]),
    "rsh_scene_device_triangles": (_P, [_P]),
    "rsh_lights_set": (C.c_int, [_P, _P, _U32]),
    "rsh_camera_set": (C.c_int, [_P, _P]),
    "rsh_camera_look_at": (C.c_int, [_P, _P, _P, _F, _U32, _U32, _P]),
    "rsh_render_frame": (C.c_int, [_P, _P, _U32, _U32, _U32, _P, _P]),
    "rsh_frame_stats_get": (C.c_int, [_P, _P]),
    "rsh_frame_hits": (C.c_int, [_P, _I32, _P]),
    "rsh_frame_shadow": (C.c_int, [_P, _I32, _P]),
    "rsh_frame_rays": (C.c_int, [_P, _I32, _I32, _P]),
    "rsh_frame_surface": (C.c_int, [_P, _I32, _P, _P]),
    "rsh_write_png": (C.c_int, [C.c_char_p, _P, _U32, _U32]),
    "rsh_hash_params_make": (C.c_int, [_P, _P, _U32, _U32, _U32, _P]),
    "rsh_raygen_primary": (C.c_int, [_P, _U32, _U32, _P, _P, _P]),
    "rsh_raygen_shadow": (C.c_int, [_P, _P, _U32, _U32, _P, _U32, _F, _P, _P, _P, _P]),
    "rsh_raygen_soft_shadow": (C.c_int, [_P, _P, _U32, _U32, _P, _U32, _F, _P, _P, _P, _P]),
    "rsh_raygen_refract": (C.c_int, [_P, _P, _P, _P, _U32, _U32, _F, _F, _P, _P, _P, _P]),
    "rsh_raygen_reflect": (C.c_int, [_P, _P, _P, _P, _U32, _U32, _F, _F, _U32, _U32, _P, _P, _P, _P]),
    "rsh_hash": (C.c_int, [_P, _U32, _P, _U32, _P, _P]),
    "rsh_compress": (C.c_int, [_P, _P, _U32, _P, _P, _P, _P, _P, _P]),
    "rsh_compress_noalloc": (C.c_int, [_P, _U32, _P, _P, _P, _P, _P, _P]),
    "rsh_sort_pairs": (C.c_int, [_P, _P, _P, _P, _P, _U32, _P, _U32, _P]),
    "rsh_decompress": (C.c_int, [_P, _P, _P, _P, _P, _P, _U32, _P, _P, _P]),
    "rsh_hierarchy_capacity": (_U32, [_U32, _U32, _P]),
    "rsh_build_rsh": (C.c_int, [_P, _P, _U32, _P, _U32, _P, _P]),
    "rsh_traverse": (C.c_int, [_P, _P, _P, _U32, _P, _U32, _P, _U64, _P, _P]),
    "rsh_intersect_any": (C.c_int, [_P, _P, _P, _U32, _P, _U32, _P, _P, _P, _P]),
    "rsh_intersect_closest": (C.c_int, [_P, _P, _P, _U32, _P, _U32, _P, _P, _P, _P]),
    "rsh_resolve_hits": (C.c_int, [_P, _P, _P, _P, _U32, _P, _P, _P]),
    "rsh_trace_rays": (C.c_int, [_P, _P, _P, _U32, C.c_int, _P, _P, _P]),
    "rsh_batch_trace": (C.c_int, [_P, _P, _U32, _P]),
    "rsh_batch_graph_create": (C.c_int, [_P, _P, _U32, _P, _P]),
    "rsh_batch_graph_launch": (C.c_int, [_P, _P]),
    "rsh_batch_graph_destroy": (C.c_int, [_P]),
    "rsh_batch_stats_get": (C.c_int, [_P, _P]),
    "rsh_autotune": (C.c_int, [_P, _P, _U32, _P, _U32, _P, _U32, _P, _U32, _P, _P]),
    "rsh_trace_rays_fused": (C.c_int, [_P, _P, _P, _U32, C.c_int, _P, _P, _P]),
    "rsh_scene_set_tuning": (C.c_int, [_P, _P]),
    "rsh_scene_get_tuning": (C.c_int, [_P, _P]),
    "rsh_autotune_scenes": (C.c_int, [_P, _P, _U32, _P, _P, _P, _P]),
    "rsh_server_create": (C.c_int, [_P, _P, _U32, _U64, _U32, _P]),
    "rsh_server_submit": (C.c_int, [_P, _P, _P]),
    "rsh_server_request_bytes": (C.c_int, [_P, _P]),
    "rsh_server_wait": (C.c_int, [_P, _U64, _U32, _P, _P, _P]),
    "rsh_server_cancel": (C.c_int, [_P, _U64]),
    "rsh_server_set_step_rays": (C.c_int, [_P, _U64]),
    "rsh_server_stats": (C.c_int, [_P, _P, _P, _P, _P]),
    "rsh_server_destroy": (C.c_int, [_P]),
}


def load(path: str | os.PathLike | None = None):
    """Loads librsh.so (built by `rsh._build.build()`); raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def lib():
    return load()


def last_error() -> str:
    s = lib().rsh_last_error_string()
    return s.decode() if s else ""


def check(status: int, where: str):
    if status != RSH_OK:
        raise RshError(status, where, last_error())


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, DeviceArray):
        return a.ptr
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if isinstance(a, int):
        return a
    return C.addressof(a)


# ---------------------------------------------------------------- device memory
class DeviceArray:
    """A device allocation with a numpy dtype and shape (plumbing for tests and the bench)."""

    def __init__(self, shape, dtype, zero: bool = False):
        self.dtype = np.dtype(dtype)
        self.shape = tuple(np.atleast_1d(np.asarray(shape, dtype=np.int64)).tolist()) if not isinstance(shape, int) else (shape,)
        self.nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        p = C.c_void_p()
        check(lib().rsh_malloc(C.byref(p), max(self.nbytes, 16)), "rsh_malloc")
        self.ptr = p.value
        if zero:
            self.fill_bytes(0)

    @classmethod
    def from_numpy(cls, a: np.ndarray, stream=None) -> "DeviceArray":
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype)
        d.upload(a, stream)
        return d

    def upload(self, a: np.ndarray, stream=None):
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        check(lib().rsh_memcpy_h2d(self.ptr, a.ctypes.data, a.nbytes, stream), "rsh_memcpy_h2d")
        if stream is None:
            check(lib().rsh_stream_synchronize(None), "sync")

    def numpy(self, count: int | None = None, stream=None) -> np.ndarray:
        n = int(np.prod(self.shape)) if count is None else count
        out = np.empty(n, dtype=self.dtype)
        if n:
            check(lib().rsh_memcpy_d2h(out.ctypes.data, self.ptr, out.nbytes, stream), "rsh_memcpy_d2h")
        check(lib().rsh_stream_synchronize(stream), "sync")
        if count is None:
            out = out.reshape(self.shape)
        return out

    def fill_bytes(self, value: int, stream=None):
        check(lib().rsh_memset(self.ptr, value, self.nbytes, stream), "rsh_memset")

    def free(self):
        if getattr(self, "ptr", None):
            lib().rsh_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def default_config(**kw) -> Config:
    c = Config()
    lib().rsh_config_default(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def hash_params(lo, hi, grid_bits: int, dir_log2: int, tag_bits: int = 0) -> HashParams:
    hp = HashParams()
    lo_a = (C.c_float * 3)(*map(float, lo))
    hi_a = (C.c_float * 3)(*map(float, hi))
    check(lib().rsh_hash_params_make(lo_a, hi_a, grid_bits, dir_log2, tag_bits, C.byref(hp)), "rsh_hash_params_make")
    return hp


def camera_look_at(eye, target, up, fov_degrees: float, width: int, height: int) -> Camera:
    cam = Camera()
    e = (C.c_float * 3)(*map(float, eye))
    t = (C.c_float * 3)(*map(float, target))
    u = (C.c_float * 3)(*map(float, up))
    check(lib().rsh_camera_look_at(e, t, u, float(fov_degrees), width, height, C.byref(cam)), "rsh_camera_look_at")
    return cam


def make_lights(lights) -> "C.Array":
    arr = (Light * max(1, len(lights)))()
    for i, l in enumerate(lights):
        arr[i].position[:] = list(map(float, l["position"]))
        arr[i].color[:] = list(map(float, l.get("color", (1.0, 1.0, 1.0))))
        arr[i].diffuse_intensity = float(l.get("diffuse", 1.0))
        arr[i].specular_intensity = float(l.get("specular", 1.0))
    return arr


def load_obj(path) -> dict:
    """Reads an OBJ (+ MTL) file through rsh_obj_load; returns numpy copies of the scene arrays:
    positions / normals float32 [T,3,4], material_ids / object_ids uint32 [T], materials float32 [M,8]."""
    ptr = C.POINTER(ObjData)()
    check(lib().rsh_obj_load(str(path).encode(), C.byref(ptr)), "rsh_obj_load")
    try:
        d = ptr.contents.desc
        T, M = d.triangle_count, d.material_count

        def arr(addr, n, dt, shape):
            if n == 0:
                return np.zeros(shape, dt)
            return np.ctypeslib.as_array(C.cast(addr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                         (n,)).reshape(shape).copy()
        out = {"positions": arr(d.positions, 12 * T, np.float32, (T, 3, 4)),
               "normals": arr(d.normals, 12 * T, np.float32, (T, 3, 4)),
               "material_ids": arr(d.material_ids, T, np.uint32, (T,)),
               "object_ids": arr(d.object_ids, T, np.uint32, (T,)),
               "materials": arr(d.materials, 8 * M, np.float32, (M, 8)),
               "object_count": ptr.contents.object_count}
    finally:
        lib().rsh_obj_free(ptr)
    return out


class Scene:
    """A device-resident scene (positions/normals float32 [T,3,4]; material ids uint32 [T])."""

    def __init__(self, ctx: "Context", positions: np.ndarray, normals=None, material_ids=None, materials=None,
                 object_ids=None):
        self.ctx = ctx
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3, 4)
        self.positions = pos
        self.normals = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3, 4)
        self.material_ids = None if material_ids is None else np.ascontiguousarray(material_ids, dtype=np.uint32)
        mats = materials if materials is not None else np.array([[0.8, 0.8, 0.8, 0.5, 0.5, 0.5, 0.5, 32.0]], np.float32)
        self.materials = np.ascontiguousarray(mats, dtype=np.float32).reshape(-1, 8)
        d = SceneDesc()
        d.positions = pos.ctypes.data
        d.normals = self.normals.ctypes.data if self.normals is not None else None
        d.material_ids = self.material_ids.ctypes.data if self.material_ids is not None else None
        self.object_ids = None if object_ids is None else np.ascontiguousarray(object_ids, dtype=np.uint32)
        d.object_ids = self.object_ids.ctypes.data if self.object_ids is not None else None
        d.materials = self.materials.ctypes.data
        d.triangle_count = pos.shape[0]
        d.material_count = self.materials.shape[0]
        h = C.c_void_p()
        check(lib().rsh_scene_upload(ctx.handle, C.byref(d), C.byref(h)), "rsh_scene_upload")
        self.handle = h.value
        self.tri_count = pos.shape[0]

    def bounds(self):
        lo = (C.c_float * 3)()
        hi = (C.c_float * 3)()
        check(lib().rsh_scene_bounds(self.handle, lo, hi), "rsh_scene_bounds")
        return np.array(lo[:], np.float32), np.array(hi[:], np.float32)

    def levels(self) -> list[np.ndarray]:
        out = []
        for l in range(lib().rsh_scene_levels(self.handle)):
            n = lib().rsh_scene_level_size(self.handle, l)
            a = np.empty(n, OBJNODE_DTYPE)
            check(lib().rsh_scene_get_level(self.handle, l, a.ctypes.data), "rsh_scene_get_level")
            out.append(a)
        return out

    def set_transforms(self, model, normal=None, stream=None):
        """Per-object row-major 4x4 model (and normal) matrices, [K,16] or [K,4,4]; see rsh_scene_set_transforms."""
        m = np.ascontiguousarray(np.asarray(model, np.float32).reshape(-1, 16))
        n = None if normal is None else np.ascontiguousarray(np.asarray(normal, np.float32).reshape(-1, 16))
        check(lib().rsh_scene_set_transforms(self.ctx.handle, self.handle, m.ctypes.data,
                                             None if n is None else n.ctypes.data, m.shape[0], stream),
              "rsh_scene_set_transforms")

    def set_tuning(self, grid_bits=TUNE_DEFAULT, dir_log2=TUNE_DEFAULT, ray_level=TUNE_DEFAULT):
        """This scene's own hash width and switch level in the batched form (TUNE_DEFAULT: the context's)."""
        t = SceneTuning(grid_bits, dir_log2, ray_level)
        check(lib().rsh_scene_set_tuning(self.handle, C.byref(t)), "rsh_scene_set_tuning")

    def tuning(self) -> dict:
        t = SceneTuning()
        check(lib().rsh_scene_get_tuning(self.handle, C.byref(t)), "rsh_scene_get_tuning")
        return {"grid_bits": t.grid_bits, "dir_log2": t.dir_log2, "ray_level": t.ray_level}

    def triangles(self) -> np.ndarray:
        """The scene's current triangles in original order (float32 [T,3,4], w as uploaded)."""
        T = self.tri_count
        tris = np.empty((T, 3, 4), np.float32)
        check(lib().rsh_memcpy_d2h(tris.ctypes.data, lib().rsh_scene_device_triangles(self.handle), 48 * T, None),
              "d2h")
        out = np.empty_like(tris)
        out[self.order()] = tris
        out[:, 0, 3] = self.positions[:, 0, 3]  # cluster order keeps the original id in v0.w
        return out

    def box_tree(self):
        """The single-ray box tree: (root entry, slots [n, 8] float32 with u32 words in columns 3 and 7,
        triangles [T, 12] in its depth-first order)."""
        root = C.c_uint32()
        n = lib().rsh_scene_box_tree(self.handle, C.byref(root), None, None)
        boxes = np.empty((max(n, 1), 8), np.float32)
        T = lib().rsh_scene_triangle_count(self.handle)
        tris = np.empty((max(T, 1), 12), np.float32)
        lib().rsh_scene_box_tree(self.handle, None, boxes.ctypes.data, tris.ctypes.data)
        return root.value, boxes[:n], tris[:T]

    def order(self) -> np.ndarray:
        a = np.empty(self.tri_count, np.uint32)
        check(lib().rsh_scene_get_order(self.handle, a.ctypes.data), "rsh_scene_get_order")
        return a

    def destroy(self):
        if self.handle:
            lib().rsh_scene_destroy(self.ctx.handle, self.handle)
            self.handle = None


class Context:
    def __init__(self, config: Config | None = None, **kw):
        cfg = config or default_config(**kw)
        h = C.c_void_p()
        check(lib().rsh_create(C.byref(cfg), C.byref(h)), "rsh_create")
        self.handle = h.value
        self.config = cfg

    def set_config(self, **kw):
        for k, v in kw.items():
            setattr(self.config, k, v)
        check(lib().rsh_set_config(self.handle, C.byref(self.config)), "rsh_set_config")

    def autotune_scenes(self, segments, count: int, grid_bits=(), dir_log2=(), ray_levels=(), packet_sizes=(),
                        reps: int = 2, stream=None, fused_blocks=()) -> tuple:
        """rsh_autotune_scenes over a BatchSegment array; returns (tuned ms, untuned ms) of the whole batch.
        The chosen packet size and CTAs per SM land in this context, the rest in each scene (Scene.tuning())."""
        grid_bits, dir_log2, ray_levels = list(grid_bits), list(dir_log2), list(ray_levels)
        packet_sizes, fused_blocks = list(packet_sizes), list(fused_blocks)
        lists = [(C.c_uint32 * max(1, len(v)))(*v)
                 for v in (grid_bits, dir_log2, ray_levels, packet_sizes, fused_blocks)]
        sp = TuneSpace(C.cast(lists[0], C.c_void_p), len(grid_bits), C.cast(lists[1], C.c_void_p), len(dir_log2),
                       C.cast(lists[2], C.c_void_p), len(ray_levels), C.cast(lists[3], C.c_void_p),
                       len(packet_sizes), reps, C.cast(lists[4], C.c_void_p), len(fused_blocks))
        best, untuned = C.c_float(), C.c_float()
        check(lib().rsh_autotune_scenes(self.handle, segments, count, C.byref(sp), stream, C.byref(best),
                                        C.byref(untuned)), "rsh_autotune_scenes")
        check(lib().rsh_get_config(self.handle, C.byref(self.config)), "rsh_get_config")
        return best.value, untuned.value

    def scene(self, positions, normals=None, material_ids=None, materials=None, object_ids=None) -> Scene:
        return Scene(self, positions, normals, material_ids, materials, object_ids)

    def set_lights(self, lights):
        arr = make_lights(lights)
        check(lib().rsh_lights_set(self.handle, arr, len(lights)), "rsh_lights_set")

    def set_camera(self, cam: Camera):
        check(lib().rsh_camera_set(self.handle, C.byref(cam)), "rsh_camera_set")

    def render(self, scene: Scene, width: int, height: int, depth: int, rgba: DeviceArray | None = None, stream=None):
        check(lib().rsh_render_frame(self.handle, scene.handle, width, height, depth, _ptr(rgba), stream),
              "rsh_render_frame")

    def stats(self) -> dict:
        s = FrameStats()
        check(lib().rsh_frame_stats_get(self.handle, C.byref(s)), "rsh_frame_stats_get")
        return s.as_dict()

    def frame_hits(self, bounce: int, npix: int) -> np.ndarray:
        a = np.empty(npix, np.uint64)
        check(lib().rsh_frame_hits(self.handle, bounce, a.ctypes.data), "rsh_frame_hits")
        return a

    def frame_shadow(self, bounce: int, n: int) -> np.ndarray:
        a = np.empty(n, np.uint32)
        check(lib().rsh_frame_shadow(self.handle, bounce, a.ctypes.data), "rsh_frame_shadow")
        return a

    def frame_rays(self, bounce: int, shadow: bool, n: int) -> np.ndarray:
        a = np.empty(n, RAY_DTYPE)
        check(lib().rsh_frame_rays(self.handle, bounce, int(shadow), a.ctypes.data), "rsh_frame_rays")
        return a

    def frame_surface(self, bounce: int, npix: int):
        p = np.empty((npix, 4), np.float32)
        n = np.empty((npix, 4), np.float32)
        check(lib().rsh_frame_surface(self.handle, bounce, p.ctypes.data, n.ctypes.data), "rsh_frame_surface")
        return p, n

    def test_counters(self, reset: bool = True, stream=None):
        """(node tests, ray x triangle tests) accumulated since the last reset."""
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().rsh_test_counters(self.handle, C.byref(a), C.byref(b), int(reset), stream), "rsh_test_counters")
        return a.value, b.value

    def check_device_errors(self, stream=None):
        check(lib().rsh_check_device_errors(self.handle, stream), "device error word")

    def trace(self, scene: Scene, rays: np.ndarray, any_hit: bool, fused: bool = False) -> np.ndarray:
        """Traces host rays through the whole pipeline; returns hit records (closest) or flags (any)."""
        n = len(rays)
        d_rays = DeviceArray.from_numpy(np.ascontiguousarray(rays, RAY_DTYPE))
        if any_hit:
            out = DeviceArray(n, np.uint32)
            fn = lib().rsh_trace_rays_fused if fused else lib().rsh_trace_rays
            check(fn(self.handle, scene.handle, d_rays.ptr, n, 1, None, out.ptr, None), "trace")
        else:
            out = DeviceArray(n, np.uint64)
            fn = lib().rsh_trace_rays_fused if fused else lib().rsh_trace_rays
            check(fn(self.handle, scene.handle, d_rays.ptr, n, 0, out.ptr, None, None), "trace")
        return out.numpy()

    def destroy(self):
        if self.handle:
            lib().rsh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
