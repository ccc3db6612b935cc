"""Seeded synthetic scenes for the benchmark configurations (numpy; host-side input generation only).

The reference renders OBJ assets (office.obj, Cornell built from Cube.obj + sphere.obj, Sponza — the last
missing from the reference tree). These generators stand in with seeded scenes of the shapes, sizes and
value distributions of the five configurations:

  S  Cornell-style box: 10 axis-aligned quads + 2 icospheres (subdiv 3), 2,580 triangles, 512x512, 1 light
  O  object soup: 2000 jittered icospheres (subdiv 2) + 16 ground quads, 640,032 triangles, 1920x1080,
     2 lights, depth 3
  P  procedural architecture: 40x40 tessellated pillars + floor/ceiling slabs + arches (~1.0M triangles),
     1920x1080, 4 lights, depth 2, cosine-lobe perturbed reflections
  B  batching: random soups (10k..1M triangles) and ray batches on their surfaces
  Srv serving: request streams over resident scenes

Seeds: 0x5EED0000 + configuration index; one numpy Generator stream per generator stage.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SEED_BASE = 0x5EED0000
CONFIG_INDEX = {"S": 0, "O": 1, "P": 2, "B": 3, "Srv": 4}


@dataclass
class SceneData:
    name: str
    positions: np.ndarray          # [T,3,4] float32 (w = 1)
    normals: np.ndarray            # [T,3,4] float32 (w = 0)
    material_ids: np.ndarray       # [T] uint32
    materials: np.ndarray          # [M,8] float32: diffuse rgb + reflectance, specular rgb + shininess
    eye: tuple = (0.0, 0.0, 3.4)
    target: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    fov: float = 60.0
    width: int = 512
    height: int = 512
    depth: int = 1
    lights: list = field(default_factory=list)
    jitter: float = 0.0
    seed: int = SEED_BASE

    @property
    def tri_count(self) -> int:
        return int(self.positions.shape[0])


def _rng(cfg: str, stage: int) -> np.random.Generator:
    return np.random.default_rng([SEED_BASE + CONFIG_INDEX[cfg], stage])


def _pack(verts: np.ndarray, faces: np.ndarray, vnormals: np.ndarray | None = None):
    """verts [V,3], faces [F,3] -> positions/normals [F,3,4] float32."""
    tri = verts[faces].astype(np.float32)
    pos = np.concatenate([tri, np.ones((*tri.shape[:2], 1), np.float32)], axis=2)
    if vnormals is None:
        e1 = tri[:, 1] - tri[:, 0]
        e2 = tri[:, 2] - tri[:, 0]
        n = np.cross(e1, e2)
        n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
        nt = np.repeat(n[:, None, :], 3, axis=1)
    else:
        nt = vnormals[faces].astype(np.float32)
    nrm = np.concatenate([nt, np.zeros((*nt.shape[:2], 1), np.float32)], axis=2).astype(np.float32)
    return np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(nrm, np.float32)


def icosphere(subdiv: int):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[k] = len(verts) - 1
            return cache[k]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, np.int64)


def quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3)."""
    v = np.array([p0, p1, p2, p3], np.float64)
    return v, np.array([[0, 1, 2], [0, 2, 3]], np.int64)


def _materials(rng: np.random.Generator, m: int) -> np.ndarray:
    mats = np.zeros((m, 8), np.float32)
    mats[:, 0:3] = rng.uniform(0.2, 0.9, (m, 3))
    mats[:, 3] = rng.uniform(0.0, 1.0, m)          # reflectance U(0,1)
    mats[:, 4:7] = 0.5
    mats[:, 7] = 32.0
    return mats


# ---------------------------------------------------------------- S
def cornell() -> SceneData:
    rng = _rng("S", 2)
    parts = []
    # 5 walls of the [-1,1]^3 box, facing inwards
    walls = [
        quad((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)),   # floor (+y)
        quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1)),       # ceiling (-y)
        quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)),   # back (+z)
        quad((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)),   # left (+x)
        quad((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1)),       # right (-x)
    ]
    # a low block in the back-left corner: top + 4 sides
    x0, x1, z0, z1, y0, y1 = -0.9, -0.5, -0.9, -0.5, -1.0, -0.2
    block = [
        quad((x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)),
        quad((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)),
        quad((x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)),
        quad((x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)),
        quad((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)),
    ]
    pos_l, nrm_l, mid_l = [], [], []
    for i, (v, f) in enumerate(walls + block):
        p, n = _pack(v, f)
        pos_l.append(p)
        nrm_l.append(n)
        mid_l.append(np.full(len(f), min(i, 5), np.uint32))
    sv, sf = icosphere(3)
    for j, (c, r) in enumerate((((-0.4, -0.6, 0.2), 0.3), ((0.4, -0.6, -0.3), 0.3))):
        p, n = _pack(sv * r + np.array(c), sf, sv)
        pos_l.append(p)
        nrm_l.append(n)
        mid_l.append(np.full(len(sf), 6 + j, np.uint32))
    mats = _materials(rng, 8)
    light = {"position": (0.0, 0.95, 0.0), "color": (1, 1, 1), "diffuse": 1.0, "specular": 0.6}
    return SceneData("S", np.concatenate(pos_l), np.concatenate(nrm_l), np.concatenate(mid_l), mats,
                     eye=(0.0, 0.0, 3.4), target=(0, 0, 0), fov=60.0, width=512, height=512, depth=1,
                     lights=[light], seed=SEED_BASE + 0)


# ---------------------------------------------------------------- O
def soup(n_spheres: int = 2000, width: int = 1920, height: int = 1080, cfg: str = "O", seed_stage: int = 0,
         extent: float = 50.0, subdiv: int = 2) -> SceneData:
    rng = _rng(cfg, seed_stage)
    sv, sf = icosphere(subdiv)
    centers = rng.uniform(-extent, extent, (n_spheres, 3))
    radii = rng.lognormal(0.0, 0.5, n_spheres)
    V = sv.shape[0]
    jit = rng.normal(0.0, 0.05, (n_spheres, V, 3)) * radii[:, None, None]
    verts = sv[None] * radii[:, None, None] + jit + centers[:, None, :]
    tri = verts[:, sf]                                    # [N, F, 3, 3]
    tri = tri.reshape(-1, 3, 3)
    vn = (sv[None] * np.ones((n_spheres, 1, 1)))[:, sf].reshape(-1, 3, 3)
    ones = np.ones((*tri.shape[:2], 1))
    pos = np.concatenate([tri, ones], 2).astype(np.float32)
    nrm = np.concatenate([vn, np.zeros_like(ones)], 2).astype(np.float32)
    mids = np.repeat(np.arange(n_spheres) % 16, sf.shape[0]).astype(np.uint32)
    # 16 ground quads (4x4) below the soup
    g = []
    y = -extent - 5.0
    step = 2 * (extent + 50.0) / 4
    for i in range(4):
        for j in range(4):
            x0 = -(extent + 50.0) + i * step
            z0 = -(extent + 50.0) + j * step
            g.append(quad((x0, y, z0), (x0, y, z0 + step), (x0 + step, y, z0 + step), (x0 + step, y, z0)))
    gp, gn = zip(*[_pack(v, f) for v, f in g])
    pos = np.concatenate([pos, *gp])
    nrm = np.concatenate([nrm, *gn])
    mids = np.concatenate([mids, np.full(2 * len(g), 16, np.uint32)])
    mats = _materials(_rng(cfg, 2), 17)
    lights = [{"position": (0.0, extent + 30.0, 0.0), "diffuse": 1.0, "specular": 0.5},
              {"position": (extent + 20.0, 10.0, extent + 20.0), "diffuse": 0.8, "specular": 0.5}]
    return SceneData(cfg, pos, nrm, mids, mats, eye=(0.0, 0.35 * extent, 2.6 * extent), target=(0, 0, 0),
                     fov=60.0, width=width, height=height, depth=3, lights=lights,
                     seed=SEED_BASE + CONFIG_INDEX[cfg])


# ---------------------------------------------------------------- P
def architecture(grid: int = 40, segments: int = 34, rings: int = 8, width: int = 1920, height: int = 1080,
                 slab_cells: int = 100, arch_segments: int = 16) -> SceneData:
    """40x40 pillars (cylinders: segments x rings), floor + ceiling slabs, arches between pillars along x."""
    spacing, radius, height_y = 4.0, 0.5, 10.0
    th = np.linspace(0.0, 2 * np.pi, segments, endpoint=False)
    ys = np.linspace(0.0, height_y, rings + 1)
    # one cylinder around the origin
    ring_pts = np.stack([np.cos(th), np.zeros_like(th), np.sin(th)], 1)       # [S,3] unit
    verts = (ring_pts[None, :, :] * radius + np.stack([np.zeros_like(ys), ys, np.zeros_like(ys)], 1)[:, None, :])
    vn = np.broadcast_to(ring_pts[None], verts.shape)
    verts = verts.reshape(-1, 3)
    vn = vn.reshape(-1, 3)
    faces = []
    for r in range(rings):
        for s in range(segments):
            a = r * segments + s
            b = r * segments + (s + 1) % segments
            c = (r + 1) * segments + (s + 1) % segments
            d = (r + 1) * segments + s
            faces += [(a, d, c), (a, c, b)]
    faces = np.array(faces, np.int64)
    cyl = verts[faces]                         # [F,3,3]
    cyln = vn[faces]
    gx, gz = np.meshgrid(np.arange(grid) * spacing, np.arange(grid) * spacing, indexing="ij")
    offs = np.stack([gx.ravel(), np.zeros(grid * grid), gz.ravel()], 1)        # [G,3]
    ptri = (cyl[None] + offs[:, None, None, :]).reshape(-1, 3, 3)
    pn = np.broadcast_to(cyln[None], (grid * grid, *cyln.shape)).reshape(-1, 3, 3)
    mids = np.repeat((np.arange(grid * grid) % 8).astype(np.uint32), cyl.shape[0])
    parts_p, parts_n, parts_m = [ptri], [pn], [mids]
    # floor and ceiling slabs: tessellated grids
    lo, hi = -spacing, (grid - 1) * spacing + spacing
    xs = np.linspace(lo, hi, slab_cells + 1)
    for y, up in ((0.0, 1.0), (height_y, -1.0)):
        X, Z = np.meshgrid(xs, xs, indexing="ij")
        P = np.stack([X, np.full_like(X, y), Z], -1)
        a = P[:-1, :-1].reshape(-1, 3)
        b = P[1:, :-1].reshape(-1, 3)
        c = P[1:, 1:].reshape(-1, 3)
        d = P[:-1, 1:].reshape(-1, 3)
        if up > 0:
            t1 = np.stack([a, d, c], 1)
            t2 = np.stack([a, c, b], 1)
        else:
            t1 = np.stack([a, c, d], 1)
            t2 = np.stack([a, b, c], 1)
        t = np.concatenate([t1, t2])
        parts_p.append(t)
        parts_n.append(np.broadcast_to(np.array([0.0, up, 0.0]), t.shape))
        parts_m.append(np.full(len(t), 8 if up > 0 else 9, np.uint32))
    # arches: a semicircular band between neighbouring pillars along x, front and back faces
    ar = spacing / 2 - radius
    ang = np.linspace(0.0, np.pi, arch_segments + 1)
    for zoff in (-0.3, 0.3):
        base = []
        for k in range(arch_segments):
            a0, a1 = ang[k], ang[k + 1]
            p0 = (spacing / 2 - ar * np.cos(a0), 7.0 + ar * np.sin(a0))
            p1 = (spacing / 2 - ar * np.cos(a1), 7.0 + ar * np.sin(a1))
            q0 = (spacing / 2 - (ar + 0.4) * np.cos(a0), 7.0 + (ar + 0.4) * np.sin(a0))
            q1 = (spacing / 2 - (ar + 0.4) * np.cos(a1), 7.0 + (ar + 0.4) * np.sin(a1))
            A = (p0[0], p0[1], zoff)
            B = (p1[0], p1[1], zoff)
            Cc = (q1[0], q1[1], zoff)
            D = (q0[0], q0[1], zoff)
            base += [(A, B, Cc), (A, Cc, D)]
        base = np.array(base, np.float64)                        # [2*arch_segments,3,3]
        ax, az = np.meshgrid(np.arange(grid - 1) * spacing, np.arange(grid) * spacing, indexing="ij")
        ao = np.stack([ax.ravel(), np.zeros(ax.size), az.ravel()], 1)
        t = (base[None] + ao[:, None, None, :]).reshape(-1, 3, 3)
        parts_p.append(t)
        parts_n.append(np.broadcast_to(np.array([0.0, 0.0, np.sign(zoff)]), t.shape))
        parts_m.append(np.full(len(t), 10, np.uint32))
    tri = np.concatenate(parts_p)
    nt = np.concatenate([np.asarray(x, np.float64) for x in parts_n])
    ones = np.ones((*tri.shape[:2], 1))
    pos = np.concatenate([tri, ones], 2).astype(np.float32)
    nrm = np.concatenate([nt, np.zeros_like(ones)], 2).astype(np.float32)
    mids = np.concatenate(parts_m)
    mats = _materials(_rng("P", 2), 11)
    c = (grid - 1) * spacing
    lights = [{"position": (0.25 * c, 9.0, 0.25 * c), "diffuse": 0.9, "specular": 0.4},
              {"position": (0.75 * c, 9.0, 0.25 * c), "diffuse": 0.9, "specular": 0.4},
              {"position": (0.25 * c, 9.0, 0.75 * c), "diffuse": 0.9, "specular": 0.4},
              {"position": (0.75 * c, 9.0, 0.75 * c), "diffuse": 0.9, "specular": 0.4}]
    return SceneData("P", pos, nrm, mids, mats, eye=(-6.0, 5.0, -6.0), target=(0.5 * c, 3.0, 0.5 * c),
                     fov=60.0, width=width, height=height, depth=2, lights=lights, jitter=1.0,
                     seed=SEED_BASE + 2)


# ---------------------------------------------------------------- B / Srv helpers
def random_soup(n_tris: int, rng: np.random.Generator, extent: float = 20.0) -> SceneData:
    """A soup of jittered icospheres (subdiv 1, 80 triangles each) with about n_tris triangles."""
    n_sph = max(1, n_tris // 80)
    sv, sf = icosphere(1)
    centers = rng.uniform(-extent, extent, (n_sph, 3))
    radii = rng.lognormal(-0.5, 0.5, n_sph)
    verts = sv[None] * radii[:, None, None] + centers[:, None, :]
    verts = verts + rng.normal(0, 0.05, verts.shape) * radii[:, None, None]
    tri = verts[:, sf].reshape(-1, 3, 3)
    vn = (sv[None] * np.ones((n_sph, 1, 1)))[:, sf].reshape(-1, 3, 3)
    ones = np.ones((*tri.shape[:2], 1))
    pos = np.concatenate([tri, ones], 2).astype(np.float32)
    nrm = np.concatenate([vn, np.zeros_like(ones)], 2).astype(np.float32)
    mids = np.repeat((np.arange(n_sph) % 8).astype(np.uint32), sf.shape[0])
    return SceneData("soup", pos, nrm, mids, _materials(rng, 8), eye=(0.0, 0.0, 3.0 * extent), fov=60.0)


def surface_rays(scene: SceneData, n: int, rng: np.random.Generator, eps: float = 0.01) -> np.ndarray:
    """Rays leaving triangle surfaces (uniform barycentrics); direction uniform on the sphere or the mirror
    reflection of a view direction, 50/50; origin offset by eps along the direction."""
    from . import RAY_DTYPE
    T = scene.tri_count
    t = rng.integers(0, T, n)
    u = rng.random(n)
    v = rng.random(n)
    flip = u + v > 1
    u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
    P = scene.positions[t, :, :3].astype(np.float64)
    p = P[:, 0] * (1 - u - v)[:, None] + P[:, 1] * u[:, None] + P[:, 2] * v[:, None]
    nrm = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    d_uni = rng.normal(size=(n, 3))
    d_uni /= np.linalg.norm(d_uni, axis=1, keepdims=True)
    view = p - np.array(scene.eye)
    view /= np.maximum(np.linalg.norm(view, axis=1, keepdims=True), 1e-30)
    d_ref = view - 2 * np.sum(view * nrm, 1, keepdims=True) * nrm
    d_ref /= np.maximum(np.linalg.norm(d_ref, axis=1, keepdims=True), 1e-30)
    pick = rng.random(n) < 0.5
    d = np.where(pick[:, None], d_uni, d_ref)
    rays = np.zeros(n, RAY_DTYPE)
    rays["o"] = (p + eps * d).astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = eps
    rays["tmax"] = np.inf
    return rays


def batch_config(n_batches: int = 256, n_scenes: int = 16, min_rays: int = 4096, max_rays: int = 2_000_000,
                 min_tris: int = 10_000, max_tris: int = 1_000_000, seed_stage: int = 0):
    """Config B: scenes with log-uniform triangle counts and batches with log-uniform sizes."""
    rng = _rng("B", seed_stage)
    tris = np.exp(rng.uniform(np.log(min_tris), np.log(max_tris), n_scenes)).astype(np.int64)
    scenes = [random_soup(int(t), np.random.default_rng([SEED_BASE + 3, 100 + i])) for i, t in enumerate(tris)]
    sizes = np.exp(rng.uniform(np.log(min_rays), np.log(max_rays), n_batches)).astype(np.int64)
    which = rng.integers(0, n_scenes, n_batches)
    any_hit = rng.random(n_batches) < 0.5
    return scenes, sizes, which, any_hit


def by_name(name: str) -> SceneData:
    return {"S": cornell, "O": soup, "P": architecture}[name]()
