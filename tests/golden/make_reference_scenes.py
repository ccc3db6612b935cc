"""Writes the reference's own two scenes as test fixtures, rebuilt from the reference's model files, with the
numbers the reference recorded for them (its per-frame test dumps at 512x512).

  reference_cornell.npz  the "Kornell" scene (main.cpp:2020-2140): models/Cube.obj as six walls
                         (positions, Euler rotations and scales of main.cpp:2027-2054, materials
                         silver/silver/gold/ruby/saphire/emerald) and models/sphere/sphere.obj scaled 25x at
                         (0, -12.5, 0); 792 triangles. Camera: zoom 4.5, latitude 0.5, longitude 225, target
                         (4.35, -24.35, 1.5) (main.cpp:1927-1939); light (0, 45, 0), colour 0.8, diffuse and
                         specular 0.75 (main.cpp:1824-1838).
  reference_office.npz   the office scene (main.cpp:1975-2018): models/office.obj scaled 10x at (0, -15, 0);
                         36,308 triangles. Camera: zoom 0.5, latitude 30.5, longitude 215, target
                         (-4.5, 7.25, 1.5) (main.cpp:1910-1925); light (-15, 15, 7.5), white, 0.75 / 0.75
                         (main.cpp:1807-1821).

Both store the rest pose as read from the OBJ files (per-object model space, as the reference uploads it)
plus one model matrix and one normal matrix per object, built as the reference builds them: model =
T * R * S with R from the x, y, z Euler angles in that order (Transform.cpp:21-46), normal matrix = the
inverse transpose of the model matrix without its translation (main.cpp:1131-1146). The office keeps its
indexed form (vertex, normal and face index arrays) to stay small.

Recorded numbers (output/tests/configuration-n8/test-{crsh,rah}-d2-n8-{cornell,office}.txt, produced by
TestManager::dump, TestManager.cpp:226-282): ray totals of each iteration (Cornell: shadow rays, then
reflection iterations 1 and 2; office: shadow rays), the triangle total, and the brute-force and
algorithm totals (node-vs-triangle-sphere tests plus 8 rays per connected leaf, TestManager.cpp:281).

Run here, where the reference tree is present; the GPU tests read only the fixtures.
"""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np

REF = Path("/root/reference")
MODELS = REF / "projects" / "CUDA-Engine" / "models"
DUMPS = REF / "output" / "tests" / "configuration-n8"
OUT = Path(__file__).resolve().parent


def read_obj(path: Path):
    """v / vn / f (v, v/t, v//n, v/t/n; 1-based or negative indices) and usemtl. Returns vertices,
    normals, per-face vertex and normal indices (0-based; -1 = no normal) and per-face material names."""
    V, N, fv, fn, fm = [], [], [], [], []
    mat = None
    for line in path.read_text().splitlines():
        p = line.split()
        if not p:
            continue
        if p[0] == "v":
            V.append([float(x) for x in p[1:4]])
        elif p[0] == "vn":
            N.append([float(x) for x in p[1:4]])
        elif p[0] == "usemtl":
            mat = p[1]
        elif p[0] == "f":
            idx = []
            for w in p[1:]:
                parts = w.split("/")
                vi = int(parts[0])
                ni = int(parts[2]) if len(parts) > 2 and parts[2] else 0
                vi = vi - 1 if vi > 0 else len(V) + vi
                ni = ni - 1 if ni > 0 else (len(N) + ni if ni < 0 else -1)
                idx.append((vi, ni))
            for k in range(1, len(idx) - 1):  # fan
                tri = (idx[0], idx[k], idx[k + 1])
                fv.append([t[0] for t in tri])
                fn.append([t[1] for t in tri])
                fm.append(mat)
    return (np.array(V, np.float32), np.array(N, np.float32), np.array(fv, np.int64), np.array(fn, np.int64), fm)


def read_mtl(path: Path) -> dict:
    """newmtl -> (Kd, Ks, Ns)."""
    out, cur = {}, None
    for line in path.read_text().splitlines():
        p = line.split()
        if not p:
            continue
        if p[0] == "newmtl":
            cur = p[1]
            out[cur] = [[0.75, 0.75, 0.75], [0.0, 0.0, 0.0], 100.0]
        elif cur and p[0] == "Kd":
            out[cur][0] = [float(x) for x in p[1:4]]
        elif cur and p[0] == "Ks":
            out[cur][1] = [float(x) for x in p[1:4]]
        elif cur and p[0] == "Ns":
            out[cur][2] = float(p[1])
    return out


def material_row(m, reflectance=1.0):
    kd, ks, ns = m
    return [kd[0], kd[1], kd[2], reflectance, ks[0], ks[1], ks[2], ns]


def model_matrices(position, rotation_deg, scale):
    """Row-major 4x4 model matrix T * Rx * Ry * Rz * S and its normal matrix (inverse transpose of the
    upper 3x3, no translation), both float32."""
    ax, ay, az = np.radians(rotation_deg)
    rx = np.array([[1, 0, 0], [0, np.cos(ax), -np.sin(ax)], [0, np.sin(ax), np.cos(ax)]])
    ry = np.array([[np.cos(ay), 0, np.sin(ay)], [0, 1, 0], [-np.sin(ay), 0, np.cos(ay)]])
    rz = np.array([[np.cos(az), -np.sin(az), 0], [np.sin(az), np.cos(az), 0], [0, 0, 1]])
    m3 = rx @ ry @ rz @ np.diag(scale)
    m = np.eye(4)
    m[:3, :3] = m3
    m[:3, 3] = position
    nm = np.eye(4)
    nm[:3, :3] = np.linalg.inv(m3).T
    return m.astype(np.float32), nm.astype(np.float32)


def orbit_camera(zoom, latitude, longitude, target, radius=25.0):
    """Camera::loadView's eye and up (Camera.cpp:92-102) for an orbit camera (CAMERA_RADIUS 25,
    Camera.h:40)."""
    lat, lon = np.radians(latitude - 90.0), np.radians(longitude)
    t = np.array(target, np.float64)
    eye = t + zoom * radius * np.array([np.sin(lat) * np.cos(lon), np.cos(lat), -np.sin(lat) * np.sin(lon)])
    up = np.array([0.0, np.cos(np.radians(latitude)), 0.0])
    return eye.astype(np.float32), t.astype(np.float32), up.astype(np.float32)


def read_dump(path: Path) -> dict:
    """Ray totals, triangle total, brute-force and algorithm totals of every iteration in a test dump."""
    it = {"rays": [], "tris": [], "brute": [], "algorithm": []}
    for line in path.read_text().splitlines():
        m = re.match(r"Ray Total:\s+(\d+)", line)
        if m:
            it["rays"].append(int(m.group(1)))
        m = re.match(r"TriangleTotal:\s+(\d+)", line)
        if m:
            it["tris"].append(int(m.group(1)))
        m = re.match(r"\[Algorithm\] Brute Force Total:\s+(\d+)", line)
        if m:
            it["brute"].append(int(m.group(1)))
        m = re.match(r"\[Algorithm\] Algorithm Total:\s+(\d+)", line)
        if m:
            it["algorithm"].append(int(m.group(1)))
    return {k: np.array(v, np.int64) for k, v in it.items()}


def tri_arrays(V, N, fv, fn):
    """Per-triangle float4 vertex positions (w = 1) and normals (w = 0), [T, 3, 4]."""
    T = len(fv)
    pos = np.zeros((T, 3, 4), np.float32)
    nrm = np.zeros((T, 3, 4), np.float32)
    pos[:, :, :3] = V[fv]
    pos[:, :, 3] = 1.0
    ok = fn >= 0
    nrm[:, :, :3][ok] = N[fn[ok]]
    return pos, nrm


def cornell():
    V, N, fv, fn, _ = read_obj(MODELS / "Cube.obj")
    SV, SN, sfv, sfn, _ = read_obj(MODELS / "sphere" / "sphere.obj")
    walls = [((0, 50, 0), (0, 0, 0), (200, 0.5, 200), "silver"), ((0, -50, 0), (0, 0, 0), (200, 0.5, 200), "silver"),
             ((-100, 0, 0), (0, 0, 90), (100, 0.5, 200), "gold"), ((100, 0, 0), (0, 0, 90), (100, 0.5, 200), "ruby"),
             ((0, 0, 100), (90, 0, 0), (200, 0.5, 100), "saphire"), ((0, 0, -100), (90, 0, 0), (200, 0.5, 100), "emerald")]
    cube_pos, cube_nrm = tri_arrays(V, N, fv, fn)
    sph_pos, sph_nrm = tri_arrays(SV, SN, sfv, sfn)
    pos, nrm, obj, mid, model, normal, mats = [], [], [], [], [], [], []
    for k, (p, r, s, mname) in enumerate(walls):
        m, nm = model_matrices(p, r, s)
        pos.append(cube_pos)
        nrm.append(cube_nrm)
        obj.append(np.full(len(cube_pos), k, np.uint32))
        mid.append(np.full(len(cube_pos), k, np.uint32))
        model.append(m)
        normal.append(nm)
        mats.append(material_row(read_mtl(MODELS / f"{mname}.mtl")[next(iter(read_mtl(MODELS / f'{mname}.mtl')))]))
    m, nm = model_matrices((0, -12.5, 0), (0, 0, 0), (25, 25, 25))
    pos.append(sph_pos)
    nrm.append(sph_nrm)
    obj.append(np.full(len(sph_pos), 6, np.uint32))
    mid.append(np.full(len(sph_pos), 6, np.uint32))
    model.append(m)
    normal.append(nm)
    gold = read_mtl(MODELS / "sphere" / "gold.mtl")
    mats.append(material_row(gold[next(iter(gold))]))
    eye, target, up = orbit_camera(4.5, 0.5, 225.0, (4.35, -24.35, 1.50))
    crsh = read_dump(DUMPS / "test-crsh-d2-n8-cornell.txt")
    rah = read_dump(DUMPS / "test-rah-d2-n8-cornell.txt")
    np.savez_compressed(
        OUT / "reference_cornell.npz", rest_positions=np.concatenate(pos), rest_normals=np.concatenate(nrm),
        object_ids=np.concatenate(obj), material_ids=np.concatenate(mid), materials=np.array(mats, np.float32),
        model=np.array(model), normal=np.array(normal), eye=eye, target=target, up=up, fov=np.float32(60.0),
        size=np.array([512, 512]), light_position=np.array([0.0, 45.0, 0.0], np.float32),
        light_color=np.array([0.8, 0.8, 0.8], np.float32), light_diffuse=np.float32(0.75),
        light_specular=np.float32(0.75), crsh_rays=crsh["rays"], crsh_tris=crsh["tris"], crsh_brute=crsh["brute"],
        crsh_algorithm=crsh["algorithm"], rah_rays=rah["rays"], rah_algorithm=rah["algorithm"],
        rah_brute=rah["brute"])


def office():
    V, N, fv, fn, fm = read_obj(MODELS / "office.obj")
    mtl = read_mtl(MODELS / "office.mtl")
    names = sorted(set(fm), key=lambda x: (x is None, x or ""))
    mats = [material_row(mtl.get(n, [[0.75, 0.75, 0.75], [0.0, 0.0, 0.0], 100.0])) for n in names]
    index = {n: i for i, n in enumerate(names)}
    m, nm = model_matrices((0, -15, 0), (0, 0, 0), (10, 10, 10))
    eye, target, up = orbit_camera(0.5, 30.5, 215.0, (-4.50, 7.25, 1.50))
    crsh = read_dump(DUMPS / "test-crsh-d2-n8-office.txt")
    rah = read_dump(DUMPS / "test-rah-d2-n8-office.txt")
    assert V.shape[0] < 65536 and N.shape[0] < 65536 and fn.min() >= 0
    np.savez_compressed(
        OUT / "reference_office.npz", vertices=V, normals=N, face_vertices=fv.astype(np.uint16),
        face_normals=fn.astype(np.uint16), material_ids=np.array([index[n] for n in fm], np.uint16),
        materials=np.array(mats, np.float32), model=m[None], normal=nm[None], eye=eye, target=target, up=up,
        fov=np.float32(60.0), size=np.array([512, 512]), light_position=np.array([-15.0, 15.0, 7.5], np.float32),
        light_color=np.array([1.0, 1.0, 1.0], np.float32), light_diffuse=np.float32(0.75),
        light_specular=np.float32(0.75), crsh_rays=crsh["rays"], crsh_tris=crsh["tris"], crsh_brute=crsh["brute"],
        crsh_algorithm=crsh["algorithm"], rah_rays=rah["rays"], rah_algorithm=rah["algorithm"],
        rah_brute=rah["brute"])


if __name__ == "__main__":
    cornell()
    office()
    for f in ("reference_cornell.npz", "reference_office.npz"):
        print(f, (OUT / f).stat().st_size, "bytes")
