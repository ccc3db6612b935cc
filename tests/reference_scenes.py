"""The reference's own scenes (Cornell box and office), loaded from the fixtures that
tests/golden/make_reference_scenes.py rebuilt from the reference's model files, with the ray totals and
test counts the reference recorded for them at 512x512.

The triangles are stored in their rest pose with one model and one normal matrix per object (as the
reference uploads them); `load` moves them to world space with the oracle's restatement of UpdateVertex
(RayTracer.cu:448-511), the same arithmetic as rsh_scene_set_transforms.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

import oracle
from rsh.scenes import SceneData

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name: str):
    """Returns (SceneData in world space, rest pose dict, recorded numbers dict) for "cornell" or "office"."""
    d = np.load(GOLDEN / f"reference_{name}.npz")
    if name == "office":
        V, N = d["vertices"], d["normals"]
        fv, fn = d["face_vertices"].astype(np.int64), d["face_normals"].astype(np.int64)
        T = len(fv)
        rest_pos = np.zeros((T, 3, 4), np.float32)
        rest_nrm = np.zeros((T, 3, 4), np.float32)
        rest_pos[:, :, :3] = V[fv]
        rest_pos[:, :, 3] = 1.0
        rest_nrm[:, :, :3] = N[fn]
        obj = np.zeros(T, np.uint32)
    else:
        rest_pos, rest_nrm, obj = d["rest_positions"], d["rest_normals"], d["object_ids"].astype(np.uint32)
    model = d["model"].reshape(-1, 16)
    normal = d["normal"].reshape(-1, 16)
    pos, nrm = oracle.transform(rest_pos, rest_nrm, obj, model, normal)
    W, H = (int(x) for x in d["size"])
    light = {"position": tuple(float(x) for x in d["light_position"]),
             "color": tuple(float(x) for x in d["light_color"]),
             "diffuse": float(d["light_diffuse"]), "specular": float(d["light_specular"])}
    s = SceneData(name=f"reference {name}", positions=np.ascontiguousarray(pos, np.float32),
                  normals=np.ascontiguousarray(nrm, np.float32),
                  material_ids=d["material_ids"].astype(np.uint32), materials=d["materials"].astype(np.float32),
                  eye=tuple(float(x) for x in d["eye"]), target=tuple(float(x) for x in d["target"]),
                  up=tuple(float(x) for x in d["up"]), fov=float(d["fov"]), width=W, height=H,
                  depth=2, lights=[light])
    rest = {"positions": rest_pos, "normals": rest_nrm, "object_ids": obj, "model": model, "normal": normal}
    rec = {k: d[k] for k in ("crsh_rays", "crsh_tris", "crsh_brute", "crsh_algorithm", "rah_rays", "rah_algorithm",
                             "rah_brute")}
    return s, rest, rec


def oracle_ray_totals(s, depth_reflect=2, eps=0.01, grid_bits=4, dir_log2=6):
    """The reference's per-frame iterations (main.cpp:1234-1303) on the oracle: shadow rays from the primary
    surface, then reflection rays of the primary surface and of the next bounce. Returns the three ray totals
    (after trimming) and the intermediate arrays."""
    W, H = s.width, s.height
    cam = oracle.camera_look_at(s.eye, s.target, s.up, s.fov, W, H)
    lo = s.positions[..., :3].reshape(-1, 3).min(0)
    hi = s.positions[..., :3].reshape(-1, 3).max(0)
    scale = oracle.hash_scale(lo, hi, grid_bits)
    prays, pix = oracle.raygen_primary(cam, W, H)
    ph = oracle.brute(s.positions, prays, False)
    spos, snrm = oracle.resolve(s.positions, s.normals, s.material_ids, prays, ph, pix, W * H)
    lp = np.array([l["position"] for l in s.lights], np.float32)
    srays, skeys = oracle.raygen_shadow(spos, snrm, W, H, lp, eps, lo, scale, grid_bits, dir_log2)
    totals = [int((skeys != oracle.KEY_NONE).sum())]
    prev, eye = None, cam[:3]
    out = {"primary_hits": int((ph != oracle.HIT_NONE).sum()), "shadow_rays": srays, "shadow_keys": skeys}
    for b in range(depth_reflect):
        rr, rk = oracle.raygen_reflect(spos, snrm, prev, eye if prev is None else None, W, H, eps, 0.0, 0, b, lo,
                                       scale, grid_bits, dir_log2)
        v = rk != oracle.KEY_NONE
        totals.append(int(v.sum()))
        rh = oracle.brute(s.positions, rr, False)
        out[f"reflection_rays{b}"] = rr
        out[f"reflection_hits{b}"] = rh
        spos, snrm = oracle.resolve(s.positions, s.normals, s.material_ids, rr, rh, None, W * H)
        prev = rr
    return totals, out
