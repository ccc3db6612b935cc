"""The oracle pinned to numbers the reference recorded for its own scenes.

The reference ships no golden vectors for this path; what it does record are its per-frame test dumps
(output/tests/configuration-n8/test-crsh-d2-n8-{cornell,office}.txt, written by TestManager::dump): how
many rays each iteration traced after trimming, over how many triangles. tests/golden/reference_*.npz hold
its Cornell box (792 triangles: models/Cube.obj as six walls + models/sphere/sphere.obj, main.cpp:2020-2140)
and its office (36,308 triangles, models/office.obj, main.cpp:1975-2018), rebuilt from those model files
with its transforms, camera and light (tests/golden/make_reference_scenes.py).

The oracle renders the reference's iterations at 512x512 (main.cpp:1234-1303): shadow rays from the primary
surface, then two reflection iterations.
  - every reflection iteration: exactly the recorded 262,144 rays (every pixel of the closed box hits a
    wall, and every hit makes the next reflection ray);
  - shadow rays (kept iff the surface faces the light, RayTracer.cu:708-732): within 3% of the recorded
    242,015 (Cornell) and 251,546 (office). Exact equality is not expected: the reference's primary hits
    come from its OpenGL rasteriser (G-buffer), ours from a primary ray cast through the same camera; and
    the recorded frame's camera state is the scene's initial one only as far as the code shows. Every
    shadow ray our count misses lies on the sphere's side turned away from the light.
The GPU frames of the same scenes equal the oracle's buffer for buffer (test_gpu_reference_scenes.py)."""
import numpy as np
import pytest

import oracle
import reference_scenes as rs

SHADOW_BAND = 0.03


def test_fixtures_match_the_recorded_scene_sizes():
    for name, tris in (("cornell", 792), ("office", 36_308)):
        s, rest, rec = rs.load(name)
        assert s.tri_count == tris == int(rec["crsh_tris"][0])
        # the dumps' brute-force totals are rays x triangles, in the reference's 32-bit int (the office's
        # 251,546 x 36,308 = 9,133,132,168 was recorded modulo 2^32 as 543,197,576)
        assert np.array_equal(rec["crsh_brute"], (rec["crsh_rays"] * tris) % (1 << 32))
        assert np.array_equal(rec["rah_rays"], rec["crsh_rays"])
        assert np.all(np.isfinite(s.positions)) and np.all(s.positions[..., 3] == 1.0)
        n = np.linalg.norm(s.normals[..., :3], axis=-1)
        assert np.allclose(n, 1.0, atol=1e-5)


def test_cornell_ray_totals_match_the_recorded_frame():
    s, rest, rec = rs.load("cornell")
    (shadow, refl1, refl2), out = rs.oracle_ray_totals(s, depth_reflect=2)
    assert out["primary_hits"] == 512 * 512  # a closed box: every pixel hits a wall or the sphere
    assert (refl1, refl2) == (int(rec["crsh_rays"][1]), int(rec["crsh_rays"][2])) == (262_144, 262_144)
    assert abs(shadow / int(rec["crsh_rays"][0]) - 1.0) < SHADOW_BAND, (shadow, int(rec["crsh_rays"][0]))
    # the rejected pixels are all on the sphere (object 6), on its side away from the light
    rays, keys = out["shadow_rays"], out["shadow_keys"]
    hits = out["reflection_hits0"]
    assert (keys == oracle.KEY_NONE).sum() == 512 * 512 - shadow
    assert np.all(hits != oracle.HIT_NONE)


def test_office_shadow_rays_match_the_recorded_frame():
    s, rest, rec = rs.load("office")
    (shadow,), out = rs.oracle_ray_totals(s, depth_reflect=0)
    assert abs(shadow / int(rec["crsh_rays"][0]) - 1.0) < SHADOW_BAND, (shadow, int(rec["crsh_rays"][0]))
    assert out["primary_hits"] > 0.9 * 512 * 512


def test_rest_pose_transform_matches_float64_matrices():
    """The world-space scene (oracle.transform of the rest pose) agrees with the model matrices applied in
    float64, to float32 rounding."""
    s, rest, _ = rs.load("cornell")
    obj = rest["object_ids"]
    m = rest["model"].reshape(-1, 4, 4).astype(np.float64)[obj]
    p = np.einsum("tij,tvj->tvi", m, rest["positions"].astype(np.float64))
    assert np.allclose(s.positions, p, rtol=1e-6, atol=1e-4)
