"""The three frame configurations at their stated sizes, each rendered by the plain per-frame path and by the
batched form (RSH_FLAG_FUSED), and checked stage by stage against the oracle (frame_check.check_frame):

  S  Cornell-style box + 2 icospheres, 2,580 triangles, 512x512, 1 point light, depth 1: every primary,
     shadow and reflection ray of the frame against brute force over every triangle.
  O  object soup, 640,032 triangles, 1920x1080, 2 point lights, depth 3 (shadow + mirror reflection per
     bounce).
  P  procedural architecture, 1,010,240 triangles, 1920x1080, 4 point lights, depth 2, cosine-lobe
     perturbed reflections.

For O and P every ray buffer and surface buffer of the frame is compared bit for bit with the oracle's
recomputation from the GPU's previous stage, and a seeded sample of 16,384 rays per ray type (primary,
shadow, reflection) per bounce is brute-forced over every triangle: hit records (triangle id and the float
bits of t) and shadow flags must be identical. The two forms get the same sample, so a bug in the code they
share (ray generation, the watertight test, hit resolve, shading) cannot hide behind their agreement."""
import numpy as np
import pytest

import frame_check
import oracle
import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu

SAMPLE = 16384


def _both_forms(name, sample):
    s = scenes.by_name(name)
    ctx = rsh.Context(rsh.default_config(reflect_jitter=float(s.jitter), seed=s.seed))
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    cache = frame_check.BruteCache()
    out = {}
    for form, flags in (("plain", 0), ("batched", rsh.FLAG_FUSED)):
        ctx.set_config(flags=flags)
        st, checked = frame_check.check_frame(ctx, s, sc, s.width, s.height, s.depth, float(s.jitter),
                                              sample=sample, seed=0x5EED0000, cache=cache)
        out[form] = (st, checked)
    # the batched form's work counters (the roofline's numerator): with RSH_FLAG_SEQUENTIAL_RAYS (every ray
    # on one lane from its first step to its last) they equal the oracle's restatement of its traversal
    # (per-ray box descent from the root) over the frame's own secondary rays, test for test; by default a
    # drained warp shares its last rays' subtrees among its idle lanes, which changes the counts only through
    # the order the hits are met in (a far subtree is no longer culled by its ray's nearer hits)
    ctx.set_config(flags=rsh.FLAG_FUSED | rsh.FLAG_SEQUENTIAL_RAYS)
    ctx.render(sc, s.width, s.height, s.depth)
    seq = ctx.stats()
    lo, hi = sc.bounds()
    oh = oracle.ObjH(s.positions, ctx.config.cluster_size, lo, hi)
    npix, L = s.width * s.height, len(s.lights)
    nodes = tris = 0
    for b in range(s.depth):
        for rays, any_hit in ((ctx.frame_rays(b, True, npix * L), True), (ctx.frame_rays(b, False, npix), False)):
            _, (n, t) = oh.trace_box(rays[rays["tmax"] > rays["tmin"]], any_hit)
            nodes, tris = nodes + n, tris + t
    assert (seq["node_tests"], seq["tri_tests"]) == (nodes, tris)
    st = out["batched"][0]
    assert abs(st["node_tests"] / nodes - 1.0) < 0.10 and abs(st["tri_tests"] / tris - 1.0) < 0.10
    sc.destroy()
    ctx.destroy()
    # both forms trace the same rays
    assert out["plain"][0]["shadow_rays"] == out["batched"][0]["shadow_rays"]
    assert out["plain"][0]["reflection_rays"] == out["batched"][0]["reflection_rays"]
    return s, out


def test_config_S_whole_frame_every_ray():
    s, out = _both_forms("S", None)
    assert (s.width, s.height, s.tri_count, s.depth, len(s.lights)) == (512, 512, 2580, 1, 1)
    st, checked = out["batched"]
    assert checked["primary"] == 512 * 512
    assert checked["shadow"] == st["shadow_rays"] and checked["reflection"] == st["reflection_rays"]
    assert st["shadow_rays"] > 100_000 and st["reflection_rays"] > 100_000


@pytest.mark.parametrize("name", ["O", "P"])
def test_full_size_frame_sampled_against_brute_force(name):
    s, out = _both_forms(name, SAMPLE)
    want = {"O": (1920, 1080, 640_032, 3, 2), "P": (1920, 1080, 1_010_240, 2, 4)}[name]
    assert (s.width, s.height, s.tri_count, s.depth, len(s.lights)) == want
    for form in ("plain", "batched"):
        st, checked = out[form]
        # a full sample of every ray type in every bounce
        assert checked["primary"] == SAMPLE
        assert checked["shadow"] == SAMPLE * s.depth and checked["reflection"] == SAMPLE * s.depth
        assert st["shadow_rays"] > 1_000_000 and st["reflection_rays"] > 1_000_000
