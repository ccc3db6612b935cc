"""The reference's own scenes on the GPU, entered the way the reference's engine enters them: the rest pose
as read from its model files, one object id per triangle, then per-object model and normal matrices
through rsh_scene_set_transforms (main.cpp:1131-1196 -> TriangleUpdateWrapper). The moved triangles equal
the oracle's (bit for bit); the 512x512 frames, in both forms, equal the oracle stage by stage with every
ray checked against brute force (frame_check); and the per-iteration ray totals are the oracle's, which
test_reference_scenes.py pins to the numbers the reference recorded for these scenes.

Last, the reference's CRSH-versus-RAH ablation (RayTracer.cu:1361-1405, main.cpp:1016-1037) on its
Cornell box: each recorded iteration's rays (shadow, reflection 1, reflection 2) traced by the plain path
with sorted packets (CRSH) and with unsorted ones (RSH_FLAG_RAH), packets all the way down to the triangle
clusters. Both give exactly the brute-force records; the work each does (node tests + ray x triangle
tests, the reference's 'Algorithm Total', TestManager.cpp:281) is printed as a fraction of rays x
triangles beside the reference's recorded fractions."""
import numpy as np
import pytest

import frame_check
import oracle
import reference_scenes as rs
import rsh

pytestmark = pytest.mark.gpu


def _scene(ctx, name):
    s, rest, rec = rs.load(name)
    sc = ctx.scene(rest["positions"], rest["normals"], s.material_ids, s.materials, object_ids=rest["object_ids"])
    sc.set_transforms(rest["model"].reshape(-1, 4, 4), rest["normal"].reshape(-1, 4, 4))
    ctx.check_device_errors()
    assert sc.triangles().tobytes() == s.positions.tobytes()
    return s, sc, rec


@pytest.mark.parametrize("name,depth", [("cornell", 2), ("office", 1)])
def test_reference_scene_frames_every_ray(name, depth):
    ctx = rsh.Context(rsh.default_config())
    s, sc, rec = _scene(ctx, name)
    cache = frame_check.BruteCache()
    totals, _ = rs.oracle_ray_totals(s, depth_reflect=depth)
    npix = s.width * s.height
    for flags in (0, rsh.FLAG_FUSED):
        ctx.set_config(flags=flags)
        st, checked = frame_check.check_frame(ctx, s, sc, s.width, s.height, depth, 0.0, cache=cache)
        assert checked["primary"] == npix
        # the reference's iterations: shadow rays of the primary surface, then each bounce's reflections
        shadow0 = ctx.frame_rays(0, True, npix)
        assert int((shadow0["tmax"] > shadow0["tmin"]).sum()) == totals[0]
        for b in range(depth):
            r = ctx.frame_rays(b, False, npix)
            assert int((r["tmax"] > r["tmin"]).sum()) == totals[1 + b]
    sc.destroy()
    ctx.destroy()


def test_crsh_versus_rah_on_the_reference_cornell_box(capsys):
    s, rest, rec = rs.load("cornell")
    totals, out = rs.oracle_ray_totals(s, depth_reflect=2)
    T = s.tri_count
    its = [("shadow", out["shadow_rays"], True), ("reflection 1", out["reflection_rays0"], False),
           ("reflection 2", out["reflection_rays1"], False)]
    rows = []
    for ray_level in (0, 4):
        for mode, flags in (("CRSH", 0), ("RAH", rsh.FLAG_RAH)):
            ctx = rsh.Context(rsh.default_config(flags=flags, plain_ray_level=ray_level))
            sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
            for k, (it, rays, any_hit) in enumerate(its):
                keep = rays[rays["tmax"] > rays["tmin"]]
                ctx.test_counters(reset=True)
                got = ctx.trace(sc, keep, any_hit)
                nodes, tris = ctx.test_counters(reset=True)
                assert np.array_equal(got, oracle.brute(s.positions, keep, any_hit)), (mode, it)
                R = len(keep)
                ref = int(rec["crsh_algorithm" if mode == "CRSH" else "rah_algorithm"][k])
                rows.append((ray_level, mode, it, R, nodes, tris, (nodes + tris) / (R * T), ref / (int(rec["crsh_rays"][k]) * T)))
            sc.destroy()
            ctx.destroy()
    with capsys.disabled():
        print("\nreference Cornell box, 512x512: work / (rays x triangles)")
        for r in rows:
            print(f"  switch level {r[0]} {r[1]:4s} {r[2]:12s} rays {r[3]:7d} node tests {r[4]:9d} "
                  f"tri tests {r[5]:9d}  ours {100 * r[6]:6.2f}%  reference {100 * r[7]:6.2f}%")
    # packets of sorted rays never do more node tests than packets of unsorted ones
    for it in ("shadow", "reflection 1", "reflection 2"):
        crsh = [r for r in rows if r[0] == 0 and r[1] == "CRSH" and r[2] == it][0]
        rah = [r for r in rows if r[0] == 0 and r[1] == "RAH" and r[2] == it][0]
        assert crsh[4] <= rah[4], it
