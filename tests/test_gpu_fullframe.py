"""The full-size architecture frame (1,010,240 triangles, 1920x1080, 4 point lights, depth 2, cosine-lobe
reflections: 16.6 M shadow and 4.1 M reflection rays) traced by the batched form and by the plain
per-frame path: every primary hit, shadow flag and reflection hit of every bounce agrees. The two paths
share no traversal code (k_fused against k_traverse + k_intersect), so a ray that one of them drops shows
up here, at a size the brute-force oracle cannot check whole; each disagreement is settled by brute force
on that ray alone, so the failure message says which path is wrong."""
import numpy as np
import pytest

import oracle
import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu


def _frame(ctx, sc, s, flags):
    ctx.set_config(flags=flags)
    W, H = s.width, s.height
    rgba = rsh.DeviceArray(W * H, np.uint32)
    ctx.render(sc, W, H, s.depth, rgba)
    ctx.check_device_errors()
    npix, L = W * H, len(s.lights)
    out = {"prim": ctx.frame_hits(-1, npix), "img": rgba.numpy()}
    for b in range(s.depth):
        out[f"shadow{b}"] = ctx.frame_shadow(b, npix * L)
        out[f"hits{b}"] = ctx.frame_hits(b, npix)
        out[f"refl_rays{b}"] = ctx.frame_rays(b, False, npix)
    return out


def _settle(ctx, s, b, key, idx, plain, fused):
    """Brute force on the disagreeing rays of one buffer: how many each path got right."""
    npix, L = s.width * s.height, len(s.lights)
    any_hit = key.startswith("shadow")
    rays = ctx.frame_rays(b, True, npix * L)[idx] if any_hit else fused[f"refl_rays{b}"][idx]
    bf = oracle.brute(s.positions, rays, any_hit)
    return int((plain[key][idx] == bf).sum()), int((fused[key][idx] == bf).sum())


@pytest.mark.parametrize("ray_level", [6, 15])  # packets above the top level / rays alone from the root
def test_fused_and_plain_paths_agree_on_the_full_frame(ray_level):
    s = scenes.by_name("P")
    ctx = rsh.Context(rsh.default_config(reflect_jitter=float(s.jitter), seed=s.seed, ray_level=ray_level))
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    ctx.set_camera(rsh.camera_look_at(s.eye, s.target, s.up, s.fov, s.width, s.height))
    ctx.set_lights(s.lights)
    plain = _frame(ctx, sc, s, 0)
    fused = _frame(ctx, sc, s, rsh.FLAG_FUSED)  # the fused frame's buffers stay current for _settle
    assert np.array_equal(plain["prim"], fused["prim"])
    report = []
    for b in range(s.depth):
        assert plain[f"refl_rays{b}"].tobytes() == fused[f"refl_rays{b}"].tobytes(), f"bounce {b} rays"
        for key in (f"shadow{b}", f"hits{b}"):
            idx = np.nonzero(plain[key] != fused[key])[0]
            if len(idx):
                ok_plain, ok_fused = _settle(ctx, s, b, key, idx[:256], plain, fused)
                report.append(f"{key}: {len(idx)} differ; of the first {min(len(idx), 256)}, brute force agrees "
                              f"with plain {ok_plain}, with fused {ok_fused}")
    assert not report, "; ".join(report)
    assert np.array_equal(plain["img"], fused["img"])
    sc.destroy()
    ctx.destroy()
