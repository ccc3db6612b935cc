"""The per-frame path (rsh_render_frame) checked stage by stage against the oracle: every intermediate
buffer of the frame is recomputed on the CPU from the GPU's previous stage and must match bit for bit;
every hit record / shadow flag must equal the brute-force oracle; the image must equal the oracle's
shading of the same buffers within 2/255 per channel (host and device powf / log2f may differ by an ulp)."""
import numpy as np
import pytest

import frame_check
import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu


def _check_frame(ctx, s, sc, W, H, depth, jitter, samples=1):
    """Every ray of the frame against the oracle (frame_check.check_frame with no sampling)."""
    st, _ = frame_check.check_frame(ctx, s, sc, W, H, depth, jitter, samples=samples)
    return st


@pytest.mark.parametrize("ray_level", [0, 3])
@pytest.mark.parametrize("jitter", [0.0, 1.0])
def test_frame_cornell(cornell, jitter, ray_level):
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8, reflect_jitter=jitter,
                      ray_level=ray_level, plain_ray_level=ray_level)
    sc = ctx.scene(cornell.positions, cornell.normals, cornell.material_ids, cornell.materials)
    st = _check_frame(ctx, cornell, sc, 128, 96, 2, jitter)
    assert st["secondary_ms"] > 0
    sc.destroy()
    ctx.destroy()


def test_frame_soup_small():
    s = scenes.soup(n_spheres=300, width=96, height=64, extent=20.0)
    s.lights = s.lights[:2]
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=16, cluster_size=8)
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    _check_frame(ctx, s, sc, 96, 64, 3, 0.0)
    sc.destroy()
    ctx.destroy()


def test_fused_frame_equals_plain_frame():
    """RSH_FLAG_FUSED (batched form inside the frame) must give the same hits, flags and image."""
    s = scenes.soup(n_spheres=400, width=128, height=96, extent=25.0)
    outs = []
    for flags in (0, rsh.FLAG_FUSED, rsh.FLAG_FUSED | rsh.FLAG_NO_COMPRESS):
        ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8, reflect_jitter=1.0, flags=flags)
        sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
        ctx.set_camera(rsh.camera_look_at(s.eye, s.target, s.up, s.fov, 128, 96))
        ctx.set_lights(s.lights)
        rgba = rsh.DeviceArray(128 * 96, np.uint32)
        ctx.render(sc, 128, 96, 3, rgba)
        ctx.check_device_errors()
        st = ctx.stats()
        res = [ctx.frame_hits(-1, 128 * 96)]
        for b in range(3):
            res += [ctx.frame_hits(b, 128 * 96), ctx.frame_shadow(b, 128 * 96 * len(s.lights))]
        res.append(rgba.numpy())
        outs.append((res, st))
        sc.destroy()
        ctx.destroy()
    for other in outs[1:]:
        for a, b in zip(outs[0][0], other[0]):
            assert np.array_equal(a, b)
        assert outs[0][1]["shadow_rays"] == other[1]["shadow_rays"]
        assert outs[0][1]["reflection_rays"] == other[1]["reflection_rays"]


@pytest.mark.parametrize("ray_level", [0, 3])
def test_rah_ablation_same_results_more_work(cornell, ray_level):
    """RAH (no hashing/sorting, main.cpp:1016-1037) gives the same hits and flags as CRSH; with packets the
    unsorted rays make wider cones, so the traversal does more node tests (the thesis' CRSH vs RAH
    comparison, Thesis_Evaluation.tex:217-219)."""
    W, H = 128, 128
    res = {}
    for flags in (0, rsh.FLAG_RAH):
        ctx = rsh.Context(grid_bits=5, dir_log2=5, packet_size=8, cluster_size=8, flags=flags, ray_level=ray_level,
                          plain_ray_level=ray_level)
        sc = ctx.scene(cornell.positions, cornell.normals, cornell.material_ids, cornell.materials)
        ctx.set_camera(rsh.camera_look_at(cornell.eye, cornell.target, cornell.up, cornell.fov, W, H))
        ctx.set_lights(cornell.lights)
        ctx.render(sc, W, H, 2)
        st = ctx.stats()
        res[flags] = ([ctx.frame_hits(b, W * H) for b in range(2)] + [ctx.frame_shadow(b, W * H) for b in range(2)], st)
        sc.destroy()
        ctx.destroy()
    for a, b in zip(res[0][0], res[rsh.FLAG_RAH][0]):
        assert np.array_equal(a, b)
    if ray_level == 0:
        assert res[rsh.FLAG_RAH][1]["node_tests"] > res[0][1]["node_tests"]


@pytest.mark.parametrize("ray_level", [0, 3])
def test_frame_rah_against_the_oracle(cornell, ray_level):
    """RAH frames (unsorted packets) pass the whole stage-by-stage check: every hit and flag equals brute
    force, not only the CRSH frame's."""
    ctx = rsh.Context(grid_bits=5, dir_log2=5, packet_size=8, cluster_size=8, flags=rsh.FLAG_RAH,
                      reflect_jitter=1.0, ray_level=ray_level, plain_ray_level=ray_level)
    sc = ctx.scene(cornell.positions, cornell.normals, cornell.material_ids, cornell.materials)
    _check_frame(ctx, cornell, sc, 128, 96, 2, 1.0)
    sc.destroy()
    ctx.destroy()


@pytest.mark.parametrize("flags", [0, rsh.FLAG_FUSED])
def test_frame_soft_shadows(cornell, flags):
    """RSH_FLAG_SOFT_SHADOWS: 16 shadow rays per light, each traced exactly, shaded with the reference's
    sample weights; the same frame as the oracle in both forms, with a penumbra."""
    W, H = 64, 48
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8, reflect_jitter=1.0,
                      flags=flags | rsh.FLAG_SOFT_SHADOWS)
    sc = ctx.scene(cornell.positions, cornell.normals, cornell.material_ids, cornell.materials)
    st = _check_frame(ctx, cornell, sc, W, H, 2, 1.0, samples=16)
    flags0 = ctx.frame_shadow(0, W * H * 16).reshape(H, 16, W)
    part = (flags0 != 0).any(axis=1) & ~(flags0 != 0).all(axis=1)
    assert part.sum() > 0  # some pixels see part of the light
    assert st["shadow_rays"] > 0
    sc.destroy()
    ctx.destroy()


def test_frame_from_obj_file(cornell, tmp_path):
    """A scene read by rsh_obj_load (OBJ + MTL) renders through the whole frame like any other: the Cornell
    scene written out as OBJ text (9-digit floats, vertex normals, one material per object) reads back to
    the same arrays and passes the stage-by-stage frame check."""
    import dataclasses

    s = cornell
    T = s.tri_count
    lines, mtl = ["mtllib scene.mtl"], []
    for k, m in enumerate(s.materials):
        mtl += [f"newmtl m{k}", "Kd %.9g %.9g %.9g" % tuple(m[:3]), "Ks %.9g %.9g %.9g" % tuple(m[4:7]),
                "Ns %.9g" % m[7]]
    for t in range(T):
        for v in range(3):
            lines.append("v %.9g %.9g %.9g" % tuple(s.positions[t, v, :3]))
            lines.append("vn %.9g %.9g %.9g" % tuple(s.normals[t, v, :3]))
    cur = None
    for t in range(T):
        if s.material_ids[t] != cur:
            cur = s.material_ids[t]
            lines.append(f"usemtl m{cur}")
        a = 3 * t + 1
        lines.append(f"f {a}//{a} {a + 1}//{a + 1} {a + 2}//{a + 2}")
    (tmp_path / "scene.obj").write_text("\n".join(lines) + "\n")
    (tmp_path / "scene.mtl").write_text("\n".join(mtl) + "\n")
    d = rsh.load_obj(tmp_path / "scene.obj")
    assert np.array_equal(d["positions"][:, :, :3], s.positions[:, :, :3])
    assert np.array_equal(d["normals"][:, :, :3], s.normals[:, :, :3])
    assert np.array_equal(d["material_ids"], s.material_ids.astype(np.uint32) + 1)
    assert np.allclose(d["materials"][1:, [0, 1, 2, 4, 5, 6, 7]], s.materials[:, [0, 1, 2, 4, 5, 6, 7]])
    so = dataclasses.replace(s, positions=d["positions"], normals=d["normals"], material_ids=d["material_ids"],
                             materials=d["materials"])
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8, flags=rsh.FLAG_FUSED)
    sc = ctx.scene(so.positions, so.normals, so.material_ids, so.materials)
    _check_frame(ctx, so, sc, 64, 48, 2, 0.0)
    sc.destroy()
    ctx.destroy()
