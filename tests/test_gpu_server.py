"""Serving loop: continuous batching over resident scenes. Each request's results must be the same alone
and in the mix, and equal to the per-frame path (rsh_render_frame) for the same camera/lights/depth."""
import ctypes as C

import numpy as np
import pytest

import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu


def _request(scene_index, cam, W, H, depth, lights):
    r = rsh.Request()
    r.scene_index = scene_index
    r.camera = cam
    r.width, r.height, r.depth, r.light_count = W, H, depth, len(lights)
    arr = rsh.make_lights(lights)
    for i in range(len(lights)):
        r.lights[i] = arr[i]
    return r


def _run(ctx, scs, reqs, budget=4 << 30, max_inflight=64):
    L = rsh.lib()
    arr = (C.c_void_p * len(scs))(*[s.handle for s in scs])
    srv = C.c_void_p()
    rsh.check(L.rsh_server_create(ctx.handle, arr, len(scs), budget, max_inflight, C.byref(srv)), "server")
    ids = []
    for r in reqs:
        i = C.c_uint64()
        rsh.check(L.rsh_server_submit(srv, C.byref(r), C.byref(i)), "submit")
        ids.append(i.value)
    outs = []
    for r, i in zip(reqs, ids):
        npix = r.width * r.height
        hits = np.empty(npix * r.depth, np.uint64)
        flags = np.empty(npix * r.light_count * r.depth, np.uint32)
        res = rsh.RequestResult()
        st = L.rsh_server_wait(srv, i, 120_000, C.byref(res), hits.ctypes.data, flags.ctypes.data)
        outs.append((st, hits, flags, res.finish_ms - res.submit_ms))
    stats = [C.c_uint64() for _ in range(4)]
    L.rsh_server_stats(srv, *[C.byref(x) for x in stats])
    L.rsh_server_destroy(srv)
    return outs, [x.value for x in stats]


@pytest.fixture(scope="module")
def setup():
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8, reflect_jitter=1.0)
    s0 = scenes.cornell()
    s1 = scenes.soup(n_spheres=300, extent=20.0)
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in (s0, s1)]
    yield ctx, (s0, s1), scs
    for s in scs:
        s.destroy()
    ctx.destroy()


def test_server_alone_equals_mixed_equals_frame(setup):
    ctx, sd, scs = setup
    rng = np.random.default_rng(3)
    reqs = []
    for k in range(7):
        si = k % 2
        s = sd[si]
        W, H = [(64, 64), (96, 48), (40, 72)][k % 3]
        eye = np.array(s.eye) + rng.normal(0, 0.1, 3) * (1 if si == 0 else 10)
        cam = rsh.camera_look_at(eye, s.target, s.up, s.fov, W, H)
        lights = (s.lights * 2)[: 1 + k % 3]
        reqs.append(_request(si, cam, W, H, 1 + k % 3, lights))
    mixed, stats = _run(ctx, scs, reqs)
    assert stats[0] == len(reqs)          # completed
    assert stats[2] >= 2                  # several requests were in flight together
    for k, r in enumerate(reqs):
        alone, _ = _run(ctx, scs, [r])
        assert mixed[k][0] == rsh.RSH_OK and alone[0][0] == rsh.RSH_OK
        assert np.array_equal(mixed[k][1], alone[0][1]), f"hits of request {k}"
        assert np.array_equal(mixed[k][2], alone[0][2]), f"flags of request {k}"
        # the per-frame path with the same inputs gives the same records
        ctx.set_camera(r.camera)
        ctx.set_lights([{"position": tuple(r.lights[i].position)} for i in range(r.light_count)])
        ctx.render(scs[r.scene_index], r.width, r.height, r.depth)
        npix = r.width * r.height
        for b in range(r.depth):
            assert np.array_equal(ctx.frame_hits(b, npix), mixed[k][1][b * npix:(b + 1) * npix])
            nl = npix * r.light_count
            assert np.array_equal(ctx.frame_shadow(b, nl), mixed[k][2][b * nl:(b + 1) * nl])


def test_server_admission_and_cancel(setup):
    ctx, sd, scs = setup
    s = sd[0]
    cam = rsh.camera_look_at(s.eye, s.target, s.up, s.fov, 64, 64)
    big = _request(0, rsh.camera_look_at(s.eye, s.target, s.up, s.fov, 2048, 2048), 2048, 2048, 3, s.lights * 4)
    small = _request(0, cam, 64, 64, 1, s.lights)
    outs, stats = _run(ctx, scs, [big, small], budget=64 << 20)  # the big one can never fit
    assert outs[0][0] == rsh.RSH_ERR_OOM
    assert outs[1][0] == rsh.RSH_OK
    # cancellation before it runs
    L = rsh.lib()
    arr = (C.c_void_p * len(scs))(*[x.handle for x in scs])
    srv = C.c_void_p()
    rsh.check(L.rsh_server_create(ctx.handle, arr, len(scs), 1 << 30, 1, C.byref(srv)), "server")
    ids = []
    for _ in range(4):
        i = C.c_uint64()
        rsh.check(L.rsh_server_submit(srv, C.byref(small), C.byref(i)), "submit")
        ids.append(i.value)
    rsh.check(L.rsh_server_cancel(srv, ids[-1]), "cancel")
    sts = [L.rsh_server_wait(srv, i, 60_000, None, None, None) for i in ids]
    assert sts[:3] == [rsh.RSH_OK] * 3
    assert sts[3] in (rsh.RSH_ERR_INVALID, rsh.RSH_OK)  # cancelled unless it already finished
    bad = rsh.Request()
    bad.scene_index = 9
    assert L.rsh_server_submit(srv, C.byref(bad), None) == rsh.RSH_ERR_INVALID
    L.rsh_server_destroy(srv)
