"""Batched form: fused persistent traversal + intersection, segmented hash/sort over many scenes, CUDA-graph
replay and the autotuner, all checked against the brute-force oracle through the C ABI."""
import ctypes as C

import numpy as np
import pytest

import oracle
import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8)
    yield c
    c.destroy()


@pytest.mark.parametrize("ray_level", [0, 2, 15])
@pytest.mark.parametrize("P", [8, 16, 32])
@pytest.mark.parametrize("any_hit", [False, True])
def test_fused_vs_brute(P, any_hit, ray_level):
    # fewer CTAs per SM than fit (1 and 3) for some points: the persistent launches cover every unit anyway
    c = rsh.Context(grid_bits=5, dir_log2=4, packet_size=P, cluster_size=8, ray_level=ray_level,
                    fused_blocks={8: 0, 16: 1, 32: 3}[P])
    s = scenes.random_soup(40_000, np.random.default_rng(P))
    sc = c.scene(s.positions, s.normals, s.material_ids, s.materials)
    rng = np.random.default_rng(100 + P)
    rays = scenes.surface_rays(s, 70_001, rng)
    if any_hit:
        rays["tmax"] = rng.uniform(0.05, 15.0, len(rays)).astype(np.float32)
    rays["tmax"][::97] = -1.0
    out = c.trace(sc, rays, any_hit, fused=True)
    c.check_device_errors()
    bf = oracle.brute(s.positions, rays, any_hit)
    assert np.array_equal(out, bf)
    sc.destroy()
    c.destroy()


def test_fused_cornell_closest_and_ties(ctx, cornell):
    s = cornell
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    rays = scenes.surface_rays(s, 50_000, np.random.default_rng(9))
    out = ctx.trace(sc, rays, False, fused=True)
    assert np.array_equal(out, oracle.brute(s.positions, rays, False))
    sc.destroy()


@pytest.mark.parametrize("flags", [0, rsh.FLAG_NO_COMPRESS])  # runs of equal keys, or the slots sorted as they are
def test_batch_segments_many_scenes(ctx, flags):
    ctx.set_config(flags=flags)
    rng = np.random.default_rng(77)
    sd = [scenes.random_soup(int(t), np.random.default_rng(200 + i)) for i, t in enumerate([12_000, 35_000, 80_000])]
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in sd]
    sizes = [5_000, 1, 0, 40_000, 4_099, 17_000, 64, 3]
    which = [0, 1, 2, 2, 1, 0, 2, 1]
    anyh = [False, True, False, True, False, True, False, True]
    host_rays, dev = [], []
    segs = (rsh.BatchSegment * len(sizes))()
    for i, (n, w, a) in enumerate(zip(sizes, which, anyh)):
        r = scenes.surface_rays(sd[w], max(n, 1), rng)[:n]
        if a:
            r["tmax"] = rng.uniform(0.1, 10.0, n).astype(np.float32)
        host_rays.append(r)
        dr = rsh.DeviceArray.from_numpy(r) if n else rsh.DeviceArray(1, rsh.RAY_DTYPE)
        out = rsh.DeviceArray(max(n, 1), np.uint32 if a else np.uint64)
        dev.append((dr, out))
        segs[i].scene = scs[w].handle
        segs[i].rays = dr.ptr
        segs[i].n = n
        segs[i].any_hit = int(a)
        segs[i].hits = None if a else out.ptr
        segs[i].flags = out.ptr if a else None
    rsh.check(rsh.lib().rsh_batch_trace(ctx.handle, segs, len(sizes), None), "batch")
    ctx.check_device_errors()
    for i, (n, w, a) in enumerate(zip(sizes, which, anyh)):
        if n == 0:
            continue
        got = dev[i][1].numpy(n)
        want = oracle.brute(sd[w].positions, host_rays[i], a)
        bad = np.nonzero(got != want)[0]
        assert len(bad) == 0, (f"segment {i}: {len(bad)} of {n} differ, first at {bad[:8].tolist()}, "
                               f"got {got[bad[:4]].tolist()}, want {want[bad[:4]].tolist()}")
    # graph capture + replay gives the same results
    st = C.c_void_p()
    rsh.check(rsh.lib().rsh_stream_create(C.byref(st)), "stream")
    g = C.c_void_p()
    rsh.check(rsh.lib().rsh_batch_graph_create(ctx.handle, segs, len(sizes), st, C.byref(g)), "graph")
    for i, (n, w, a) in enumerate(zip(sizes, which, anyh)):
        if n:
            dev[i][1].fill_bytes(0x5A)
    rsh.check(rsh.lib().rsh_batch_graph_launch(g, st), "launch")
    rsh.check(rsh.lib().rsh_stream_synchronize(st), "sync")
    for i, (n, w, a) in enumerate(zip(sizes, which, anyh)):
        if n == 0:
            continue
        assert np.array_equal(dev[i][1].numpy(n), oracle.brute(sd[w].positions, host_rays[i], a)), f"graph seg {i}"
    rsh.lib().rsh_batch_graph_destroy(g)
    rsh.lib().rsh_stream_destroy(st)
    for sc in scs:
        sc.destroy()
    ctx.set_config(flags=0)


def test_autotune_picks_a_valid_config(ctx):
    s = scenes.random_soup(20_000, np.random.default_rng(5))
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    rays = scenes.surface_rays(s, 30_000, np.random.default_rng(6))
    dr = rsh.DeviceArray.from_numpy(rays)
    out = rsh.DeviceArray(len(rays), np.uint64)
    segs = (rsh.BatchSegment * 1)()
    segs[0].scene, segs[0].rays, segs[0].n, segs[0].any_hit, segs[0].hits = sc.handle, dr.ptr, len(rays), 0, out.ptr
    gb = (C.c_uint32 * 2)(4, 6)
    db = (C.c_uint32 * 2)(3, 5)
    ps = (C.c_uint32 * 2)(8, 16)
    best = rsh.Config()
    rsh.check(rsh.lib().rsh_autotune(ctx.handle, segs, 1, gb, 2, db, 2, ps, 2, None, C.byref(best)), "autotune")
    assert best.grid_bits in (4, 6) and best.dir_log2 in (3, 5) and best.packet_size in (8, 16)
    rsh.check(rsh.lib().rsh_batch_trace(ctx.handle, segs, 1, None), "batch")
    assert np.array_equal(out.numpy(), oracle.brute(s.positions, rays, False))
    ctx.set_config(grid_bits=5, dir_log2=4, packet_size=8)
    sc.destroy()


@pytest.mark.parametrize("flags", [0, rsh.FLAG_NO_COMPRESS])
def test_many_segments_drop_low_hash_bits(flags):
    """300 segments need 9 tag bits: with a 27-bit hash (grid 5, dir 6) the key would need 36 bits, so the
    batch drops the hash's 5 lowest bits (ordering only); every segment's results still equal brute force."""
    ctx = rsh.Context(grid_bits=5, dir_log2=6, packet_size=8, cluster_size=6, flags=flags)
    rng = np.random.default_rng(31)
    sd = [scenes.random_soup(int(t), np.random.default_rng(300 + i)) for i, t in enumerate([4_000, 9_000, 15_000])]
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in sd]
    nseg = 300
    sizes = rng.integers(0, 700, nseg)
    which = rng.integers(0, 3, nseg)
    anyh = rng.random(nseg) < 0.5
    segs = (rsh.BatchSegment * nseg)()
    keep = []
    for i in range(nseg):
        n = int(sizes[i])
        r = scenes.surface_rays(sd[which[i]], max(n, 1), rng)[:n]
        dr = rsh.DeviceArray.from_numpy(r) if n else rsh.DeviceArray(1, rsh.RAY_DTYPE)
        out = rsh.DeviceArray(max(n, 1), np.uint32 if anyh[i] else np.uint64)
        keep.append((r, dr, out))
        segs[i].scene = scs[which[i]].handle
        segs[i].rays = dr.ptr
        segs[i].n = n
        segs[i].any_hit = int(anyh[i])
        segs[i].hits = None if anyh[i] else out.ptr
        segs[i].flags = out.ptr if anyh[i] else None
    rsh.check(rsh.lib().rsh_batch_trace(ctx.handle, segs, nseg, None), "batch")
    ctx.check_device_errors()
    for i in range(nseg):
        r, _, out = keep[i]
        if len(r):
            assert np.array_equal(out.numpy(len(r)), oracle.brute(sd[which[i]].positions, r, bool(anyh[i]))), i
    for sc in scs:
        sc.destroy()
    ctx.destroy()


def _segments(ctx, sd, scs, sizes, which, anyh, rng):
    segs = (rsh.BatchSegment * len(sizes))()
    keep = []
    for i, (n, w, a) in enumerate(zip(sizes, which, anyh)):
        r = scenes.surface_rays(sd[w], n, rng)
        if a:
            r["tmax"] = rng.uniform(0.1, 10.0, n).astype(np.float32)
        dr = rsh.DeviceArray.from_numpy(r)
        out = rsh.DeviceArray(n, np.uint32 if a else np.uint64)
        keep.append((r, dr, out))
        segs[i].scene = scs[w].handle
        segs[i].rays = dr.ptr
        segs[i].n = n
        segs[i].any_hit = int(a)
        segs[i].hits = None if a else out.ptr
        segs[i].flags = out.ptr if a else None
    return segs, keep


def _check_segments(sd, which, anyh, keep):
    for i, (r, _, out) in enumerate(keep):
        assert np.array_equal(out.numpy(len(r)), oracle.brute(sd[which[i]].positions, r, bool(anyh[i]))), i


def test_scene_tuning_mixed_widths_and_levels():
    """Scenes of one batch with their own hash widths (8 and 30 bits) and switch levels (0 and 15): the tag
    sits above the widest hash, each segment keeps its own level, and results equal brute force."""
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=6)
    sd = [scenes.random_soup(t, np.random.default_rng(400 + i)) for i, t in enumerate([8_000, 30_000])]
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in sd]
    scs[0].set_tuning(grid_bits=8, dir_log2=3, ray_level=0)
    scs[1].set_tuning(grid_bits=2, dir_log2=1, ray_level=15)
    assert scs[0].tuning() == {"grid_bits": 8, "dir_log2": 3, "ray_level": 0}
    assert scs[1].tuning()["ray_level"] == 15
    which, anyh = [0, 1, 0, 1, 1], [False, False, True, True, False]
    segs, keep = _segments(ctx, sd, scs, [9_000, 12_001, 5_000, 7_000, 64], which, anyh, np.random.default_rng(41))
    rsh.check(rsh.lib().rsh_batch_trace(ctx.handle, segs, len(which), None), "batch")
    ctx.check_device_errors()
    _check_segments(sd, which, anyh, keep)
    for bad in ({"grid_bits": 11}, {"dir_log2": 0}, {"ray_level": 16}):
        with pytest.raises(rsh.RshError):
            scs[0].set_tuning(**bad)
    scs[0].set_tuning()  # back to the context's
    assert scs[0].tuning() == {"grid_bits": rsh.TUNE_DEFAULT, "dir_log2": rsh.TUNE_DEFAULT,
                               "ray_level": rsh.TUNE_DEFAULT}
    for sc in scs:
        sc.destroy()
    ctx.destroy()


def test_autotune_scenes_per_scene_choice():
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=6)
    sd = [scenes.random_soup(t, np.random.default_rng(500 + i)) for i, t in enumerate([6_000, 25_000, 60_000])]
    scs = [ctx.scene(s.positions, s.normals, s.material_ids, s.materials) for s in sd]
    which, anyh = [0, 1, 2, 2, 1, 0], [False, True, False, True, False, True]
    segs, keep = _segments(ctx, sd, scs, [20_000, 30_000, 50_000, 20_000, 4_000, 9_000], which, anyh,
                           np.random.default_rng(51))
    best_ms, untuned_ms = ctx.autotune_scenes(segs, len(which), grid_bits=(4, 6), dir_log2=(3, 5),
                                              ray_levels=(2, 4), packet_sizes=(8, 16), fused_blocks=(2, 4))
    assert best_ms > 0 and untuned_ms > 0
    assert ctx.config.packet_size in (8, 16) and ctx.config.fused_blocks in (0, 2, 4)
    for sc in scs:
        t = sc.tuning()
        # a tuned value is one of the swept points or the context's own (where the descent started), or the
        # scene keeps no tuning at all (the search found nothing faster on the whole batch)
        D = rsh.TUNE_DEFAULT
        assert t["grid_bits"] in (4, 5, 6, D) and t["dir_log2"] in (3, 4, 5, D)
        assert t["ray_level"] in (2, 4, 15, rsh.default_config().ray_level, D)  # 15: every scene rays-only
    for _, _, out in keep:
        out.fill_bytes(0x5A)
    rsh.check(rsh.lib().rsh_batch_trace(ctx.handle, segs, len(which), None), "batch")
    ctx.check_device_errors()
    _check_segments(sd, which, anyh, keep)
    for sc in scs:
        sc.destroy()
    ctx.destroy()


@pytest.mark.parametrize("ray_level", [2, 15])  # the packet kernel and the rays-only kernel
def test_empty_scene_segments_miss(ray_level):
    """A scene without triangles in a batch: its segments report no hit and no occlusion; the other
    segments of the same batch still equal brute force."""
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=6, ray_level=ray_level)
    s = scenes.random_soup(20_000, np.random.default_rng(61))
    full = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    empty = ctx.scene(np.zeros((0, 3, 4), np.float32))
    rng = np.random.default_rng(62)
    rays = [scenes.surface_rays(s, n, rng) for n in (9_000, 5_000, 7_000, 3_000)]
    which = [full, empty, full, empty]
    anyh = [False, False, True, True]
    segs = (rsh.BatchSegment * 4)()
    keep = []
    for i, (r, sc, a) in enumerate(zip(rays, which, anyh)):
        dr = rsh.DeviceArray.from_numpy(r)
        out = rsh.DeviceArray(len(r), np.uint32 if a else np.uint64)
        out.fill_bytes(0x5A)  # the batch must overwrite every output
        keep.append((dr, out))
        segs[i].scene, segs[i].rays, segs[i].n, segs[i].any_hit = sc.handle, dr.ptr, len(r), int(a)
        segs[i].hits = None if a else out.ptr
        segs[i].flags = out.ptr if a else None
    rsh.check(rsh.lib().rsh_batch_trace(ctx.handle, segs, 4, None), "batch")
    ctx.check_device_errors()
    for i, (r, sc, a) in enumerate(zip(rays, which, anyh)):
        got = keep[i][1].numpy(len(r))
        if sc is empty:
            assert np.all(got == (0 if a else rsh.HIT_NONE)), i
        else:
            assert np.array_equal(got, oracle.brute(s.positions, r, a)), i
    full.destroy()
    empty.destroy()
    ctx.destroy()


@pytest.mark.parametrize("any_hit", [False, True])
def test_shared_launch_ends_change_no_result(any_hit):
    """At the end of a rays-only launch a drained warp's idle lanes take subtrees of its rays still in flight
    (the default); RSH_FLAG_SEQUENTIAL_RAYS keeps every ray on one lane. Both give the brute-force records and
    flags, and the sequential counts equal the oracle's box descent of the same rays, test for test."""
    c = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8)
    s = scenes.random_soup(60_000, np.random.default_rng(31))
    sc = c.scene(s.positions, s.normals, s.material_ids, s.materials)
    rng = np.random.default_rng(32)
    rays = scenes.surface_rays(s, 90_001, rng)
    if any_hit:
        rays["tmax"] = rng.uniform(0.05, 40.0, len(rays)).astype(np.float32)
    rays["tmax"][::101] = -1.0
    bf = oracle.brute(s.positions, rays, any_hit)
    shared = c.trace(sc, rays, any_hit, fused=True)
    n_shared = c.test_counters(reset=True)
    c.set_config(flags=rsh.FLAG_SEQUENTIAL_RAYS)
    seq = c.trace(sc, rays, any_hit, fused=True)
    n_seq = c.test_counters(reset=True)
    c.check_device_errors()
    assert np.array_equal(shared, bf) and np.array_equal(seq, bf)
    lo, hi = sc.bounds()
    oh = oracle.ObjH(s.positions, c.config.cluster_size, lo, hi)
    _, n_orc = oh.trace_box(rays[rays["tmax"] > rays["tmin"]], any_hit)
    assert tuple(n_seq) == tuple(int(x) for x in n_orc)
    assert abs(n_shared[0] / n_seq[0] - 1.0) < 0.10
    sc.destroy()
    c.destroy()
