"""Stage-level parity of the sm_103a kernels against the CPU oracle, through the C ABI.

Bar: bit-exact for keys, trimmed ids, run heads/bases/sizes, the stable sort permutation, the decompressed
ray order, hierarchy nodes (byte-identical), object-hierarchy spheres, traversal candidate sets and hit
records; end to end, every closest-hit record and shadow flag equals the brute-force oracle's.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu


def _lohi(s):
    p = s.positions[..., :3].reshape(-1, 3)
    return p.min(0), p.max(0)


@pytest.fixture(scope="module")
def ctx():
    c = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8)
    yield c
    c.destroy()


def random_rays(rng, n, lo=-1.2, hi=1.2):
    r = np.zeros(n, rsh.RAY_DTYPE)
    r["o"] = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["d"] = d.astype(np.float32)
    r["tmin"] = 0.01
    r["tmax"] = np.inf
    return r


# ---------------------------------------------------------------- raygen + hash
@pytest.mark.parametrize("W,H", [(64, 64), (100, 37), (8, 8)])
def test_raygen_primary_bitexact(W, H, cornell):
    cam = rsh.camera_look_at(cornell.eye, cornell.target, cornell.up, 60.0, W, H)
    n = ((W + 7) // 8) * ((H + 7) // 8) * 64
    d_rays = rsh.DeviceArray(n, rsh.RAY_DTYPE)
    d_pix = rsh.DeviceArray(n, np.uint32)
    rsh.check(rsh.lib().rsh_raygen_primary(C.byref(cam), W, H, d_rays.ptr, d_pix.ptr, None), "raygen")
    g = d_rays.numpy()
    o_rays, o_pix = oracle.raygen_primary(cam.as_array(), W, H)
    assert np.array_equal(d_pix.numpy(), o_pix)
    assert g.tobytes() == o_rays.tobytes()


@pytest.mark.parametrize("g,b,tag_bits,tag", [(5, 4, 0, 0), (9, 2, 0, 0), (1, 1, 2, 3), (6, 5, 2, 1), (2, 6, 3, 5)])
def test_hash_bitexact(g, b, tag_bits, tag):
    rng = np.random.default_rng(11 + g)
    rays = random_rays(rng, 200_000, -3, 3)
    # edge directions: axis-aligned, zero components, negative z, and an invalid ray
    ax = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [0.6, 0.8, 0], [0, 0.6, -0.8]],
                  np.float32)
    rays["d"][: len(ax)] = ax
    rays["o"][:4] = [[-2, -2, -2], [2, 2, 2], [0, 0, 0], [5, -7, 1]]
    rays["tmax"][10] = -1.0
    lo, hi = np.array([-2, -2, -2], np.float32), np.array([2, 2, 2], np.float32)
    hp = rsh.hash_params(lo, hi, g, b, tag_bits)
    d_rays = rsh.DeviceArray.from_numpy(rays)
    d_keys = rsh.DeviceArray(len(rays), np.uint32)
    rsh.check(rsh.lib().rsh_hash(d_rays.ptr, len(rays), C.byref(hp), tag, d_keys.ptr, None), "rsh_hash")
    ok = oracle.hash_rays(rays, lo, np.array(hp.scale[:], np.float32), g, b, tag)
    gk = d_keys.numpy()
    assert gk[10] == rsh.KEY_NONE
    assert np.array_equal(gk, ok)
    assert np.all(gk[gk != rsh.KEY_NONE] < (1 << hp.key_bits))


def _primary_surface(s, W, H):
    cam = rsh.camera_look_at(s.eye, s.target, s.up, s.fov, W, H)
    rays, pix = oracle.raygen_primary(cam.as_array(), W, H)
    hits = oracle.brute(s.positions, rays, False)
    spos, snrm = oracle.resolve(s.positions, s.normals, s.material_ids, rays, hits, pix, W * H)
    return cam, spos, snrm


def test_raygen_soft_shadow_bitexact(cornell):
    """16 soft-shadow rays per (pixel, light) from the reference's 4x4 grid around the light
    (RayTracer.cu:1550-1599): same rays and keys as the oracle; centre-invalid slots stay empty."""
    s = cornell
    W, H = 64, 48
    cam, spos, snrm = _primary_surface(s, W, H)
    lo, hi = _lohi(s)
    lights = s.lights + [{"position": (0.5, 0.2, 0.9)}, {"position": (-0.7, 0.9, -0.2)}]
    lp = np.array([l["position"] for l in lights], np.float32)
    hp = rsh.hash_params(lo, hi, 5, 4, 6)
    d_spos, d_snrm = rsh.DeviceArray.from_numpy(spos), rsh.DeviceArray.from_numpy(snrm)
    n = W * H * len(lights) * 16
    d_rays = rsh.DeviceArray(n, rsh.RAY_DTYPE, zero=True)
    d_keys = rsh.DeviceArray(n, np.uint32)
    larr = rsh.make_lights(lights)
    rsh.check(rsh.lib().rsh_raygen_soft_shadow(d_spos.ptr, d_snrm.ptr, W, H, larr, len(lights), 0.01, C.byref(hp),
                                               d_rays.ptr, d_keys.ptr, None), "soft shadow")
    orays, okeys = oracle.raygen_shadow(spos, snrm, W, H, lp, 0.01, lo, np.array(hp.scale[:]), 5, 4, samples=16)
    assert np.array_equal(d_keys.numpy(), okeys)
    v = okeys != rsh.KEY_NONE
    assert v.sum() > 1000
    assert d_rays.numpy()[v].tobytes() == orays[v].tobytes()
    # the 16 samples of a slot start at distinct points around the light and all end at the surface point
    o = orays.reshape(H, len(lights), 16, W)
    vv = v.reshape(H, len(lights), 16, W)
    y, l, x = np.argwhere(vv.all(axis=2))[0]
    starts = o["o"][y, l, :, x]
    assert len({tuple(q) for q in starts.round(6)}) == 16
    hc, _ = oracle.raygen_shadow(spos, snrm, W, H, lp, 0.01, lo, np.array(hp.scale[:]), 5, 4)
    centre = hc.reshape(H, len(lights), W)[y, l, x]
    end = starts + o["d"][y, l, :, x] * (o["tmax"][y, l, :, x] + 0.01)[:, None]  # o + d (tmax + eps) = p
    end_c = centre["o"] + centre["d"] * (centre["tmax"] + 0.01)
    assert np.allclose(end, end_c[None, :], atol=1e-4)
    with pytest.raises(rsh.RshError):  # 4 lights x 16 samples need 6 tag bits
        rsh.check(rsh.lib().rsh_raygen_soft_shadow(d_spos.ptr, d_snrm.ptr, W, H, larr, len(lights), 0.01,
                                                   C.byref(rsh.hash_params(lo, hi, 5, 4, 2)), d_rays.ptr,
                                                   d_keys.ptr, None), "soft shadow tag bits")


def test_raygen_refract_bitexact(ctx, cornell):
    """Refraction rays (CreateRefractionRays, RayTracer.cu:793-842): from the eye at eta = 1/1.52, from
    those rays again, and from the eye at eta = 1.52 where grazing view rays meet total internal reflection
    (no ray); same rays and keys as the oracle, and the refracted rays trace to the brute-force hits."""
    s = cornell
    W, H = 96, 80
    cam, spos, snrm = _primary_surface(s, W, H)
    lo, hi = _lohi(s)
    hp = rsh.hash_params(lo, hi, 5, 4, 0)
    d_spos, d_snrm = rsh.DeviceArray.from_numpy(spos), rsh.DeviceArray.from_numpy(snrm)
    m = W * H
    d_r = rsh.DeviceArray(m, rsh.RAY_DTYPE, zero=True)
    d_k = rsh.DeviceArray(m, np.uint32)
    eye = (C.c_float * 3)(*cam.eye)
    rsh.check(rsh.lib().rsh_raygen_refract(d_spos.ptr, d_snrm.ptr, None, eye, W, H, 0.01, 1.0 / 1.52, C.byref(hp),
                                           d_r.ptr, d_k.ptr, None), "refract")
    o_r, o_k = oracle.raygen_refract(spos, snrm, None, cam.as_array()[:3], W, H, 0.01, 1.0 / 1.52, lo,
                                     np.array(hp.scale[:]), 5, 4)
    assert np.array_equal(d_k.numpy(), o_k)
    v = o_k != rsh.KEY_NONE
    assert v.sum() > 1000
    assert d_r.numpy()[v].tobytes() == o_r[v].tobytes()
    d_r2 = rsh.DeviceArray(m, rsh.RAY_DTYPE, zero=True)
    rsh.check(rsh.lib().rsh_raygen_refract(d_spos.ptr, d_snrm.ptr, d_r.ptr, None, W, H, 0.01, 1.52, C.byref(hp),
                                           d_r2.ptr, d_k.ptr, None), "refract2")
    o_r2, o_k2 = oracle.raygen_refract(spos, snrm, o_r, None, W, H, 0.01, 1.52, lo, np.array(hp.scale[:]), 5, 4)
    assert np.array_equal(d_k.numpy(), o_k2)
    v2 = o_k2 != rsh.KEY_NONE
    assert d_r2.numpy()[v2].tobytes() == o_r2[v2].tobytes()
    d_r3 = rsh.DeviceArray(m, rsh.RAY_DTYPE, zero=True)
    rsh.check(rsh.lib().rsh_raygen_refract(d_spos.ptr, d_snrm.ptr, None, eye, W, H, 0.01, 1.52, C.byref(hp),
                                           d_r3.ptr, d_k.ptr, None), "refract3")
    o_r3, o_k3 = oracle.raygen_refract(spos, snrm, None, cam.as_array()[:3], W, H, 0.01, 1.52, lo,
                                       np.array(hp.scale[:]), 5, 4)
    assert np.array_equal(d_k.numpy(), o_k3)
    v3 = o_k3 != rsh.KEY_NONE
    assert d_r3.numpy()[v3].tobytes() == o_r3[v3].tobytes()
    assert (v & ~v3).sum() > 0 and v3.sum() > 0  # grazing view rays: total internal reflection, no ray
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    rays = o_r[v]
    assert np.array_equal(ctx.trace(sc, rays, False), oracle.brute(s.positions, rays, False))
    assert np.array_equal(ctx.trace(sc, rays, False, fused=True), oracle.brute(s.positions, rays, False))
    sc.destroy()
    with pytest.raises(rsh.RshError):
        rsh.check(rsh.lib().rsh_raygen_refract(d_spos.ptr, d_snrm.ptr, None, eye, W, H, 0.01, 0.0, C.byref(hp),
                                               d_r.ptr, d_k.ptr, None), "refract eta 0")


@pytest.mark.parametrize("jitter", [0.0, 1.0])
def test_raygen_secondary_bitexact(cornell, jitter):
    s = cornell
    W, H = 96, 80
    cam, spos, snrm = _primary_surface(s, W, H)
    lo, hi = _lohi(s)
    lights = s.lights + [{"position": (0.5, 0.2, 0.9)}, {"position": (-0.7, 0.9, -0.2)}]
    lp = np.array([l["position"] for l in lights], np.float32)
    hp = rsh.hash_params(lo, hi, 5, 4, 2)
    d_spos, d_snrm = rsh.DeviceArray.from_numpy(spos), rsh.DeviceArray.from_numpy(snrm)
    n = W * H * len(lights)
    d_rays = rsh.DeviceArray(n, rsh.RAY_DTYPE, zero=True)
    d_keys = rsh.DeviceArray(n, np.uint32)
    larr = rsh.make_lights(lights)
    rsh.check(rsh.lib().rsh_raygen_shadow(d_spos.ptr, d_snrm.ptr, W, H, larr, len(lights), 0.01, C.byref(hp),
                                          d_rays.ptr, d_keys.ptr, None), "shadow")
    orays, okeys = oracle.raygen_shadow(spos, snrm, W, H, lp, 0.01, lo, np.array(hp.scale[:]), 5, 4)
    gk = d_keys.numpy()
    assert np.array_equal(gk, okeys)
    v = okeys != rsh.KEY_NONE
    assert v.sum() > 1000
    assert d_rays.numpy()[v].tobytes() == orays[v].tobytes()
    # reflection from the camera, then a second bounce from those rays
    hp0 = rsh.hash_params(lo, hi, 5, 4, 0)
    m = W * H
    d_r = rsh.DeviceArray(m, rsh.RAY_DTYPE, zero=True)
    d_k = rsh.DeviceArray(m, np.uint32)
    eye = (C.c_float * 3)(*cam.eye)
    rsh.check(rsh.lib().rsh_raygen_reflect(d_spos.ptr, d_snrm.ptr, None, eye, W, H, 0.01, jitter, 77, 0,
                                           C.byref(hp0), d_r.ptr, d_k.ptr, None), "reflect")
    o_r, o_k = oracle.raygen_reflect(spos, snrm, None, cam.as_array()[:3], W, H, 0.01, jitter, 77, 0, lo,
                                     np.array(hp0.scale[:]), 5, 4)
    assert np.array_equal(d_k.numpy(), o_k)
    v = o_k != rsh.KEY_NONE
    assert d_r.numpy()[v].tobytes() == o_r[v].tobytes()
    d_r2 = rsh.DeviceArray(m, rsh.RAY_DTYPE, zero=True)
    rsh.check(rsh.lib().rsh_raygen_reflect(d_spos.ptr, d_snrm.ptr, d_r.ptr, None, W, H, 0.01, jitter, 77, 1,
                                           C.byref(hp0), d_r2.ptr, d_k.ptr, None), "reflect2")
    o_r2, o_k2 = oracle.raygen_reflect(spos, snrm, o_r, None, W, H, 0.01, jitter, 77, 1, lo,
                                       np.array(hp0.scale[:]), 5, 4)
    assert np.array_equal(d_k.numpy(), o_k2)
    v = o_k2 != rsh.KEY_NONE
    assert d_r2.numpy()[v].tobytes() == o_r2[v].tobytes()


def test_raygen_rays_at_16_byte_offset(cornell):
    """Ray arrays are written with one 32-byte store per ray when their base is 32-byte aligned; a base that
    is only 16-byte aligned takes the two 16-byte stores and must give the same bytes."""
    s = cornell
    W, H = 40, 32
    cam, spos, snrm = _primary_surface(s, W, H)
    lo, hi = _lohi(s)
    lp = np.array([l["position"] for l in s.lights], np.float32)
    hp = rsh.hash_params(lo, hi, 5, 4, 2)
    d_spos, d_snrm = rsh.DeviceArray.from_numpy(spos), rsh.DeviceArray.from_numpy(snrm)
    larr = rsh.make_lights(s.lights)
    eye = (C.c_float * 3)(*cam.eye)
    hp0 = rsh.hash_params(lo, hi, 5, 4, 0)
    for off in (0, 16):
        n = W * H * len(s.lights)
        buf = rsh.DeviceArray(32 * n + 32, np.uint8, zero=True)
        d_keys = rsh.DeviceArray(n, np.uint32)
        rsh.check(rsh.lib().rsh_raygen_shadow(d_spos.ptr, d_snrm.ptr, W, H, larr, len(s.lights), 0.01, C.byref(hp),
                                              buf.ptr + off, d_keys.ptr, None), "shadow")
        orays, okeys = oracle.raygen_shadow(spos, snrm, W, H, lp, 0.01, lo, np.array(hp.scale[:]), 5, 4)
        got = buf.numpy()[off:off + 32 * n].view(rsh.RAY_DTYPE)
        v = okeys != rsh.KEY_NONE
        assert v.sum() > 100
        assert np.array_equal(d_keys.numpy(), okeys)
        assert got[v].tobytes() == orays[v].tobytes()
        m = W * H
        rbuf = rsh.DeviceArray(32 * m + 32, np.uint8, zero=True)
        d_k = rsh.DeviceArray(m, np.uint32)
        rsh.check(rsh.lib().rsh_raygen_reflect(d_spos.ptr, d_snrm.ptr, None, eye, W, H, 0.01, 0.0, 77, 0,
                                               C.byref(hp0), rbuf.ptr + off, d_k.ptr, None), "reflect")
        o_r, o_k = oracle.raygen_reflect(spos, snrm, None, cam.as_array()[:3], W, H, 0.01, 0.0, 77, 0, lo,
                                         np.array(hp0.scale[:]), 5, 4)
        assert np.array_equal(d_k.numpy(), o_k)
        v = o_k != rsh.KEY_NONE
        assert v.sum() > 100
        assert rbuf.numpy()[off:off + 32 * m].view(rsh.RAY_DTYPE)[v].tobytes() == o_r[v].tobytes()


# ---------------------------------------------------------------- compress / sort / decompress
def _keys_cases():
    rng = np.random.default_rng(5)
    cases = {}
    cases["empty"] = np.zeros(0, np.uint32)
    cases["one"] = np.array([7], np.uint32)
    cases["one_none"] = np.array([rsh.KEY_NONE], np.uint32)
    cases["all_none"] = np.full(10000, rsh.KEY_NONE, np.uint32)
    cases["all_equal"] = np.full(20000, 42, np.uint32)
    runs = np.repeat(rng.integers(0, 1 << 20, 60000).astype(np.uint32), rng.integers(1, 40, 60000))
    runs[rng.random(len(runs)) < 0.3] = rsh.KEY_NONE
    cases["runs"] = runs
    cases["tile_edges"] = np.repeat(np.arange(3, dtype=np.uint32), [3071, 2, 3073])
    big = np.repeat(rng.integers(0, 1 << 25, 500000).astype(np.uint32), rng.integers(1, 30, 500000))
    big[rng.random(len(big)) < 0.45] = rsh.KEY_NONE
    cases["big"] = big
    return cases


@pytest.mark.parametrize("name", list(_keys_cases().keys()))
def test_compress_bitexact(ctx, name):
    keys = _keys_cases()[name]
    n = len(keys)
    d_keys = rsh.DeviceArray.from_numpy(keys) if n else rsh.DeviceArray(1, np.uint32)
    d_tr = rsh.DeviceArray(max(n, 1), np.uint32)
    d_ck = rsh.DeviceArray(n + 1, np.uint32)
    d_cb = rsh.DeviceArray(n + 1, np.uint32)
    d_cs = rsh.DeviceArray(n + 1, np.uint32)
    d_cnt = rsh.DeviceArray(2, np.uint32)
    rsh.check(rsh.lib().rsh_compress(ctx.handle, d_keys.ptr, n, d_tr.ptr, d_ck.ptr, d_cb.ptr, d_cs.ptr, d_cnt.ptr,
                                     None), "rsh_compress")
    ctx.check_device_errors()
    R, Cn = d_cnt.numpy()
    tr, ck, cb, cs = oracle.compress(keys)
    assert (R, Cn) == (len(tr), len(ck))
    assert np.array_equal(d_tr.numpy(R), tr)
    assert np.array_equal(d_ck.numpy(Cn), ck)
    assert np.array_equal(d_cb.numpy(Cn + 1), cb)
    assert np.array_equal(d_cs.numpy(Cn), cs)


@pytest.mark.parametrize("n,bits", [(0, 24), (1, 8), (3839, 16), (3840, 24), (3841, 31), (100_003, 27),
                                    (2_000_000, 32), (777_777, 9)])
def test_sort_pairs_stable_bitexact(ctx, n, bits):
    rng = np.random.default_rng(n + bits)
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, min(hi, 1 << 32), n, dtype=np.uint64).astype(np.uint32)
    if n > 100:
        keys[: n // 3] = keys[n // 3]  # many duplicates: stability matters
    vals = rng.permutation(n).astype(np.uint32)
    d_k = rsh.DeviceArray.from_numpy(keys) if n else rsh.DeviceArray(1, np.uint32)
    d_v = rsh.DeviceArray.from_numpy(vals) if n else rsh.DeviceArray(1, np.uint32)
    d_ko = rsh.DeviceArray(max(n, 1), np.uint32)
    d_vo = rsh.DeviceArray(max(n, 1), np.uint32)
    rsh.check(rsh.lib().rsh_sort_pairs(ctx.handle, d_k.ptr, d_v.ptr, d_ko.ptr, d_vo.ptr, n, None, bits, None), "sort")
    ctx.check_device_errors()
    ko, vo = oracle.sort_pairs(keys, vals, bits)
    assert np.array_equal(d_ko.numpy(n), ko)
    assert np.array_equal(d_vo.numpy(n), vo)
    # iota values (vals_in = NULL) and a device-side count smaller than n_max
    if n > 10:
        m = n // 2
        d_cnt = rsh.DeviceArray.from_numpy(np.array([m], np.uint32))
        rsh.check(rsh.lib().rsh_sort_pairs(ctx.handle, d_k.ptr, None, d_ko.ptr, d_vo.ptr, n, d_cnt.ptr, bits, None),
                  "sort")
        ko, vo = oracle.sort_pairs(keys[:m], None, bits)
        assert np.array_equal(d_ko.numpy(m), ko)
        assert np.array_equal(d_vo.numpy(m), vo)


@pytest.mark.parametrize("n", [5, 100_003])
def test_sort_pairs_keys_at_4_byte_offset(ctx, n):
    """The histogram pass loads 16 keys with four 16-byte loads when the key array is 16-byte aligned;
    a key array that starts 4 bytes into an allocation takes the 4-byte loads and sorts the same."""
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 20, n + 1, dtype=np.uint64).astype(np.uint32)
    keys[1: n // 2] = keys[n // 2]
    d_k = rsh.DeviceArray.from_numpy(keys)
    d_ko = rsh.DeviceArray(n, np.uint32)
    d_vo = rsh.DeviceArray(n, np.uint32)
    rsh.check(rsh.lib().rsh_sort_pairs(ctx.handle, d_k.ptr + 4, None, d_ko.ptr, d_vo.ptr, n, None, 20, None), "sort")
    ctx.check_device_errors()
    ko, vo = oracle.sort_pairs(keys[1:], None, 20)
    assert np.array_equal(d_ko.numpy(n), ko)
    assert np.array_equal(d_vo.numpy(n), vo)


@pytest.mark.parametrize("name", ["runs", "big", "all_equal", "one", "tile_edges"])
def test_decompress_bitexact(ctx, name):
    keys = _keys_cases()[name]
    n = len(keys)
    tr, ck, cb, cs = oracle.compress(keys)
    sk, sv = oracle.sort_pairs(ck, None, 32)
    want_k, want_i = oracle.decompress(sk, sv, cb, tr)
    d = {k: rsh.DeviceArray.from_numpy(v) for k, v in
         dict(sk=sk, sv=sv, cb=cb, tr=tr, cnt=np.array([len(tr), len(ck)], np.uint32)).items()}
    d_ok = rsh.DeviceArray(n, np.uint32)
    d_oi = rsh.DeviceArray(n, np.uint32)
    rsh.check(rsh.lib().rsh_decompress(ctx.handle, d["sk"].ptr, d["sv"].ptr, d["cb"].ptr, d["tr"].ptr, d["cnt"].ptr, n,
                                       d_ok.ptr, d_oi.ptr, None), "decompress")
    ctx.check_device_errors()
    R = len(tr)
    assert np.array_equal(d_oi.numpy(R), want_i)
    assert np.array_equal(d_ok.numpy(R), want_k)
    # the result is a permutation of the trimmed rays, stable within equal keys
    assert np.array_equal(np.sort(d_oi.numpy(R)), np.sort(tr))


# ---------------------------------------------------------------- hierarchy build
@pytest.mark.parametrize("P", [8, 16, 32])
def test_build_rsh_bitexact(P):
    rng = np.random.default_rng(P)
    n = 50_001
    rays = random_rays(rng, n)
    rays["tmax"][rng.random(n) < 0.05] = -1.0          # inactive rays inside packets
    rays["tmax"][rng.random(n) < 0.3] = rng.uniform(0.1, 5, 1).astype(np.float32)[0]
    ids = rng.permutation(n).astype(np.uint32)
    m = n - 1234                                        # device count below max_rays
    off = (C.c_uint32 * 4)()
    cap = rsh.lib().rsh_hierarchy_capacity(n, P, off)
    d_rays = rsh.DeviceArray.from_numpy(rays)
    d_ids = rsh.DeviceArray.from_numpy(ids)
    d_cnt = rsh.DeviceArray.from_numpy(np.array([m], np.uint32))
    d_nodes = rsh.DeviceArray(cap, rsh.NODE_DTYPE, zero=True)
    rsh.check(rsh.lib().rsh_build_rsh(d_rays.ptr, d_ids.ptr, n, d_cnt.ptr, P, d_nodes.ptr, None), "build")
    g = d_nodes.numpy()
    o, ooff = oracle.build_rsh(rays, ids, m, P, max_rays=n)
    assert list(off) == list(ooff)
    n0 = (m + P - 1) // P
    n1 = (n0 + 7) // 8
    n2 = (n1 + 7) // 8
    for lvl, cnt in enumerate((n0, n1, n2)):
        a = g[off[lvl]: off[lvl] + cnt]
        b = o[off[lvl]: off[lvl] + cnt]
        assert a.tobytes() == b.tobytes(), f"level {lvl}"
    # conservative: every active ray's origin is inside its leaf sphere and direction inside the cone
    leaves = g[:n0]
    k = np.arange(m)
    r = rays[ids[:m]]
    act = r["tmax"] > r["tmin"]
    lf = leaves[k // P]
    dist = np.linalg.norm(r["o"] - lf["c"], axis=1)
    assert np.all(dist[act] <= lf["radius"][act] * (1 + 1e-6) + 1e-6)
    cosang = np.sum(r["d"] * lf["axis"], 1)
    full = ~(lf["cos_spread"] > 0)
    assert np.all((cosang >= lf["cos_spread"])[act & ~full])


# ---------------------------------------------------------------- object hierarchy, traversal, intersection
@pytest.fixture(scope="module")
def soup_scene():
    return scenes.random_soup(60_000, np.random.default_rng(3))


@pytest.mark.parametrize("which", ["cornell", "soup"])
def test_object_hierarchy_bitexact(ctx, which, cornell, soup_scene):
    s = cornell if which == "cornell" else soup_scene
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    lo, hi = sc.bounds()
    lo2, hi2 = _lohi(s)
    assert np.array_equal(lo, lo2) and np.array_equal(hi, hi2)
    oh = oracle.ObjH(s.positions, 8, lo, hi)
    order, tris, sph = oh.arrays()
    assert np.array_equal(sc.order(), order)
    levels = sc.levels()
    assert [len(l) for l in levels] == oh.levels()
    assert len(levels[-1]) <= 8
    flat = np.concatenate([np.stack([l["c"][:, 0], l["c"][:, 1], l["c"][:, 2], l["radius"]], 1) for l in levels])
    assert flat.astype(np.float32).tobytes() == sph.tobytes()
    # explicit child ranges equal the oracle's; clusters hold <= 8 triangles, nodes <= 8 children
    kids = oh.kids()
    T = s.tri_count
    assert np.array_equal(np.append(levels[0]["first_tri"], T), kids[0])
    assert levels[0]["tri_count"].max() <= 8 and levels[0]["tri_count"].min() >= 1
    for l in range(1, len(levels)):
        assert np.array_equal(np.append(levels[l]["first_child"], len(levels[l - 1])), kids[l])
        assert levels[l]["child_count"].max() <= 8 and levels[l]["child_count"].min() >= 1
        # a node's triangles are exactly its children's
        fc, cc = levels[l]["first_child"], levels[l]["child_count"]
        below = levels[l - 1]
        assert np.array_equal(levels[l]["first_tri"], below["first_tri"][fc])
        last = fc + cc - 1
        assert np.array_equal(levels[l]["first_tri"] + levels[l]["tri_count"],
                              below["first_tri"][last] + below["tri_count"][last])
    # every vertex lies inside its cluster sphere
    cl = np.repeat(np.arange(len(levels[0])), levels[0]["tri_count"])
    v = tris.reshape(T, 3, 4)[:, :, :3]
    c = flat[cl, :3]
    d = np.linalg.norm(v - c[:, None, :], axis=2).max(1)
    assert np.all(d <= flat[cl, 3])
    sc.destroy()


@pytest.mark.parametrize("which", ["cornell", "soup", "one", "six", "architecture"])
def test_box_tree_bitexact(ctx, which, cornell, soup_scene):
    """The single-ray box tree (PLOC clustering collapsed to 8-wide nodes) built on the GPU equals the
    oracle's restatement slot for slot, with its triangles in the same depth-first order; a scene of one
    triangle, or of no more triangles than a cluster holds, is a single cluster under the root."""
    from rsh import scenes

    if which == "cornell":
        s = cornell
    elif which == "soup":
        s = soup_scene
    elif which == "architecture":
        s = scenes.architecture(grid=6, segments=12, rings=3)
    else:
        n = 1 if which == "one" else 6
        s = scenes.SceneData(name=which, positions=cornell.positions[:n].copy(), normals=cornell.normals[:n].copy(),
                             material_ids=cornell.material_ids[:n].copy(), materials=cornell.materials)
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    lo, hi = sc.bounds()
    oh = oracle.ObjH(s.positions, ctx.config.cluster_size, lo, hi)
    root, boxes, tris = sc.box_tree()
    oroot, oboxes, otris = oh.box_tree()
    assert root == oroot and boxes.shape == oboxes.shape
    assert boxes[1:].tobytes() == oboxes[1:].tobytes()
    assert tris.tobytes() == otris.tobytes()
    # every triangle in exactly one cluster, every cluster within the cluster size
    w = boxes.view(np.uint32)
    cl = (w[:, 7] >> 31) == 1
    cnt = w[cl, 7] & 0x7FFFFFFF
    assert cnt.sum() == s.tri_count and cnt.max() <= ctx.config.cluster_size
    covered = np.sort(np.concatenate([np.arange(a, a + c) for a, c in zip(w[cl, 3], cnt)]))
    assert np.array_equal(covered, np.arange(s.tri_count))
    if which in ("one", "six"):
        assert root >> 27 == 1 and ((root >> 24) & 7) == 0 and cl.sum() == 1
    sc.destroy()


def _stage_pipeline(ctx, sc, s, rays, any_hit, P=8, cap=1 << 25):
    """Runs hash -> compress -> sort -> decompress -> build -> traverse -> intersect stage by stage on the
    GPU and the same chain on the oracle; returns both."""
    n = len(rays)
    lo, hi = sc.bounds()
    hp = rsh.hash_params(lo, hi, ctx.config.grid_bits, ctx.config.dir_log2, 0)
    L = rsh.lib()
    d_rays = rsh.DeviceArray.from_numpy(rays)
    d_keys = rsh.DeviceArray(n, np.uint32)
    rsh.check(L.rsh_hash(d_rays.ptr, n, C.byref(hp), 0, d_keys.ptr, None), "hash")
    d_tr, d_ck, d_cb = rsh.DeviceArray(n, np.uint32), rsh.DeviceArray(n + 1, np.uint32), rsh.DeviceArray(n + 1, np.uint32)
    d_cnt = rsh.DeviceArray(2, np.uint32)
    rsh.check(L.rsh_compress(ctx.handle, d_keys.ptr, n, d_tr.ptr, d_ck.ptr, d_cb.ptr, None, d_cnt.ptr, None), "cmp")
    d_sk, d_sv = rsh.DeviceArray(n, np.uint32), rsh.DeviceArray(n, np.uint32)
    rsh.check(L.rsh_sort_pairs(ctx.handle, d_ck.ptr, None, d_sk.ptr, d_sv.ptr, n, d_cnt.ptr + 4, hp.key_bits, None),
              "sort")
    d_sortk, d_ids = rsh.DeviceArray(n, np.uint32), rsh.DeviceArray(n, np.uint32)
    rsh.check(L.rsh_decompress(ctx.handle, d_sk.ptr, d_sv.ptr, d_cb.ptr, d_tr.ptr, d_cnt.ptr, n, d_sortk.ptr, d_ids.ptr,
                               None), "dec")
    off = (C.c_uint32 * 4)()
    capn = L.rsh_hierarchy_capacity(n, P, off)
    d_nodes = rsh.DeviceArray(capn, rsh.NODE_DTYPE, zero=True)
    rsh.check(L.rsh_build_rsh(d_rays.ptr, d_ids.ptr, n, d_cnt.ptr, P, d_nodes.ptr, None), "build")
    d_cand = rsh.DeviceArray(cap, np.uint64)
    d_cc = rsh.DeviceArray(1, np.uint64)
    rsh.check(L.rsh_traverse(ctx.handle, sc.handle, d_nodes.ptr, n, d_cnt.ptr, P, d_cand.ptr, cap, d_cc.ptr, None),
              "traverse")
    ncand = int(d_cc.numpy()[0])
    if any_hit:
        d_out = rsh.DeviceArray(n, np.uint32, zero=True)
        rsh.check(L.rsh_intersect_any(sc.handle, d_rays.ptr, d_ids.ptr, n, d_cnt.ptr, P, d_cand.ptr, d_cc.ptr,
                                      d_out.ptr, None), "any")
    else:
        d_out = rsh.DeviceArray(n, np.uint64)
        d_out.fill_bytes(0xFF)
        rsh.check(L.rsh_intersect_closest(sc.handle, d_rays.ptr, d_ids.ptr, n, d_cnt.ptr, P, d_cand.ptr, d_cc.ptr,
                                          d_out.ptr, None), "closest")
    ctx.check_device_errors()
    R = int(d_cnt.numpy()[0])
    gpu = dict(keys=d_keys.numpy(), ids=d_ids.numpy(R), nodes=d_nodes.numpy(), cand=np.sort(d_cand.numpy(ncand)),
               out=d_out.numpy(), R=R)
    # oracle chain
    okeys = oracle.hash_rays(rays, lo, np.array(hp.scale[:]), hp.grid_bits, hp.dir_log2, 0)
    tr, ck, cb, cs = oracle.compress(okeys)
    sk, sv = oracle.sort_pairs(ck, None, hp.key_bits)
    _, oids = oracle.decompress(sk, sv, cb, tr)
    onodes, _ = oracle.build_rsh(rays, oids, len(oids), P, max_rays=n)
    oh = oracle.ObjH(s.positions, ctx.config.cluster_size, lo, hi)
    ocand, _ = oh.traverse(onodes, len(oids), P, max_rays=n)
    oout = oh.intersect(rays, oids, len(oids), P, ocand, any_hit, n)
    orc = dict(keys=okeys, ids=oids, nodes=onodes, cand=ocand, out=oout, R=len(oids))
    return gpu, orc


@pytest.mark.parametrize("any_hit", [False, True])
@pytest.mark.parametrize("which", ["cornell", "soup"])
def test_pipeline_stages_bitexact_and_vs_brute(ctx, which, any_hit, cornell, soup_scene):
    s = cornell if which == "cornell" else soup_scene
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    rng = np.random.default_rng(21)
    rays = scenes.surface_rays(s, 30_000 if which == "cornell" else 8_000, rng)
    if any_hit:
        rays["tmax"] = rng.uniform(0.05, 3.0, len(rays)).astype(np.float32)
    rays["tmax"][:50] = -1.0  # a few invalid rays
    g, o = _stage_pipeline(ctx, sc, s, rays, any_hit)
    assert np.array_equal(g["keys"], o["keys"])
    assert g["R"] == o["R"] == len(rays) - 50
    assert len(g["cand"]) < (1 << 25)
    assert np.array_equal(g["ids"], o["ids"])
    assert g["nodes"][: len(o["nodes"])].tobytes() == o["nodes"].tobytes()
    assert np.array_equal(g["cand"], o["cand"])
    assert np.array_equal(g["out"], o["out"])
    bf = oracle.brute(s.positions, rays, any_hit)
    assert np.array_equal(g["out"], bf)
    sc.destroy()


@pytest.mark.parametrize("ray_level", [0, 2, 15])
@pytest.mark.parametrize("any_hit", [False, True])
def test_trace_rays_vs_brute(ctx, any_hit, soup_scene, ray_level):
    s = soup_scene
    ctx.set_config(ray_level=ray_level, plain_ray_level=ray_level)
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials)
    rng = np.random.default_rng(8)
    rays = scenes.surface_rays(s, 100_000, rng)
    if any_hit:
        rays["tmax"] = rng.uniform(0.05, 20.0, len(rays)).astype(np.float32)
    out = ctx.trace(sc, rays, any_hit)
    bf = oracle.brute(s.positions, rays, any_hit)
    assert np.array_equal(out, bf)
    ctx.set_config(ray_level=6, plain_ray_level=4)
    sc.destroy()


@pytest.mark.parametrize("ray_level", [0, 3])
def test_overflow_resume_matches_brute(cornell, ray_level):
    c = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=8, candidate_capacity=5000,
                    ray_level=ray_level, plain_ray_level=ray_level)
    s = cornell
    sc = c.scene(s.positions, s.normals, s.material_ids, s.materials)
    rays = scenes.surface_rays(s, 20_000, np.random.default_rng(4))
    out = c.trace(sc, rays, False)
    assert np.array_equal(out, oracle.brute(s.positions, rays, False))
    sc.destroy()
    c.destroy()


def test_watertight_shared_edges(ctx):
    """Rays through shared edges and vertices of a closed mesh must hit (watertightness)."""
    sv, sf = scenes.icosphere(2)
    pos, nrm = scenes._pack(sv, sf, sv)
    sc = ctx.scene(pos, nrm)
    # aim from outside at edge midpoints and at vertices
    edges = np.concatenate([sf[:, [0, 1]], sf[:, [1, 2]], sf[:, [2, 0]]])
    targets = np.concatenate([(sv[edges[:, 0]] + sv[edges[:, 1]]) * 0.5, sv]).astype(np.float32)
    rng = np.random.default_rng(2)
    o = (targets * 3.0 + rng.normal(0, 0.2, targets.shape)).astype(np.float32)
    d = targets - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(len(o), rsh.RAY_DTYPE)
    rays["o"] = o
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.inf
    out = ctx.trace(sc, rays, False)
    bf = oracle.brute(pos, rays, False)
    assert np.array_equal(out, bf)
    assert np.all(out != rsh.HIT_NONE), "a ray through an edge or vertex slipped through the mesh"
    sc.destroy()
