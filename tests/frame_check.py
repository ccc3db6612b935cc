"""Stage-by-stage check of one rendered frame against the oracle (shared by the GPU frame tests).

Every buffer of the frame is recomputed by the oracle from the GPU's previous stage and compared bit for bit:
the primary rays, each bounce's shadow and reflection rays, and the surface buffers resolved from the hits.
Hit records and shadow flags are compared with the oracle's brute force over every triangle (the
CUDA-Naive-Engine semantics, NE/RayTracer.cu:276-291 any hit, :344-360 closest hit): for every ray
(sample=None) or for a seeded sample of `sample` rays per ray type per bounce (the full-size frames, whose
whole brute force would take hours on the host). The image must equal the oracle's shading of the same
buffers within 2/255 per channel (host and device powf / log2f may differ by an ulp).
"""
from __future__ import annotations

import numpy as np

import oracle
import rsh


class BruteCache:
    """Brute-force results per (ray type, bounce), reused when the next frame's sampled rays are the same
    bytes (the plain and batched forms of one frame generate identical rays)."""

    def __init__(self):
        self.store = {}

    def get(self, key, positions, rays, any_hit):
        raw = rays.tobytes()
        hit = self.store.get(key)
        if hit is not None and hit[0] == raw:
            return hit[1]
        res = oracle.brute(positions, rays, any_hit)
        self.store[key] = (raw, res)
        return res


def _pick(valid_idx, sample, rng):
    if sample is None or len(valid_idx) <= sample:
        return valid_idx
    return np.sort(rng.choice(valid_idx, sample, replace=False))


def check_frame(ctx, s, sc, W, H, depth, jitter, samples=1, sample=None, seed=0, cache=None, image=True):
    """Renders (W, H, depth) with ctx's configuration and checks it; returns (frame stats, rays checked by
    brute force per ray type)."""
    rng = np.random.default_rng(seed)
    cache = cache if cache is not None else BruteCache()
    lights = s.lights
    L = len(lights)
    LS = L * samples
    cam = rsh.camera_look_at(s.eye, s.target, s.up, s.fov, W, H)
    ctx.set_camera(cam)
    ctx.set_lights(lights)
    rgba = rsh.DeviceArray(W * H, np.uint32)
    ctx.render(sc, W, H, depth, rgba)
    ctx.check_device_errors()
    st = ctx.stats()
    npix = W * H
    lo, hi = sc.bounds()
    g, b = ctx.config.grid_bits, ctx.config.dir_log2
    scale = oracle.hash_scale(lo, hi, g)
    checked = {"primary": 0, "shadow": 0, "reflection": 0}
    # primary rays (8x8 tile order) and their closest hits
    prays, pix = oracle.raygen_primary(cam.as_array(), W, H)
    assert ctx.frame_rays(-1, False, len(prays)).tobytes() == prays.tobytes()
    ph = ctx.frame_hits(-1, npix)
    valid = np.nonzero(pix != 0xFFFFFFFF)[0]
    idx = _pick(valid, sample, rng)
    bf = cache.get(("primary", -1), s.positions, prays[idx], False)
    assert np.array_equal(ph[pix[idx]], bf), f"primary hits: {(ph[pix[idx]] != bf).sum()} of {len(idx)} differ"
    checked["primary"] += len(idx)
    gh = np.full(len(prays), oracle.HIT_NONE, np.uint64)
    gh[valid] = ph[pix[valid]]
    spos, snrm = ctx.frame_surface(-1, npix)
    ospos, osnrm = oracle.resolve(s.positions, s.normals, s.material_ids, prays, gh, pix, npix)
    assert spos.tobytes() == ospos.tobytes() and snrm.tobytes() == osnrm.tobytes()
    prev = None
    lp = np.array([l["position"] for l in lights], np.float32)
    nshadow = nrefl = 0
    accum = np.zeros((npix, 4), np.float32)
    eye = cam.as_array()[:3]
    for bnc in range(depth):
        # shadow rays from the GPU's surface buffer, then their flags
        srays = ctx.frame_rays(bnc, True, npix * LS)
        orays, okeys = oracle.raygen_shadow(spos, snrm, W, H, lp, ctx.config.epsilon, lo, scale, g, b, samples)
        v = okeys != oracle.KEY_NONE
        nshadow += int(v.sum())
        assert srays[v].tobytes() == orays[v].tobytes(), f"bounce {bnc} shadow rays"
        sflags = ctx.frame_shadow(bnc, npix * LS)
        assert np.all(sflags[~v] == 0)
        idx = _pick(np.nonzero(v)[0], sample, rng)
        bf = cache.get(("shadow", bnc), s.positions, orays[idx], True)
        assert np.array_equal(sflags[idx], bf), f"bounce {bnc} shadow flags: {(sflags[idx] != bf).sum()} differ"
        checked["shadow"] += len(idx)
        if image:
            oracle.shade(spos, snrm, s.materials, sflags, accum, W, H, lights, eye, bnc, prev, samples)
        # reflection rays, their closest hits and the next surface buffer
        rrays = ctx.frame_rays(bnc, False, npix)
        o_r, o_k = oracle.raygen_reflect(spos, snrm, prev, eye if prev is None else None, W, H,
                                         ctx.config.epsilon, jitter, ctx.config.seed, bnc, lo, scale, g, b)
        v = o_k != oracle.KEY_NONE
        nrefl += int(v.sum())
        assert rrays[v].tobytes() == o_r[v].tobytes(), f"bounce {bnc} reflection rays"
        rh = ctx.frame_hits(bnc, npix)
        assert np.all(rh[~v] == oracle.HIT_NONE)
        idx = _pick(np.nonzero(v)[0], sample, rng)
        bf = cache.get(("reflection", bnc), s.positions, o_r[idx], False)
        assert np.array_equal(rh[idx], bf), f"bounce {bnc} reflection hits: {(rh[idx] != bf).sum()} differ"
        checked["reflection"] += len(idx)
        spos2, snrm2 = ctx.frame_surface(bnc, npix)
        o2p, o2n = oracle.resolve(s.positions, s.normals, s.material_ids, rrays, rh, None, npix)
        assert spos2.tobytes() == o2p.tobytes() and snrm2.tobytes() == o2n.tobytes()
        spos, snrm, prev = spos2, snrm2, rrays
    assert st["shadow_rays"] == nshadow and st["reflection_rays"] == nrefl
    if image:
        img = rgba.numpy()
        assert np.any(img & 0xFFFFFF)  # something was lit
        # the last reflection surface is shaded once more, unshadowed, then packed
        oracle.shade(spos, snrm, s.materials, None, accum, W, H, lights, eye, depth, prev, samples)
        want = oracle.pack(accum)
        diff = np.abs(img.view(np.uint8).reshape(-1, 4).astype(np.int32) - want.view(np.uint8).reshape(-1, 4))
        assert diff.max() <= 2, diff.max()
    return st, checked
