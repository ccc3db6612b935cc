"""Generates tests/golden/cornell_32.npz: small known-answer vectors of every pipeline stage.

The reference cannot run here (CUDA 6.5 / texture references / Win32 + GL) and ships no golden vectors
for this path, so these vectors come from the CPU oracle on a 32x32 frame of the Cornell-style scene.
They pin the oracle (and, through the GPU tests, the kernels) against regressions; they do not pin
parity with the reference's own outputs. Re-run after an intentional change:
    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "ray-tracer_gb300")]

import oracle  # noqa: E402
from rsh import scenes  # noqa: E402

W = H = 32
G, B, P, K = 5, 4, 8, 8
EPS = 0.01


def camera(s):
    eye = np.array(s.eye, np.float64)
    tgt = np.array(s.target, np.float64)
    up = np.array(s.up, np.float64)
    d = tgt - eye
    dist = np.linalg.norm(d)
    f = d / dist
    hh = 2 * dist * np.tan(np.radians(s.fov / 2))
    hw = hh * W / H
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    u /= np.linalg.norm(u)
    return np.concatenate([eye, f * dist, r * hw, u * hh]).astype(np.float32)


def compute():
    s = scenes.cornell()
    lo = s.positions[..., :3].reshape(-1, 3).min(0)
    hi = s.positions[..., :3].reshape(-1, 3).max(0)
    cam = camera(s)
    prays, pix = oracle.raygen_primary(cam, W, H)
    phits = oracle.brute(s.positions, prays, False)
    spos, snrm = oracle.resolve(s.positions, s.normals, s.material_ids, prays, phits, pix, W * H)
    scale = oracle.hash_scale(lo, hi, G)
    lp = np.array([l["position"] for l in s.lights], np.float32)
    srays, skeys = oracle.raygen_shadow(spos, snrm, W, H, lp, EPS, lo, scale, G, B)
    rrays, rkeys = oracle.raygen_reflect(spos, snrm, None, cam[:3], W, H, EPS, 0.0, 1, 0, lo, scale, G, B)
    tr, ck, cb, cs = oracle.compress(rkeys)
    sk, sv = oracle.sort_pairs(ck, None, 3 * G + 2 * B)
    dk, di = oracle.decompress(sk, sv, cb, tr)
    nodes, off = oracle.build_rsh(rrays, di, len(di), P, max_rays=W * H)
    oh = oracle.ObjH(s.positions, K, lo, hi)
    order, tris, sph = oh.arrays()
    kids = np.concatenate(oh.kids())
    cand, _ = oh.traverse(nodes, len(di), P, max_rays=W * H)
    rhits = oh.intersect(rrays, di, len(di), P, cand, False, W * H)
    valid_s = skeys != oracle.KEY_NONE
    sflags = oracle.brute(s.positions, srays, True) * valid_s
    return dict(cam=cam, prays=prays.view(np.uint8), pix=pix, phits=phits, spos=spos, snrm=snrm, skeys=skeys,
                srays=srays.view(np.uint8), sflags=sflags.astype(np.uint32), rkeys=rkeys, rrays=rrays.view(np.uint8),
                trimmed=tr, ckeys=ck, cbases=cb, csizes=cs, skeys_sorted=sk, svals_sorted=sv, dec_keys=dk,
                dec_ids=di, nodes=nodes.view(np.uint8), node_off=off, order=order, sph=sph, kids=kids, cand=cand,
                rhits=rhits)


if __name__ == "__main__":
    out = Path(__file__).with_name("cornell_32.npz")
    np.savez_compressed(out, **compute())
    print("wrote", out, out.stat().st_size, "bytes")
