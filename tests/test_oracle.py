"""CPU checks of the oracle itself: against the committed golden vectors, against independent numpy
restatements of the hash / compression / sort / decompression semantics, the hierarchy path against
its own brute force (conservativeness of the sphere/cone culling), and the object tree's shape: the
properties the GPU's single-ray descent encodes in 32-bit stack entries (at most 8 children a node, fewer
than 2^24 nodes) and relies on (child ranges partition each level, spheres enclose their vertices). The GPU
builds the same tree bit for bit (test_gpu_stages.py::test_object_hierarchy_bitexact). Last, the watertight
triangle test (Woop, Benthin & Wald 2013) lets no ray through a shared edge or vertex, including rays with
zero direction components."""
import numpy as np
import pytest

import oracle
from rsh import scenes

GOLDEN = np.load(__import__("pathlib").Path(__file__).with_name("golden") / "cornell_32.npz")


def test_golden_vectors_reproduce():
    import importlib.util
    from pathlib import Path

    spec = importlib.util.spec_from_file_location("mg", Path(__file__).with_name("golden") / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    got = mg.compute()
    for k in GOLDEN.files:
        assert np.array_equal(np.asarray(got[k]), GOLDEN[k]), k


# ---------------------------------------------------------------- independent numpy restatements
def _spread(v, stride, bits):
    r = np.zeros_like(v, dtype=np.uint32)
    for i in range(bits):
        r |= ((v >> np.uint32(i)) & np.uint32(1)) << np.uint32(stride * i)
    return r


def np_hash(rays, lo, scale, g, b, tag=0):
    f32 = np.float32
    o = rays["o"].astype(f32)
    d = rays["d"].astype(f32)
    gmax = f32((1 << g) - 1)
    f = (o - lo.astype(f32)) * scale.astype(f32)
    f = np.fmin(np.fmax(f, f32(0)), gmax)
    c = f.astype(np.uint32)
    cell = (_spread(c[:, 0], 3, 10) << np.uint32(2)) | (_spread(c[:, 1], 3, 10) << np.uint32(1)) | _spread(c[:, 2], 3, 10)
    s = (np.abs(d[:, 0]) + np.abs(d[:, 1])) + np.abs(d[:, 2])
    px = d[:, 0] / s
    py = d[:, 1] / s
    neg = d[:, 2] < 0
    qx = f32(1) - np.abs(py)
    qy = f32(1) - np.abs(px)
    px2 = np.where(px >= 0, qx, -qx)
    py2 = np.where(py >= 0, qy, -qy)
    px = np.where(neg, px2, px)
    py = np.where(neg, py2, py)
    B = 1 << b
    half = f32(0.5) * f32(B)
    bmax = f32(B - 1)
    u = np.fmin(np.fmax((px + f32(1)) * half, f32(0)), bmax).astype(np.uint32)
    v = np.fmin(np.fmax((py + f32(1)) * half, f32(0)), bmax).astype(np.uint32)
    dirb = (_spread(u, 2, 16) << np.uint32(1)) | _spread(v, 2, 16)
    key = (np.uint32(tag) << np.uint32(3 * g + 2 * b)) | (cell << np.uint32(2 * b)) | dirb
    valid = rays["tmax"] > rays["tmin"]
    return np.where(valid, key, np.uint32(0xFFFFFFFF)).astype(np.uint32)


@pytest.mark.parametrize("g,b", [(5, 4), (3, 6), (8, 2), (1, 1)])
def test_hash_matches_numpy_restatement(g, b):
    rng = np.random.default_rng(g * 7 + b)
    n = 50_000
    rays = np.zeros(n, oracle.RAY_DTYPE)
    rays["o"] = rng.uniform(-3, 3, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:6] = [[1, 0, 0], [0, -1, 0], [0, 0, -1], [0, 0, 1], [-0.6, 0, -0.8], [0.6, -0.8, 0]]
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = 0.01
    rays["tmax"] = np.inf
    rays["tmax"][7] = -1
    lo = np.array([-2, -2, -2], np.float32)
    hi = np.array([2, 2, 2], np.float32)
    scale = oracle.hash_scale(lo, hi, g)
    assert np.array_equal(scale, np.float32(1 << g) / (hi - lo))
    assert np.array_equal(oracle.hash_rays(rays, lo, scale, g, b, 0), np_hash(rays, lo, scale, g, b, 0))
    assert np.array_equal(oracle.hash_rays(rays, lo, scale, g, b, 1), np_hash(rays, lo, scale, g, b, 1))


def test_compress_sort_decompress_match_numpy():
    rng = np.random.default_rng(1)
    keys = np.repeat(rng.integers(0, 1000, 5000).astype(np.uint32), rng.integers(1, 9, 5000))
    keys[rng.random(len(keys)) < 0.3] = 0xFFFFFFFF
    tr, ck, cb, cs = oracle.compress(keys)
    valid = np.nonzero(keys != 0xFFFFFFFF)[0]
    assert np.array_equal(tr, valid)
    tk = keys[valid]
    heads = np.concatenate([[True], tk[1:] != tk[:-1]])
    assert np.array_equal(ck, tk[heads])
    assert np.array_equal(cb[:-1], np.nonzero(heads)[0])
    assert cb[-1] == len(tr)
    assert np.array_equal(cs, np.diff(cb))
    sk, sv = oracle.sort_pairs(ck, None, 10)
    order = np.argsort(ck, kind="stable")
    assert np.array_equal(sv, order) and np.array_equal(sk, ck[order])
    dk, di = oracle.decompress(sk, sv, cb, tr)
    # decompressed order == stable sort of the trimmed rays by key
    o2 = np.argsort(tk, kind="stable")
    assert np.array_equal(di, tr[o2])
    assert np.array_equal(dk, tk[o2])


def _np_pipeline(keys):
    valid = np.nonzero(keys != 0xFFFFFFFF)[0]
    tk = keys[valid]
    heads = np.concatenate([[True], tk[1:] != tk[:-1]]) if len(tk) else np.zeros(0, bool)
    return valid, tk, heads


@pytest.mark.parametrize("case", ["empty", "all_invalid", "one", "all_equal", "full_32_bit", "alternating"])
def test_compress_sort_decompress_edge_cases(case):
    rng = np.random.default_rng(7)
    keys = {
        "empty": np.zeros(0, np.uint32),
        "all_invalid": np.full(77, 0xFFFFFFFF, np.uint32),
        "one": np.array([12345], np.uint32),
        "all_equal": np.full(5000, 3, np.uint32),
        "full_32_bit": rng.integers(0, 0xFFFFFFFF, 20000, dtype=np.uint64).astype(np.uint32),
        "alternating": np.tile(np.array([1, 2], np.uint32), 3000),
    }[case]
    valid, tk, heads = _np_pipeline(keys)
    tr, ck, cb, cs = oracle.compress(keys)
    assert np.array_equal(tr, valid) and np.array_equal(ck, tk[heads])
    assert np.array_equal(cb, np.append(np.nonzero(heads)[0], len(tk))) and np.array_equal(cs, np.diff(cb))
    sk, sv = oracle.sort_pairs(ck, None, 32)
    order = np.argsort(ck, kind="stable")
    assert np.array_equal(sv, order) and np.array_equal(sk, ck[order])
    dk, di = oracle.decompress(sk, sv, cb, tr)
    o2 = np.argsort(tk, kind="stable")
    assert np.array_equal(di, valid[o2]) and np.array_equal(dk, tk[o2])


def test_hierarchy_path_equals_brute_force_cornell(cornell):
    s = cornell
    W = H = 48
    cam = np.array([0, 0, 3.4, 0, 0, -3.4, 2 * 3.4 * np.tan(np.radians(30)), 0, 0, 0,
                    2 * 3.4 * np.tan(np.radians(30)), 0], np.float32)
    rays, pix = oracle.raygen_primary(cam, W, H)
    lo = s.positions[..., :3].reshape(-1, 3).min(0)
    hi = s.positions[..., :3].reshape(-1, 3).max(0)
    oh = oracle.ObjH(s.positions, 8, lo, hi)
    nodes, _ = oracle.build_rsh(rays, None, len(rays), 8)
    cand, _ = oh.traverse(nodes, len(rays), 8)
    got = oh.intersect(rays, None, len(rays), 8, cand, False, len(rays))
    bf = oracle.brute(s.positions, rays, False)
    assert np.array_equal(got, bf)
    spos, snrm = oracle.resolve(s.positions, s.normals, s.material_ids, rays, bf, pix, W * H)
    scale = oracle.hash_scale(lo, hi, 5)
    for jitter in (0.0, 1.0):
        rr, rk = oracle.raygen_reflect(spos, snrm, None, cam[:3], W, H, 0.01, jitter, 3, 0, lo, scale, 5, 4)
        res, R, _, _ = oh.trace_keyed(rr, rk, 23, 8, False)
        v = rk != oracle.KEY_NONE
        assert np.array_equal(res[v], oracle.brute(s.positions, rr[v], False))
    sr, sk = oracle.raygen_shadow(spos, snrm, W, H, np.array([[0, 0.95, 0]], np.float32), 0.01, lo, scale, 5, 4)
    res, R, _, _ = oh.trace_keyed(sr, sk, 23, 8, True)
    v = sk != oracle.KEY_NONE
    assert R == int(v.sum()) > 0
    assert np.array_equal(res[v], oracle.brute(s.positions, sr[v], True))


@pytest.mark.parametrize("P", [8, 16, 32])
def test_hierarchy_path_equals_brute_force_soup(P):
    s = scenes.random_soup(8000, np.random.default_rng(4))
    rays = scenes.surface_rays(s, 6000, np.random.default_rng(5))
    lo = s.positions[..., :3].reshape(-1, 3).min(0)
    hi = s.positions[..., :3].reshape(-1, 3).max(0)
    oh = oracle.ObjH(s.positions, 8, lo, hi)
    keys = oracle.hash_rays(rays, lo, oracle.hash_scale(lo, hi, 5), 5, 4)
    res, R, _, ctr = oh.trace_keyed(rays, keys, 23, P, False)
    assert np.array_equal(res, oracle.brute(s.positions, rays, False))
    assert ctr[1] < len(rays) * s.tri_count  # the hierarchy culls
    rays["tmax"] = 2.0
    res, R, _, _ = oh.trace_keyed(rays, keys, 23, P, True)
    assert np.array_equal(res, oracle.brute(s.positions, rays, True))


# ---------------------------------------------------------------- object-tree shape
def _tree_checks(positions, cluster):
    pos = np.asarray(positions, np.float32).reshape(-1, 12)
    pts = pos.reshape(-1, 4)[:, :3]
    lo, hi = pts.min(0), pts.max(0)
    oh = oracle.ObjH(pos, cluster, lo, hi)
    sizes, kids = oh.levels(), oh.kids()
    order, tris, sph = oh.arrays()
    levels, T = len(sizes), oh.T
    off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    # the virtual root's children fit one node step; fewer than 2^24 nodes in all
    assert sizes[-1] <= 8 and sum(sizes) < (1 << 24)
    # child ranges partition the level below: clusters of 1..cluster triangles, nodes of 1..8 children
    for l in range(levels):
        k = kids[l].astype(np.int64)
        below = T if l == 0 else sizes[l - 1]
        cnt = np.diff(k)
        assert k[0] == 0 and k[-1] == below and cnt.min() >= 1
        assert cnt.max() <= (cluster if l == 0 else 8), (l, int(cnt.max()))
    # every sphere encloses every vertex of its triangle range (the cull never drops a real hit)
    tstart = kids[0].astype(np.int64)
    v = tris.reshape(-1, 3, 4)[:, :, :3].astype(np.float64)
    for l in range(levels):
        if l > 0:
            tstart = tstart[kids[l].astype(np.int64)]
        s = sph[off[l]:off[l] + sizes[l]].astype(np.float64)
        owner = np.repeat(np.arange(sizes[l]), np.diff(tstart))
        d = np.sqrt(((v - s[owner, None, :3]) ** 2).sum(-1)).max(-1)
        assert (d <= s[owner, 3]).all(), l
    # a depth-first walk by (level, first child, count) entries -- the single-ray descent's stack --
    # reaches every cluster and every triangle exactly once
    seen = np.zeros(T, np.int32)
    stack = [(levels, int(off[-1]), sizes[-1])]
    while stack:
        L, first, cnt = stack.pop()
        for c in range(first, first + cnt):
            if L == 1:
                seen[kids[0][c]:kids[0][c + 1]] += 1
            else:
                j = c - off[L - 1]
                stack.append((L - 1, int(off[L - 2] + kids[L - 1][j]), int(kids[L - 1][j + 1] - kids[L - 1][j])))
    assert (seen == 1).all()
    assert np.array_equal(np.sort(order), np.arange(T))


@pytest.mark.parametrize("cluster", [6, 32])
def test_object_tree_shape_cornell(cluster):
    _tree_checks(scenes.cornell().positions, cluster)


@pytest.mark.parametrize("cluster", [1, 6])
def test_object_tree_shape_soup(cluster):
    _tree_checks(scenes.random_soup(20000, np.random.default_rng(9)).positions, cluster)


# ---------------------------------------------------------------- watertight intersection
def _rays(o, d):
    r = np.zeros(len(o), oracle.RAY_DTYPE)
    r["o"], r["d"], r["tmin"], r["tmax"] = o, d, 0.0, np.inf
    return r


def test_watertight_grid_edges_and_vertices():
    """A flat grid of 2 x 16 x 16 triangles in z = 0, hit straight down (zero x and y direction components)
    and obliquely exactly on its shared edges (axis-aligned and diagonal) and vertices: a watertight test
    lets no such ray through, and every hit lies at the plane's distance."""
    N = 16
    ij = np.stack(np.meshgrid(np.arange(N + 1), np.arange(N + 1), indexing="ij"), -1).reshape(-1, 2)
    verts = np.concatenate([ij.astype(np.float32), np.zeros((len(ij), 1), np.float32)], 1)
    vid = lambda i, j: i * (N + 1) + j
    faces = []
    for i in range(N):
        for j in range(N):
            faces += [(vid(i, j), vid(i + 1, j), vid(i + 1, j + 1)), (vid(i, j), vid(i + 1, j + 1), vid(i, j + 1))]
    pos, _ = scenes._pack(verts, np.array(faces))
    g = np.arange(1, N, dtype=np.float32)
    h = np.arange(N, dtype=np.float32) + np.float32(0.5)
    pts = np.concatenate([
        np.stack(np.meshgrid(g, h, indexing="ij"), -1).reshape(-1, 2),   # edges along y
        np.stack(np.meshgrid(h, g, indexing="ij"), -1).reshape(-1, 2),   # edges along x
        np.stack([h, h], -1),                                             # diagonals (cell centres)
        np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2),   # inner vertices
    ]).astype(np.float32)
    targets = np.concatenate([pts, np.zeros((len(pts), 1), np.float32)], 1)
    for d in (np.array([0, 0, -1], np.float32), np.array([0.3, -0.2, -1], np.float32)):
        d = (d / np.linalg.norm(d)).astype(np.float32)
        o = (targets - 4.0 * d).astype(np.float32)
        hits = oracle.brute(pos, _rays(o, np.repeat(d[None], len(o), 0)), False)
        assert np.all(hits != oracle.HIT_NONE), "a ray through an edge or vertex slipped through the grid"
        t = (hits >> np.uint64(32)).astype(np.uint32).view(np.float32)
        assert np.allclose(t, 4.0, rtol=1e-5)
        occl = oracle.brute(pos, _rays(o, np.repeat(d[None], len(o), 0)), True)
        assert np.all(occl != 0)


def test_watertight_closed_mesh():
    """Rays from outside at every edge midpoint and vertex of a closed icosphere all hit it."""
    sv, sf = scenes.icosphere(2)
    pos, _ = scenes._pack(sv, sf, sv)
    edges = np.concatenate([sf[:, [0, 1]], sf[:, [1, 2]], sf[:, [2, 0]]])
    targets = np.concatenate([(sv[edges[:, 0]] + sv[edges[:, 1]]) * 0.5, sv]).astype(np.float32)
    o = (targets * 3.0 + np.random.default_rng(2).normal(0, 0.2, targets.shape)).astype(np.float32)
    d = targets - o
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    hits = oracle.brute(pos, _rays(o, d), False)
    assert np.all(hits != oracle.HIT_NONE)


def test_blocked_brute_force_equals_scalar_loop():
    """oracle.brute (sign prefilter over a structure-of-arrays copy, then the exact test on the survivors)
    gives exactly the scalar loop's results: closest-hit records and shadow flags, for rays from inside and
    outside the scene, rays with zero direction components (the double-precision fallback) and short
    intervals."""
    s = scenes.soup(n_spheres=60, width=8, height=8, extent=6.0)
    rng = np.random.default_rng(11)
    n = 3000
    r = np.zeros(n, oracle.RAY_DTYPE)
    r["o"] = rng.uniform(-8, 8, (n, 3))
    d = rng.normal(size=(n, 3))
    d[: n // 4, rng.integers(0, 3)] = 0.0          # zero components
    d[n // 4: n // 3] = np.eye(3)[rng.integers(0, 3, n // 3 - n // 4)]  # axis-aligned
    r["d"] = d / np.linalg.norm(d, axis=1)[:, None]
    r["tmin"] = 0.0
    r["tmax"] = np.where(rng.random(n) < 0.5, np.inf, rng.uniform(0.1, 10.0, n))
    r["tmax"][:7] = -1.0                           # empty slots
    for any_hit in (False, True):
        a = oracle.brute(s.positions, r, any_hit)
        b = oracle.brute(s.positions, r, any_hit, scalar=True)
        assert np.array_equal(a, b)
        assert (a != (0 if any_hit else oracle.HIT_NONE)).sum() > n // 10


@pytest.mark.parametrize("cluster", [3, 6])
def test_box_descent_equals_brute_force(cluster):
    """The oracle's restatement of the batched form's traversal (per-ray descent of the single-ray box tree,
    fused.cu k_fused_rays) gives exactly the brute-force records and flags, including rays with zero
    direction components and short intervals; its work counts are sums of per-ray counts. The box tree
    partitions the triangles into clusters of at most `cluster`, every node has 1 to 8 children in
    consecutive slots, and every box contains what is below it."""
    s = scenes.soup(n_spheres=120, width=8, height=8, extent=10.0)
    lo = s.positions[..., :3].reshape(-1, 3).min(0)
    hi = s.positions[..., :3].reshape(-1, 3).max(0)
    oh = oracle.ObjH(s.positions, cluster, lo, hi)
    rng = np.random.default_rng(5)
    n = 4000
    r = np.zeros(n, oracle.RAY_DTYPE)
    r["o"] = rng.uniform(-12, 12, (n, 3))
    d = rng.normal(size=(n, 3))
    d[: n // 5, rng.integers(0, 3)] = 0.0
    r["d"] = d / np.linalg.norm(d, axis=1)[:, None]
    r["tmin"] = 0.01
    r["tmax"] = np.where(rng.random(n) < 0.5, np.inf, rng.uniform(0.5, 15.0, n))
    for any_hit in (False, True):
        got, (nt, tt), per = oh.trace_box(r, any_hit, per_ray=True)
        assert np.array_equal(got, oracle.brute(s.positions, r, any_hit))
        assert per[:, 0].sum() == nt and per[:, 1].sum() == tt and tt > 0
    root, wb, wt = oh.box_tree()
    w = wb.view(np.uint32)
    is_cl = (w[:, 7] >> 31) == 1
    cnt = w[is_cl, 7] & 0x7FFFFFFF
    covered = np.sort(np.concatenate([np.arange(a, a + c) for a, c in zip(w[is_cl, 3], cnt)]))
    assert np.array_equal(covered, np.arange(s.tri_count)) and cnt.max() <= cluster
    assert np.array_equal(np.sort(wt[:, 3].view(np.uint32)), np.arange(s.tri_count))  # original ids
    seen = np.zeros(len(wb), bool)
    stack = [(root, None)]
    while stack:
        e, parent = stack.pop()
        n, f = ((e >> 24) & 7) + 1, e & 0xFFFFFF
        assert e >> 27 == 1 and 1 <= n <= 8 and f + n <= len(wb)
        for c in range(f, f + n):
            assert not seen[c]
            seen[c] = True
            if parent is not None:
                assert np.all(wb[c, :3] >= wb[parent, :3]) and np.all(wb[c, 4:7] <= wb[parent, 4:7])
            if not is_cl[c]:
                stack.append((int(w[c, 3]), c))
            else:
                tv = wt[w[c, 3]:w[c, 3] + (w[c, 7] & 0x7FFFFFFF)].reshape(-1, 3, 4)[:, :, :3].reshape(-1, 3)
                assert np.all(tv >= wb[c, :3]) and np.all(tv <= wb[c, 4:7])
    assert seen[1:].all()
    # the level tree's boxes contain their triangles and carry the child links
    bx = oh.boxes()
    levels = oh.levels()
    order, tris, _ = oh.arrays()
    c0 = bx[: levels[0]]
    first = c0[:, 3].view(np.uint32)
    cnt = c0[:, 7].view(np.uint32)
    assert first[0] == 0 and np.all(first[1:] == first[:-1] + cnt[:-1]) and cnt.sum() == s.tri_count
    # a node's link is its stack entry: level, child count and first child (absolute index)
    off = np.concatenate([[0], np.cumsum(levels)])
    for l in range(1, len(levels)):
        e = bx[off[l]:off[l + 1], 3].view(np.uint32)
        n = bx[off[l]:off[l + 1], 7].view(np.uint32)
        assert np.all(e >> 27 == l) and np.all(((e >> 24) & 7) + 1 == n) and np.all((n >= 1) & (n <= 8))
        f = e & 0xFFFFFF
        assert f[0] == off[l - 1] and np.all(f[1:] == f[:-1] + n[:-1]) and f[-1] + n[-1] == off[l]
    v = tris.reshape(-1, 3, 4)[:, :, :3]
    for j in range(0, levels[0], 97):
        tv = v[first[j]:first[j] + cnt[j]].reshape(-1, 3)
        assert np.all(tv >= c0[j, :3]) and np.all(tv <= c0[j, 4:7])
