"""Per-frame object transforms (rsh_scene_set_transforms, UpdateVertex RayTracer.cu:448-511): the moved
triangles equal the oracle's restatement bit for bit, the rebuilt bounds and object hierarchy equal the
oracle's built over the moved triangles, traced hits equal brute force over them, and identity matrices
bring back the rest pose exactly."""
import numpy as np
import pytest

import oracle
import rsh
from rsh import scenes

pytestmark = pytest.mark.gpu


def _matrices(rng, k):
    out = []
    for i in range(k):
        a = rng.uniform(0, 2 * np.pi)
        c, s = np.cos(a), np.sin(a)
        r = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
        sc = np.diag(rng.uniform(0.5, 2.0, 3)) if i == 1 else np.eye(3)  # one non-uniform scale
        m = np.eye(4)
        m[:3, :3] = r @ sc
        m[:3, 3] = rng.uniform(-5, 5, 3)
        n = np.eye(4)
        n[:3, :3] = np.linalg.inv(m[:3, :3]).T  # normal matrix: inverse transpose
        out.append((m.astype(np.float32), n.astype(np.float32)))
    return np.stack([o[0] for o in out]), np.stack([o[1] for o in out])


def test_transforms_move_the_scene_like_the_oracle():
    rng = np.random.default_rng(21)
    s = scenes.random_soup(30_000, np.random.default_rng(4))
    T = s.tri_count
    obj = (np.arange(T) * 3 // T).astype(np.uint32)  # three objects
    ctx = rsh.Context(grid_bits=5, dir_log2=4, packet_size=8, cluster_size=6)
    sc = ctx.scene(s.positions, s.normals, s.material_ids, s.materials, object_ids=obj)
    assert np.array_equal(sc.triangles(), s.positions)
    model, normal = _matrices(rng, 3)
    for nm in (normal, None):
        sc.set_transforms(model, nm)
        ctx.check_device_errors()
        pos, nrm = oracle.transform(s.positions, s.normals, obj, model, nm)
        assert sc.triangles().tobytes() == pos.tobytes()
        lo, hi = sc.bounds()
        assert np.array_equal(lo, pos[..., :3].reshape(-1, 3).min(0)) and np.array_equal(hi, pos[..., :3].reshape(-1, 3).max(0))
        oh = oracle.ObjH(pos, 6, lo, hi)
        _, _, sph = oh.arrays()
        levels = sc.levels()
        assert [len(l) for l in levels] == oh.levels()
        flat = np.concatenate([np.stack([l["c"][:, 0], l["c"][:, 1], l["c"][:, 2], l["radius"]], 1) for l in levels])
        assert flat.astype(np.float32).tobytes() == sph.tobytes()
        rays = scenes.surface_rays(scenes.SceneData(**{**s.__dict__, "positions": pos, "normals": nrm}), 20_000,
                                   np.random.default_rng(8))
        assert np.array_equal(ctx.trace(sc, rays, False), oracle.brute(pos, rays, False))
        assert np.array_equal(ctx.trace(sc, rays, True, fused=True), oracle.brute(pos, rays, True))
    # identity: the rest pose again, exactly
    sc.set_transforms(np.tile(np.eye(4, dtype=np.float32), (3, 1, 1)))
    assert np.array_equal(sc.triangles(), s.positions)
    with pytest.raises(rsh.RshError):  # fewer matrices than objects
        sc.set_transforms(model[:2])
    bad = model.copy()
    bad[0, 0, 0] = np.nan
    with pytest.raises(rsh.RshError):
        sc.set_transforms(bad)
    sc.destroy()
    ctx.destroy()
