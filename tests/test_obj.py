"""rsh_obj_load (OBJ + MTL scene reading, host only): records, index forms, fan triangulation, normals,
objects, materials and errors, checked on small files written here, and an exact round trip of a
generated mesh."""
import numpy as np
import pytest

import rsh

OBJ = """# two objects
mtllib scene.mtl
o floor
v 0 0 0
v 2 0 0
v 2 0 2
v 0 0 2
vn 0 1 0
usemtl grey
f 1//1 2//1 3//1 4//1
o box
v 0 1 0
v 1 1 0
v 0 1 1
vt 0.5 0.5
usemtl red
f -3/1 -2/1 -1/1
usemtl nosuch
f 5 6 7
"""

MTL = """newmtl red
Kd 0.9 0.1 0.1
Ks 0.2 0.2 0.2
Ns 12
newmtl grey
Kd 0.5 0.5 0.5
"""


def write(tmp_path, obj, mtl=None):
    (tmp_path / "scene.obj").write_text(obj)
    if mtl is not None:
        (tmp_path / "scene.mtl").write_text(mtl)
    return tmp_path / "scene.obj"


def test_records_and_materials(tmp_path):
    d = rsh.load_obj(write(tmp_path, OBJ, MTL))
    pos, nrm = d["positions"], d["normals"]
    assert pos.shape == (4, 3, 4)  # quad -> 2 triangles, then 2 triangles
    # fan of the quad: (1, 2, 3), (1, 3, 4)
    assert np.array_equal(pos[0, :, :3], [[0, 0, 0], [2, 0, 0], [2, 0, 2]])
    assert np.array_equal(pos[1, :, :3], [[0, 0, 0], [2, 0, 2], [0, 0, 2]])
    assert np.all(pos[:, :, 3] == 1.0) and np.all(nrm[:, :, 3] == 0.0)
    assert np.array_equal(nrm[0, :, :3], np.tile([0, 1, 0], (3, 1)))
    # no vn: the geometric normal e1 x e2 on every vertex
    e1, e2 = pos[2, 1, :3] - pos[2, 0, :3], pos[2, 2, :3] - pos[2, 0, :3]
    assert np.allclose(nrm[2, :, :3], np.cross(e1, e2))
    # negative indices -3..-1 are the last three vertices
    assert np.array_equal(pos[2, :, :3], [[0, 1, 0], [1, 1, 0], [0, 1, 1]])
    assert np.array_equal(pos[3], pos[2])
    # materials: 0 = default, then the MTL's in file order; unknown names -> 0
    m = d["materials"]
    assert m.shape == (3, 8)
    assert np.allclose(m[0], [0.75, 0.75, 0.75, 0.5, 0.75, 0.75, 0.75, 100.0])
    assert np.allclose(m[1], [0.9, 0.1, 0.1, 0.5, 0.2, 0.2, 0.2, 12.0])
    assert np.allclose(m[2], [0.5, 0.5, 0.5, 0.5, 0.75, 0.75, 0.75, 100.0])
    assert list(d["material_ids"]) == [2, 2, 1, 0]
    assert list(d["object_ids"]) == [0, 0, 1, 1] and d["object_count"] == 2


def test_without_mtl_every_face_gets_the_default(tmp_path):
    d = rsh.load_obj(write(tmp_path, "v 0 0 0\nv 1 0 0\nv 0 1 0\nusemtl x\nf 1 2 3\n"))
    assert d["materials"].shape == (1, 8) and list(d["material_ids"]) == [0]
    assert d["object_count"] == 1


def test_round_trip_of_a_generated_mesh(tmp_path):
    rng = np.random.default_rng(11)
    nv, nf = 500, 900
    # dyadic values: exact in decimal text and in float32, so parsing must reproduce them bit for bit
    v = (rng.integers(-4096, 4096, (nv, 3)) / 64.0).astype(np.float32)
    vn = (rng.integers(-64, 64, (nv, 3)) / 64.0).astype(np.float32)
    f = rng.integers(0, nv, (nf, 3))
    lines = [f"v {a:.6f} {b:.6f} {c:.6f}" for a, b, c in v] + [f"vn {a:.6f} {b:.6f} {c:.6f}" for a, b, c in vn]
    lines += [f"f {a + 1}//{a + 1} {b + 1}//{b + 1} {c + 1}//{c + 1}" for a, b, c in f]
    d = rsh.load_obj(write(tmp_path, "\n".join(lines) + "\n"))
    assert np.array_equal(d["positions"][:, :, :3], v[f])
    assert np.array_equal(d["normals"][:, :, :3], vn[f])
    assert np.all(d["material_ids"] == 0) and np.all(d["object_ids"] == 0)


@pytest.mark.parametrize("bad", ["v 0 0\n", "v 0 0 0\nv 1 0 0\nf 1 2\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n",
                                 "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 0\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1//2 2 3\n",
                                 "v 0 0 nan\n"])
def test_malformed_records_are_rejected(tmp_path, bad):
    with pytest.raises(rsh.RshError, match="malformed record"):
        rsh.load_obj(write(tmp_path, bad))


def test_missing_file_is_rejected(tmp_path):
    with pytest.raises(rsh.RshError, match="cannot read"):
        rsh.load_obj(tmp_path / "none.obj")
