"""CPU-only checks of the C ABI boundary: the library loads, exports every entry point declared in
include/rsh.h, and its host-only entry points (configuration, hash parameters, serving request sizes,
camera, PNG) behave."""
import ctypes as C
import re
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

import rsh

HEADER = Path(__file__).resolve().parent.parent / "include" / "rsh.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(rsh_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_pipeline():
    names = declared_functions()
    for n in ["rsh_create", "rsh_render_frame", "rsh_hash", "rsh_compress", "rsh_sort_pairs", "rsh_decompress",
              "rsh_build_rsh", "rsh_traverse", "rsh_intersect_any", "rsh_intersect_closest", "rsh_batch_trace",
              "rsh_server_create", "rsh_scene_upload", "rsh_lights_set", "rsh_camera_set"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = rsh.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in rsh.h but not exported: {missing}"


def test_binding_covers_every_declared_symbol():
    missing = [n for n in declared_functions() if n not in rsh.SIGNATURES]
    assert not missing, missing


def test_struct_layouts_match_header():
    assert rsh.RAY_DTYPE.itemsize == 32
    assert rsh.NODE_DTYPE.itemsize == 48
    assert rsh.OBJNODE_DTYPE.itemsize == 32
    assert C.sizeof(rsh.HashParams) == 40
    assert C.sizeof(rsh.Light) == 32
    assert C.sizeof(rsh.Camera) == 48
    assert C.sizeof(rsh.Material) == 32


def test_config_defaults_and_validation():
    c = rsh.default_config()
    assert (c.grid_bits, c.dir_log2, c.packet_size, c.cluster_size, c.ray_level, c.plain_ray_level) == \
        (4, 6, 8, 6, 15, 4)
    assert abs(c.epsilon - 0.01) < 1e-9
    lib = rsh.load()
    out = C.c_void_p()
    bad = rsh.default_config(packet_size=12)
    assert lib.rsh_create(C.byref(bad), C.byref(out)) == rsh.RSH_ERR_INVALID
    bad = rsh.default_config(grid_bits=0)
    assert lib.rsh_create(C.byref(bad), C.byref(out)) == rsh.RSH_ERR_INVALID
    assert lib.rsh_create(None, None) == rsh.RSH_ERR_INVALID
    assert lib.rsh_destroy(None) == rsh.RSH_ERR_INVALID


def test_hash_params_host_arithmetic():
    hp = rsh.hash_params((-1, -2, 0), (1, 2, 8), 5, 4, 2)
    assert hp.key_bits == 2 + 15 + 8
    assert list(hp.scale) == [np.float32(32.0) / np.float32(2.0), np.float32(32.0) / np.float32(4.0),
                              np.float32(32.0) / np.float32(8.0)]
    flat = rsh.hash_params((0, 0, 0), (0, 1, 1), 5, 4, 0)
    assert flat.scale[0] == 0.0
    with pytest.raises(rsh.RshError):
        rsh.hash_params((0, 0, 0), (1, 1, 1), 10, 6, 0)  # 42 bits
    with pytest.raises(rsh.RshError):
        rsh.hash_params((0, 0, 0), (1, 1, 1), 0, 4, 0)


def test_server_request_bytes_cover_every_region():
    """The serving loop's per-request allocation holds ten buffers, each starting on a 256-byte boundary;
    the bytes admission reserves must cover their padded sizes for any resolution (odd ones included)."""
    lib = rsh.load()

    def padded_sum(W, H, depth, L):
        npix, np_ = W * H, ((W + 7) // 8) * ((H + 7) // 8) * 64
        sizes = [np_ * 32, np_ * 4, np_ * 8, npix * 16, npix * 16, npix * L * 32, npix * 32, npix * 32,
                 npix * 8 * depth, npix * L * 4 * depth]
        return sum((n + 255) // 256 * 256 for n in sizes)

    for W, H, depth, L in [(64, 64, 1, 1), (33, 33, 2, 3), (1, 1, 1, 1), (1921, 1079, 4, 8), (7, 513, 3, 5),
                           (255, 257, 1, 2)]:
        r = rsh.Request()
        r.width, r.height, r.depth, r.light_count = W, H, depth, L
        got = C.c_uint64()
        assert lib.rsh_server_request_bytes(C.byref(r), C.byref(got)) == rsh.RSH_OK
        assert got.value >= padded_sum(W, H, depth, L) and got.value % 4096 == 0, (W, H, depth, L)
    for W, H, depth, L in [(0, 8, 1, 1), (8, 8, 0, 1), (8, 8, 5, 1), (8, 8, 1, 0), (8, 8, 1, 9),
                           (65536, 4096, 1, 8)]:
        r = rsh.Request()
        r.width, r.height, r.depth, r.light_count = W, H, depth, L
        got = C.c_uint64()
        assert lib.rsh_server_request_bytes(C.byref(r), C.byref(got)) == rsh.RSH_ERR_INVALID, (W, H, depth, L)


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_host_stub_compiles_and_links(lang, tmp_path):
    """tests/host_stub.c, an engine-style host that renders one frame through the C ABI, compiles against
    include/rsh.h with warnings as errors, as C99 and as C++17, and links against librsh.so."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    lib = rsh.load()  # builds nothing; the library must exist
    root = HEADER.parent.parent
    std = ["-std=c99"] if lang == "c" else ["-x", "c++", "-std=c++17"]
    cmd = [cc, *std, "-Wall", "-Wextra", "-Werror", "-I", str(HEADER.parent), str(root / "tests" / "host_stub.c"),
           "-L", str(Path(lib._name).parent), "-lrsh", "-o", str(tmp_path / "host_stub")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_camera_look_at_matches_engine_camera():
    cam = rsh.camera_look_at((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 60.0, 512, 256)
    dist = 3.4
    hh = 2 * dist * np.tan(np.radians(30.0))
    assert np.allclose(cam.as_array()[3:6], [0, 0, -dist], atol=1e-6)
    assert np.allclose(np.linalg.norm(cam.as_array()[9:12]), hh, rtol=1e-6)
    assert np.allclose(np.linalg.norm(cam.as_array()[6:9]), hh * 2, rtol=1e-6)
    with pytest.raises(rsh.RshError):
        rsh.camera_look_at((0, 0, 0), (0, 0, 0), (0, 1, 0), 60.0, 8, 8)


def test_png_writer(tmp_path):
    w, h = 7, 5
    img = (np.arange(w * h, dtype=np.uint32) * 0x010203) | 0xFF000000
    p = tmp_path / "x.png"
    rsh.check(rsh.load().rsh_write_png(str(p).encode(), img.ctypes.data, w, h), "png")
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        ln = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        crc = struct.unpack(">I", data[pos + 8 + ln:pos + 12 + ln])[0]
        assert zlib.crc32(typ + body) & 0xFFFFFFFF == crc
        if typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(rows[:, 0] == 0)
    px = rows[:, 1:].reshape(h, w, 4)[::-1].reshape(-1, 4)
    want = img.view(np.uint8).reshape(-1, 4)
    assert np.array_equal(px, want)


def test_oracle_camera_and_defaults_match_the_library():
    """The CPU baseline builds its camera and configuration from the oracle alone (so that it maps no
    product code); both must equal the library's."""
    import oracle

    for eye, tgt, up, fov, W, H in (((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 60.0, 512, 256),
                                     ((-6.0, 5.0, -6.0), (78.0, 3.0, 78.0), (0, 1, 0), 60.0, 1920, 1080),
                                     ((83.9, -23.4, -78.1), (4.35, -24.35, 1.5), (0, 0.99996, 0), 60.0, 512, 512)):
        a = rsh.camera_look_at(eye, tgt, up, fov, W, H).as_array()
        b = oracle.camera_look_at(eye, tgt, up, fov, W, H)
        assert a.tobytes() == b.tobytes()
    c = rsh.default_config()
    for k, v in oracle.DEFAULTS.items():
        assert getattr(c, k) == pytest.approx(v), k
