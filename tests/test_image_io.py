"""Scene and image files on the host: the Wavefront OBJ loader, binary P6 PPM read/write
(checked against the reference's own readImage / writeImage where oracle/_ref is built)
and the FP32 PFM writer.  No GPU."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr


def _write(path, text: str, newline="\n"):
    with open(path, "w", newline=newline) as f:
        f.write(text)


def test_obj_polygons_corner_forms_and_relative_indices(tmp_path):
    p = tmp_path / "m.obj"
    _write(p, """# a unit quad, a triangle with texture/normal indices, one with relative indices
mtllib none.mtl
o quad
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vn 0 0 1
g first
usemtl whatever
s off
f 1 2 3 4
f 1/1/1 2/1/1 3//1   # trailing comment
v 5 5 5
f -1 -2 -3
""", newline="\r\n")
    t = ckr.load_obj(p)
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [5, 5, 5]], np.float32)
    want = np.stack([
        np.concatenate([v[0], v[1], v[2]]),  # the quad as a fan around its first corner
        np.concatenate([v[0], v[2], v[3]]),
        np.concatenate([v[0], v[1], v[2]]),
        np.concatenate([v[4], v[3], v[2]]),  # -1 = the last vertex read so far
    ])
    assert np.array_equal(t, want)


def test_obj_round_trip_of_a_mesh(tmp_path):
    tri = ckr.icosphere(3, 0.05, 6, 1)
    verts = tri.reshape(-1, 3)
    p = tmp_path / "ico.obj"
    with open(p, "w") as f:
        for x in verts:
            f.write("v %.9g %.9g %.9g\n" % tuple(float(c) for c in x))
        for k in range(len(tri)):
            f.write("f %d %d %d\n" % (3 * k + 1, 3 * k + 2, 3 * k + 3))
    assert np.array_equal(ckr.load_obj(p), tri)  # %.9g round-trips float32 exactly


@pytest.mark.parametrize("text,code", [
    ("v 0 0 0\nv 1 0 0\nf 1 2\n", ckr.CKR_ERR_PARSE),        # fewer than three corners
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n", ckr.CKR_ERR_PARSE),  # index past the vertices
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", ckr.CKR_ERR_PARSE),  # 0 is not an index
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf -4 1 2\n", ckr.CKR_ERR_PARSE),  # relative index before the first
    ("v 0 zero 0\n", ckr.CKR_ERR_PARSE),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x\n", ckr.CKR_ERR_PARSE),
])
def test_obj_malformed(tmp_path, text, code):
    p = tmp_path / "bad.obj"
    _write(p, text)
    with pytest.raises(ckr.CkrError) as e:
        ckr.load_obj(p)
    assert e.value.status == code


def test_obj_errors_and_short_buffer(tmp_path):
    L = ckr.lib()
    n = C.c_uint32(0)
    assert L.ckr_obj_load(str(tmp_path / "missing.obj").encode(), None, 0, C.byref(n)) == ckr.CKR_ERR_IO
    assert L.ckr_obj_load(None, None, 0, C.byref(n)) == ckr.CKR_ERR_INVALID_ARGUMENT
    p = tmp_path / "two.obj"
    _write(p, "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 1\nf 1 2 3 4\n")
    buf = np.zeros((1, 9), np.float32)
    assert L.ckr_obj_load(str(p).encode(), buf.ctypes.data, 1, C.byref(n)) == ckr.CKR_ERR_TOO_LARGE
    assert n.value == 2
    empty = tmp_path / "empty.obj"
    _write(empty, "# nothing\n")
    assert ckr.load_obj(empty).shape == (0, 9)


def _image(h=5, w=7, seed=3):
    rng = np.random.default_rng(seed)
    img = rng.uniform(0, 1.2, (h, w, 3)).astype(np.float32)  # some values above 1 to clamp
    img[0, 0] = [0.0, 1.0, 254.5 / 255]
    return img


def test_p6_round_trip(tmp_path):
    img = _image()
    p = tmp_path / "a.ppm"
    ckr.write_ppm_p6(p, img)
    raw = p.read_bytes()
    assert raw.startswith(b"P6\n7 5\n255\n") and len(raw) == len(b"P6\n7 5\n255\n") + 7 * 5 * 3
    back = ckr.read_ppm_p6(p)
    want = np.floor(np.clip(img.astype(np.float64), 0, 1) * 255) / 255
    assert np.array_equal(back, want.astype(np.float32))
    # Comments after the magic line and extra text on the maxval line are accepted.
    body = raw[len(b"P6\n7 5\n255\n"):]
    (tmp_path / "c.ppm").write_bytes(b"P6\n# made by hand\n# twice\n7 5\n255   \n" + body)
    assert np.array_equal(ckr.read_ppm_p6(tmp_path / "c.ppm"), back)


@pytest.mark.parametrize("raw", [b"P3\n1 1\n255\n1 2 3\n", b"P6\n1 1\n65535\n\0\0\0\0\0\0", b"P6\n2 2\n255\n\0\0\0",
                                 b"P6\n-1 2\n255\n", b"P6"])
def test_p6_rejects(tmp_path, raw):
    p = tmp_path / "x.ppm"
    p.write_bytes(raw)
    with pytest.raises(ckr.CkrError) as e:
        ckr.read_ppm_p6(p)
    assert e.value.status == ckr.CKR_ERR_PARSE


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built")
def test_p6_matches_reference_read_and_write(tmp_path):
    L = O.ref()
    img = _image(9, 11, 5)
    # Same bytes as the reference's writeImage (which writes ./env1_cpy.ppm, with a comment line).
    rgb = np.ascontiguousarray(img.astype(np.float64))
    assert L.ref_write_image(str(tmp_path).encode(), rgb.ctypes.data, 11, 9) == 0
    ref_bytes = (tmp_path / "env1_cpy.ppm").read_bytes()
    ckr.write_ppm_p6(tmp_path / "ours.ppm", img)
    ours = (tmp_path / "ours.ppm").read_bytes()
    assert ref_bytes[-11 * 9 * 3:] == ours[-11 * 9 * 3:]
    # The reference's readImage (./env1.ppm) and ours agree on its own output.
    os.replace(tmp_path / "env1_cpy.ppm", tmp_path / "env1.ppm")
    out = np.zeros((9, 11, 3), np.float64)
    w, h = C.c_uint32(0), C.c_uint32(0)
    assert L.ref_read_image(str(tmp_path).encode(), out.ctypes.data, 99, C.byref(w), C.byref(h)) == 0
    assert (w.value, h.value) == (11, 9)
    assert np.array_equal(ckr.read_ppm_p6(tmp_path / "env1.ppm"), out.astype(np.float32))


def test_pfm(tmp_path):
    img = (np.arange(4 * 3 * 3, dtype=np.float32).reshape(4, 3, 3) - 5) * 1.5e3  # HDR and negative values kept
    p = tmp_path / "a.pfm"
    ckr.write_pfm(p, img)
    raw = p.read_bytes()
    head = b"PF\n3 4\n-1.0\n"
    assert raw.startswith(head)
    data = np.frombuffer(raw[len(head):], dtype="<f4").reshape(4, 3, 3)
    assert np.array_equal(data[::-1], img)  # rows stored bottom to top
