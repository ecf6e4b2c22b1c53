"""The reference's same-named C++ host API over the C ABI (include/ckr_dropin.hpp),
run as compiled C++ programs on the GPU:

- INTEGRATION.md section 1a's main() (the reference's main() structure: set-up calls,
  camera rays, a batched shade(), P3 output) renders chakumrender_gb300/scenes/box.xml
  to the image ckr_render_host gives with the same shader and seed;
- section 1b's main() (the C ABI directly) gives that image too;
- per-ray BvhAccel::intersectT / intersectS and shadow(), called one ray at a time
  from OpenMP threads as the reference calls them, agree with the FP64 oracle (ids
  bit-exact up to ties and boundary rays) and with the C ABI's any-hit query; the
  batched intersect equals the per-ray one; per-ray shade() is deterministic and
  agrees in the mean with the batched shade()."""
from __future__ import annotations

import ctypes as C
import subprocess

import numpy as np
import pytest

import dropin_build as D
import oracle as O
from chakumrender_gb300 import ckr
from chakumrender_gb300 import scene as S
from parity import classify

pytestmark = pytest.mark.gpu
BOX = S.SCENES / "box.xml"


@pytest.fixture(scope="module")
def programs(tmp_path_factory):
    return D.build_all(tmp_path_factory.mktemp("dropin"))


def reference_image():
    sd = S.load_xml(BOX)
    cfg = S.render_cfg(shader=S.SHADER_DIRECT_MISCV, spp=1, max_depth=1, n_light=10, n_brdf=60, seed=1)
    return S.RenderScene(sd).render_host(sd.camera, cfg)


@pytest.mark.parametrize("name", ["dropin_main", "cabi_main"])
def test_integration_main_renders_the_box(torch_cuda, programs, name, tmp_path):
    r = subprocess.run([str(programs[name]), str(BOX)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    img = D.read_pfm(tmp_path / "image.pfm")
    ref = reference_image()
    assert img.shape == ref.shape
    assert (tmp_path / "image.ppm").read_bytes().startswith(b"P3\n256 256\n255\n")
    if name == "cabi_main":
        # The same calls as reference_image(): equal up to the order of FP64 sums.
        assert np.allclose(img, ref, rtol=1e-5, atol=1e-6)
    else:
        # Camera rays computed on the host in FP64 (as src/main.cpp:77 does) instead of
        # on the device in FP32: directions differ in the last bits, so a pixel's shading
        # point moves by ~1e-7 and silhouette pixels may see another primitive.
        rel = np.abs(img - ref) / (np.abs(ref) + 1e-3)
        assert np.mean(rel.max(2) < 1e-3) > 0.995, np.mean(rel.max(2) < 1e-3)
        rel_mse = float(np.mean((img - ref) ** 2 / (ref * ref + 1e-2)))
        assert rel_mse < 1e-4, rel_mse


def test_per_ray_queries_match_oracle_and_batched(torch_cuda, programs, tmp_path):
    sd = S.load_xml(BOX)
    cam = sd.camera
    # Camera rays of a 64 x 64 crop (FP64 directions as the reference's main() forms
    # them) and rays from inside the box in uniform directions.
    rng = np.random.default_rng(5)
    pos, d0 = np.array(cam.pos, float), np.array(cam.dir, float)
    cx, cy = np.array(cam.cx, float), np.array(cam.cy, float)
    ys, xs = np.mgrid[96:160, 96:160]
    d = (cx[None] * (((xs.ravel() + 0.34) / cam.width) - .5)[:, None]
         + cy[None] * (((ys.ravel() + 0.20) / cam.height) - .5)[:, None] + d0[None])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.repeat(pos[None], len(d), 0)
    o2 = rng.uniform(0.05, 0.95, (2048, 3))
    d2 = rng.normal(size=(2048, 3))
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    o, d = np.concatenate([o, o2]), np.concatenate([d, d2])
    dist = rng.uniform(0.1, 2.0, len(o))
    n = len(o)
    inp = np.concatenate([o, d, dist[:, None]], 1)
    (tmp_path / "rays.bin").write_bytes(np.uint32(n).tobytes() + inp.astype("<f8").tobytes())
    r = subprocess.run([str(programs["queries"]), str(BOX), str(tmp_path / "rays.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rec = np.dtype([("idT", "<i4"), ("tT", "<f8"), ("N", "<f8", 3), ("idS", "<i4"), ("tS", "<f8"),
                    ("shadow", "<f8"), ("shade", "<f8", 3)])
    raw = (tmp_path / "out.bin").read_bytes()
    out = np.frombuffer(raw[: n * rec.itemsize], dtype=rec)
    id_batched = np.frombuffer(raw[n * rec.itemsize:], dtype="<i4")
    assert np.array_equal(id_batched, out["idT"])

    # Rays as the library sees them (FP32), against the FP64 oracle.
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = o, d, 1e30
    tri = np.ascontiguousarray(sd.tri9, np.float32).reshape(-1, 9)
    oid, ot = O.OracleBvh(tri).closest(rays)
    gid = np.where(out["idT"] < 0, 0xFFFFFFFF, out["idT"].astype(np.int64)).astype(np.uint32)
    c = classify(tri, rays, gid, out["tT"].astype(np.float32), oid, ot)
    assert not c["bad"] and c["edge"] + c["tie"] <= 8, c
    hit = out["idT"] >= 0
    v = tri[out["idT"][hit]].reshape(-1, 3, 3).astype(np.float64)
    nrm = np.cross(v[:, 2] - v[:, 0], v[:, 1] - v[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm *= np.where(np.sum(nrm * d[hit], 1) > 0, -1.0, 1.0)[:, None]
    assert np.allclose(out["N"][hit], nrm, atol=1e-12)

    sph = np.ascontiguousarray(sd.sph4, np.float32).reshape(-1, 4)
    sid, st = O.spheres_closest(sph, rays)
    got_s = np.where(out["idS"] < 0, 0xFFFFFFFF, out["idS"].astype(np.int64)).astype(np.uint64)
    assert np.array_equal(got_s, sid.astype(np.uint64))
    hs = out["idS"] >= 0
    assert np.allclose(out["tS"][hs], st[hs], rtol=1e-5)

    # shadow(): the any-hit query over the whole scene up to dist - 1e-5.
    scene = S.RenderScene(sd)
    srays = rays.copy()
    srays[:, 7] = (dist - 1e-5).astype(np.float32)
    occ = scene.trace_any_host(srays)
    assert np.array_equal(out["shadow"] == 0.0, occ.astype(bool))
    assert 0.05 < occ.mean() < 0.95

    # Per-ray shade() (a stream per ray) against the batched shade() (the stream of
    # pixel i): two independent estimates of the same radiance over the crop.
    cfg = S.render_cfg(shader=S.SHADER_DIRECT_MISCV, spp=1, max_depth=1, n_light=10, n_brdf=60, seed=1)
    cam_rays = rays[:4096].copy()
    cam_rays[:, 7] = 3.0e38
    batched = np.zeros((4096, 3), np.float32)
    L = ckr.lib()
    L.ckr_shade_rays_host.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    ckr.check(L.ckr_shade_rays_host(scene.handle, cam_rays.ctypes.data, 4096, C.byref(cfg), batched.ctypes.data,
                                    None), "ckr_shade_rays_host")
    per_ray = out["shade"][:4096]
    m1, m2 = per_ray.mean(0), batched.astype(np.float64).mean(0)
    assert np.all(np.abs(m1 - m2) <= 0.02 * np.abs(m2) + 1e-4), (m1, m2)
    assert np.all(np.isfinite(per_ray)) and per_ray.mean() > 0
