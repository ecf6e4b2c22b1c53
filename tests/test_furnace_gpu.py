"""White furnace: a white Lambertian object (albedo 1, GGX material with
specularCoef 0 = Lambert) under a uniform environment of radiance 1 reflects
exactly radiance 1 in every direction when every bounce is followed -- energy is
conserved and the object disappears against the sky.  Checked with the path tracer
(CKR_SHADER_PATH: environment samples and BRDF samples under MIS at every vertex,
Russian roulette off, 48 bounces):

- a sphere (convex: one bounce sees only the sky);
- the displaced icosphere, whose dents see the object itself, so the paths bounce
  between surfaces before they leave.

Every pixel that sees the object must average 1 (within its standard error); pixels
that see nothing are black, as the reference's camera rays that leave the scene."""
from __future__ import annotations

import numpy as np
import pytest

from chakumrender_gb300 import ckr
from chakumrender_gb300 import scene as S

pytestmark = pytest.mark.gpu


def white_scene(tri, sph):
    m = S.Material()
    m.brdf, m.alpha, m.spec, m.int_ior, m.ext_ior, m.reflectance = 2, 0.3, 0.0, 1.5, 1.0, 1.0
    m.color[:] = [1.0, 1.0, 1.0]
    sd = S.SceneData(tri, np.zeros(len(tri), np.uint32), sph, np.zeros(len(sph), np.uint32), [m], [])
    sd.set_env(np.ones((16, 32, 3), np.float32), axis=1, color=(1.0, 1.0, 1.0), intensity=1.0, n_samples=1)
    cam = S.Camera()
    cam.pos[:], cam.dir[:] = [0, 0, 3.2], [0, 0, -1]
    cam.cx[:], cam.cy[:] = [0.8, 0, 0], [0, 0.8, 0]
    cam.width = cam.height = 64
    return sd, cam


@pytest.mark.parametrize("shape", ["sphere", "icosphere"])
def test_white_furnace(torch_cuda, shape):
    if shape == "sphere":
        sd, cam = white_scene(np.zeros((0, 9), np.float32), np.array([[0, 0, 0, 1.0]], np.float32))
    else:
        tri = ckr.icosphere(4, 0.15, 6, 5)
        sd, cam = white_scene(tri, np.zeros((0, 4), np.float32))
    scene = S.RenderScene(sd)
    cfg = S.render_cfg(shader=S.SHADER_PATH, spp=256, max_depth=48, n_light=1, n_brdf=1, rr_prob=0.0, seed=3)
    img = scene.render_host(cam, cfg).astype(np.float64)
    assert scene.check_device() == 0
    # Which pixels see the object: the same camera rays through the closest-hit query
    # (the pixel centres of the first sample, whose sub-pixel offset is (0.34, 0.20)).
    ys, xs = np.mgrid[0:cam.height, 0:cam.width]
    d = (np.array(cam.cx)[None] * (((xs.ravel() + 0.34) / cam.width) - .5)[:, None]
         + np.array(cam.cy)[None] * (((ys.ravel() + 0.20) / cam.height) - .5)[:, None] + np.array(cam.dir)[None])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((len(d), 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = cam.pos[:], d, 1e30
    ids, _ = scene.trace_closest_host(rays)
    hit = (ids != 0xFFFFFFFF).reshape(cam.height, cam.width)[::-1]  # output rows are top first
    inner = hit.copy()  # away from the silhouette, where sub-pixel offsets change what a sample sees
    for dy, dx in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        inner &= np.roll(hit, (dy, dx), (0, 1))
    v = img[inner]
    assert inner.sum() > 400
    mean = v.mean()
    print(f"{shape}: {inner.sum()} pixels, mean radiance {mean:.5f} (min {v.min():.4f}, max {v.max():.4f})")
    se = v.std() / np.sqrt(v.size)  # pixels are independent estimates of the same value
    assert abs(mean - 1.0) < 5 * se + 1e-4, (mean, se)
    assert np.all(np.abs(v - 1.0) < 6 * v.std() + 1e-3), (v.min(), v.max(), v.std())
    # The background stays black.
    assert np.all(img[~hit & np.roll(~hit, 1, 0) & np.roll(~hit, -1, 0) & np.roll(~hit, 1, 1)
                      & np.roll(~hit, -1, 1)] == 0)
