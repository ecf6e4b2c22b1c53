"""Environment light (ckr_env_light, the reference's EnvSource): the FP64 oracle's lookup
and normalisation pinned against the reference itself (oracle/_ref), its sampler
checked against the exact luminance x solid-angle distribution and against the
reference's own importance samples, and the MIS estimator checked for bias against
the exact irradiance of a plane.  No GPU."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import scene as S

COLOR = (1.0, 0.75, 0.5)  # exact in FP32, so the reference (FP64 colour) and ours agree bit for bit
INTENSITY = 2.0


def env_image(h=16, w=32, seed=1):
    rng = np.random.default_rng(seed)
    img = rng.uniform(0, 1, (h, w, 3)).astype(np.float32)
    img[3, 5] = [20, 18, 15]   # a small bright "sun"
    img[h - 2, 7] = 0.0        # a black pixel: never sampled
    return img


def env_of(img, axis=1, n_samples=0):
    sd = S.SceneData(np.zeros((0, 9)), np.zeros(0), np.zeros((0, 4)), np.zeros(0), [S.Material()], [])
    sd.set_env(img, axis=axis, color=COLOR, intensity=INTENSITY, n_samples=n_samples)
    return sd


def directions(img, n=4000, seed=2):
    """Random directions plus the awkward ones: the axes, the poles, and phi on the
    quadrant boundaries of getThetaPhi."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    special = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
               [1, 1, 0], [1, 0, 1], [0, 1, 1], [-1, 1, -1], [1e-9, 1, 1e-9], [1e-9, -1, -1e-9]]
    d = np.concatenate([d, np.array(special, float)])
    return d / np.linalg.norm(d, axis=1, keepdims=True)


need_ref = pytest.mark.skipif(not O.ref_available(), reason="reference library not built")


@need_ref
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_lookup_and_area_match_reference(axis):
    img = env_image()
    sd = env_of(img, axis)
    d = directions(img)
    ours, area = O.env_eval(sd.env, d)
    ref_rgb, ref_area, _ = O.ref_env(img.astype(np.float64), axis, COLOR, INTENSITY, d)
    # Same pixel for every direction: EnvSource::getRadiance restated exactly.
    assert np.array_equal(ours[:, :3], ref_rgb)
    # calcArea is a left Riemann sum on a 2000 x 4000 grid; ours is exact per pixel
    # band.  About the z axis the grid's nodes fall on the image's pixel boundaries
    # and the sum is off by 3e-4 (1e-6 about x and y).
    assert abs(area / ref_area - 1) < 1e-3, (area, ref_area)


def pixel_of(d, w, h, axis):
    """The pixel a direction looks up (the oracle's lookup on a unit-per-pixel image)."""
    img = np.arange(w * h, dtype=np.float32).reshape(h, w, 1).repeat(3, 2)
    sd = S.SceneData(np.zeros((0, 9)), np.zeros(0), np.zeros((0, 4)), np.zeros(0), [S.Material()], [])
    sd.set_env(img + 1, axis=axis, color=(1, 1, 1), intensity=1.0)
    v, _ = O.env_eval(sd.env, d)
    return np.rint(v[:, 0] - 1).astype(np.int64)


@pytest.mark.parametrize("axis", [0, 1])
def test_sampler_follows_luminance_times_solid_angle(axis):
    img = env_image()
    h, w = img.shape[:2]
    sd = env_of(img, axis)
    n = 400000
    u = np.random.default_rng(3).uniform(size=(n, 3))
    d = O.env_sample(sd.env, u)
    assert np.allclose(np.linalg.norm(d, axis=1), 1, atol=1e-12)
    counts = np.bincount(pixel_of(d, w, h, axis), minlength=w * h)
    rows = np.arange(h)
    band = (np.cos(np.pi * rows / h) - np.cos(np.pi * (rows + 1) / h)) * (2 * np.pi / w)
    look, area = O.env_eval(sd.env, centres(w, h, axis))
    px = look[:, 3] * np.repeat(band, w) / area
    assert abs(px.sum() - 1) < 1e-9
    assert counts[(h - 2) * w + 7] == 0  # the black pixel is never drawn
    expect = px * n
    m = expect > 20
    chi2 = np.sum((counts[m] - expect[m]) ** 2 / expect[m])
    dof = m.sum() - 1
    assert chi2 < dof + 6 * np.sqrt(2 * dof), (chi2, dof)


def centres(w, h, axis):
    """Unit directions through the centre of every pixel, row-major."""
    r, c = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    th, ph = (r.ravel() + 0.5) * np.pi / h, (c.ravel() + 0.5) * 2 * np.pi / w
    lx, ly, lz = np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)
    if axis == 0:
        return np.stack([lz, lx, ly], 1)
    if axis == 1:
        return np.stack([lx, lz, ly], 1)
    return np.stack([lx, ly, lz], 1)


@need_ref
def test_sampler_agrees_with_reference_importance_samples():
    # The reference builds its 200,000 directions in the z-up frame its densities are
    # evaluated in (initSamples), so compare with the map about z.
    img = env_image(8, 16, 4)
    h, w = img.shape[:2]
    sd = env_of(img, 2)
    _, _, ref = O.ref_env(img.astype(np.float64), 2, COLOR, INTENSITY, np.zeros((1, 3)), 200000)
    ours = O.env_sample(sd.env, np.random.default_rng(5).uniform(size=(200000, 3)))
    a = np.bincount(pixel_of(ref, w, h, 2), minlength=w * h) / len(ref)
    b = np.bincount(pixel_of(ours, w, h, 2), minlength=w * h) / len(ours)
    # Total variation between the two pixel histograms: the reference draws from
    # discretised (2000 x 3000-bin) inverse CDFs and its sample table is clock-seeded.
    assert 0.5 * np.abs(a - b).sum() < 0.03


def plane_scene(img, n_samples=10):
    """A 40 x 40 Lambertian square at y = 0 facing +y under the environment (axis y)."""
    tri = np.array([[-20, 0, -20, 20, 0, 20, 20, 0, -20], [-20, 0, -20, -20, 0, 20, 20, 0, 20]], np.float32)
    m = S.Material()
    m.brdf, m.alpha, m.spec, m.int_ior, m.ext_ior, m.reflectance = 2, 0.3, 0.0, 1.5, 1.0, 1.0
    m.color[:] = [1.0, 1.0, 1.0]
    sd = S.SceneData(tri, np.zeros(2, np.uint32), np.zeros((0, 4)), np.zeros(0), [m], [])
    sd.set_env(img, axis=1, color=COLOR, intensity=INTENSITY, n_samples=n_samples)
    cam = S.Camera()
    cam.pos[:], cam.dir[:] = [0, 5, 0.01], [0, -1, 0]
    cam.cx[:], cam.cy[:] = [0.2, 0, 0], [0, 0, 0.2]
    cam.width = cam.height = 8
    return sd, cam


def exact_plane_radiance(img):
    """Radiance of the Lambertian plane: (1/pi) x sum over the upper-hemisphere pixels
    of L x the integral of cos theta over the pixel's solid angle."""
    h, w = img.shape[:2]
    c = np.array(COLOR) / max(COLOR) * INTENSITY
    out = np.zeros(3)
    for r in range(h):
        t0, t1 = np.pi * r / h, np.pi * (r + 1) / h
        if t0 >= np.pi / 2:
            break
        t1 = min(t1, np.pi / 2)
        wcos = 0.5 * (np.sin(t1) ** 2 - np.sin(t0) ** 2) * (2 * np.pi / w)
        out += img[r].astype(np.float64).sum(0) * c * wcos
    return out / np.pi


@pytest.mark.parametrize("shader", [S.SHADER_DIRECT_MIS, S.SHADER_PATH])
def test_estimator_unbiased_on_a_plane(shader):
    img = env_image()
    sd, cam = plane_scene(img)
    cfg = S.render_cfg(shader=shader, spp=256, max_depth=2, n_light=1, n_brdf=4 if shader == S.SHADER_DIRECT_MIS else 1)
    rgb = O.render(sd, cam, cfg)
    mean = rgb.reshape(-1, 3).mean(0)
    want = exact_plane_radiance(img)
    err = rgb.reshape(-1, 3).std(0) / np.sqrt(rgb.shape[0] * rgb.shape[1])
    assert np.all(np.abs(mean - want) < 5 * err + 1e-3 * want), (mean, want, err)
