"""GPU renderer (ckr_render, wavefront) against the FP64 oracle on the same scenes,
cameras and per-pixel random streams, and against the reference binary's images."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import scene as S
from scene_io import block_agreement, from_arrays, rel_mse, srgb8

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
BOX = S.SCENES / "box.xml"

# (shader, spp, n_light, n_brdf, max_depth, relMSE bar vs the FP64 oracle).  Both
# sides consume the same random numbers; differences come from FP32 arithmetic, the
# FP32 ray offsets and the rare paths that FP32/FP64 send to different primitives.
CASES = [
    (S.SHADER_DIRECT_MISCV, 4, 10, 60, 1, 1e-4),
    (S.SHADER_DIRECT_MIS, 4, 10, 60, 1, 1e-4),
    (S.SHADER_PATH, 16, 1, 1, 4, 1e-3),
    (S.SHADER_DIRECT_CV, 4, 25, 0, 1, 1e-4),
    (S.SHADER_EXPLICIT, 4, 10, 60, 4, 1e-3),
]


def gpu_render(torch, sd, cam, cfg):
    scene = S.RenderScene(sd)
    img = scene.render_host(cam, cfg)
    assert scene.check_device() == 0
    return img.astype(np.float64)


@pytest.mark.parametrize("shader,spp,nl,nb,depth,bar", CASES)
def test_box_vs_oracle(torch_cuda, shader, spp, nl, nb, depth, bar):
    sd = S.load_xml(BOX)
    cfg = S.render_cfg(shader=shader, spp=spp, n_light=nl, n_brdf=nb, max_depth=depth)
    g = gpu_render(torch_cuda, sd, sd.camera, cfg)
    o = O.render(sd, sd.camera, cfg)
    # The control-variate estimator may dip below zero per pixel (V f - f_ltc < 0).
    assert np.all(np.isfinite(g)) and (g.min() >= 0 or shader == S.SHADER_DIRECT_CV)
    e = rel_mse(g, o)
    print(f"shader {shader}: relMSE vs oracle {e:.3e}, mean {g.mean():.5f} vs {o.mean():.5f}")
    assert e <= bar
    assert abs(g.mean() - o.mean()) <= 1e-3 * o.mean() + 1e-6


@pytest.mark.parametrize("name,shader", [("scene0", S.SHADER_DIRECT_MISCV), ("scene1", S.SHADER_DIRECT_MIS),
                                         ("scene0", S.SHADER_DIRECT_CV)])
def test_reference_scenes_vs_oracle(torch_cuda, name, shader):
    sd = from_arrays(np.load(GOLD / "ref_scenes.npz"), name)
    cfg = S.render_cfg(shader=shader, spp=1, n_light=25 if shader == S.SHADER_DIRECT_CV else 10, n_brdf=60)
    g = gpu_render(torch_cuda, sd, sd.camera, cfg)
    o = O.render(sd, sd.camera, cfg)
    e = rel_mse(g, o)
    print(f"{name}: relMSE vs oracle {e:.3e}")
    # FP32 against FP64 with the same random streams: the images agree sample by
    # sample, so the bar is far below 1-spp noise (measured 1.3e-7 and 2.8e-5).
    # scene0's tilted plates have normals with an exactly zero x component, which
    # picks ref_frame's second branch; a fused cross product would leave a residue
    # there, rotate every BRDF sample's frame and cost relMSE ~1.
    assert e <= 1e-4
    mean, p99 = block_agreement(g, srgb8(o).astype(np.uint8))
    assert mean <= 0.01 and p99 <= 0.1, (mean, p99)


@pytest.mark.parametrize("name", ["box", "scene0"])
def test_default_shader_vs_reference_image(torch_cuda, name):
    ref8 = np.load(GOLD / "ref_images.npz")[name]
    sd = S.load_xml(BOX) if name == "box" else from_arrays(np.load(GOLD / "ref_scenes.npz"), "scene0")
    g = gpu_render(torch_cuda, sd, sd.camera, S.render_cfg(shader=S.SHADER_DIRECT_MISCV, spp=1, n_light=10, n_brdf=60))
    mean, p99 = block_agreement(g, ref8)
    assert mean <= 0.01 and p99 <= 0.1, (mean, p99)


def test_render_determinism_and_device_api(torch_cuda):
    torch = torch_cuda
    sd = S.load_xml(BOX)
    cam = sd.camera
    cfg = S.render_cfg(shader=S.SHADER_PATH, spp=8, max_depth=4)
    scene = S.RenderScene(sd)
    a = scene.render_host(cam, cfg)
    rgb = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device="cuda")
    acc = torch.empty((cam.height, cam.width, 3), dtype=torch.float64, device="cuda")
    scene.render(cam, cfg, rgb.data_ptr(), acc.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    b = rgb.cpu().numpy()
    # FP64 atomics in a different order can change the last FP32 bit at most.
    assert np.allclose(a, b, rtol=1e-6, atol=1e-7)
    assert np.allclose(acc.cpu().numpy() / cfg.spp, b, rtol=1e-6, atol=1e-7)
    # Different seeds give different noise, same mean.
    cfg2 = S.render_cfg(shader=S.SHADER_PATH, spp=8, max_depth=4, seed=2)
    c = scene.render_host(cam, cfg2)
    assert not np.array_equal(a, c) and abs(a.mean() - c.mean()) < 0.02 * a.mean()
