"""ckr_render_noalloc: rendering without device allocation, for callers that cannot call
cudaMalloc while they render (renderers embedded in a host that owns all device memory,
frame loops that cannot take an allocation's synchronisation).  Its output must equal
ckr_render's on the same scene, camera and streams, on two calls in a row (the second
call reuses the static arena the first one left behind).

This file sorts last so that a run stopping at the first failure has run everything
else first."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from chakumrender_gb300 import scene as S

pytestmark = pytest.mark.gpu


def noalloc(scene, cam, cfg, torch):
    L = S._setup()
    f = L.ckr_render_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    out = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device="cuda")
    st = f(scene.handle, C.byref(cam), C.byref(cfg), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return st, out.cpu().numpy()


@pytest.mark.parametrize("shader,spp,nl,nb,depth", [(S.SHADER_PATH, 16, 1, 1, 4),
                                                    (S.SHADER_DIRECT_MISCV, 2, 10, 60, 1),
                                                    (S.SHADER_DIRECT_MIS, 2, 10, 60, 1),
                                                    (S.SHADER_EXPLICIT, 2, 10, 60, 4)])
def test_noalloc_matches_render(torch_cuda, shader, spp, nl, nb, depth):
    sd = S.load_xml(S.SCENES / "box.xml")
    cam = sd.camera
    cfg = S.render_cfg(shader=shader, spp=spp, n_light=nl, n_brdf=nb, max_depth=depth)
    scene = S.RenderScene(sd)
    ref = scene.render_host(cam, cfg)
    for _ in range(2):
        st, img = noalloc(scene, cam, cfg, torch_cuda)
        assert st == 0
        assert scene.check_device(torch_cuda.cuda.current_stream().cuda_stream) == 0
        # The same tolerance as the renderer's determinism test: FP64 sums in another
        # order may change the last FP32 bit.
        assert np.allclose(img, ref, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("shader", [S.SHADER_PATH, S.SHADER_PATH_NEE])
def test_regenerating_render_matches_waves(torch_cuda, shader):
    """A path-tracer render of more than one wave of paths on a tree of three or more
    levels (here 4,194,304 paths against 2^21 slots, a 5,120-triangle icosphere in the
    many-light room with 64 emitters in 4 clusters) starts a new camera path in the slot
    of every path that ends; the same paths rendered in fixed waves of 32,768
    (ckr_render_noalloc) give the same image."""
    sd = S.manylight_scene(S.manylight_spec(subdiv=4, width=512, height=512, nemit=64, nclusters=4))
    cam = sd.camera
    cfg = S.render_cfg(shader=shader, spp=16, n_light=1, n_brdf=1, max_depth=5)
    scene = S.RenderScene(sd)
    assert scene.info().max_depth >= 3  # deep enough for regeneration
    ref = scene.render_host(cam, cfg)
    st, img = noalloc(scene, cam, cfg, torch_cuda)
    assert st == 0
    assert np.all(np.isfinite(ref)) and ref.mean() > 0
    assert np.allclose(img, ref, rtol=1e-6, atol=1e-7)


def test_noalloc_rejects_oversized_images(torch_cuda):
    sd = S.load_xml(S.SCENES / "box.xml")
    cam = sd.camera
    cam.width, cam.height = 1024, 512  # 524288 pixels > 262144
    scene = S.RenderScene(sd)
    L = S._setup()
    L.ckr_render_noalloc.argtypes = [C.c_void_p] * 5
    L.ckr_render_noalloc.restype = C.c_int
    out = torch_cuda.empty(16, dtype=torch_cuda.float32, device="cuda")
    st = L.ckr_render_noalloc(scene.handle, C.byref(cam), C.byref(S.render_cfg()), out.data_ptr(), None)
    assert st == -10  # CKR_ERR_TOO_LARGE
