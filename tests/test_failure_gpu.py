"""Failure paths fire and leave the GPU usable, driven without a fault:

- the network kernels' bounded mbarrier wait: an inference whose first layer's MMAs
  are never issued waits on a phase nothing completes, gives up after a small poll
  limit, reports CKR_ERR_ITERATION_LIMIT through ckr_proposal_status, frees its tensor
  memory and returns; the next inference is correct;
- the shadow-queue capacity check: a render given a queue too small for its shadow
  rays drops them and reports CKR_ERR_QUEUE_OVERFLOW through the scene's status word;
  the next render is the normal image."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr
from chakumrender_gb300 import scene as S
from chakumrender_gb300.proposal import Proposal

pytestmark = pytest.mark.gpu


def test_stalled_network_wait_reports_iteration_limit(torch_cuda):
    torch = torch_cuda
    ml = S.manylight_scene(S.manylight_spec(subdiv=2, width=16, height=9, nemit=128, nclusters=64))
    prop = Proposal(S.RenderScene(ml), seed=3)
    centre, scale, nc = prop.encoding()
    rng = np.random.default_rng(1)
    rec = np.zeros((512, 12), np.float32)
    rec[:, 0:3] = rng.uniform(-4, 4, (512, 3))
    rec[:, 3] = 0.5
    rec[:, 4:7] = [0, 1, 0]
    rec[:, 8:11] = [0, 0, 1]
    params = (rng.normal(size=O.MLP_NPARAMS) * 0.15).astype(np.float32)
    prop.set_params(params)
    d_rec = torch.from_numpy(rec).cuda()
    d_p = torch.zeros((512, 64), dtype=torch.float16, device="cuda")
    L = ckr.lib()
    f = L.ckr_internal_proposal_infer_stalled
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
    f.restype = C.c_int
    assert f(prop.handle, d_rec.data_ptr(), 512, d_p.data_ptr(), 1024, None) == 0
    torch.cuda.synchronize()
    assert prop.status()[0] == -6  # CKR_ERR_ITERATION_LIMIT
    assert prop.status()[0] == 0  # the status word was read and cleared
    # The context is usable and the next inference is right.
    prop.infer(d_rec.data_ptr(), 512, d_p.data_ptr())
    torch.cuda.synchronize()
    assert prop.status()[0] == 0
    tv = 0.5 * np.abs(d_p.float().cpu().numpy() - O.mlp_forward(params.astype(np.float64), rec, centre, scale,
                                                                  nc)).sum(1)
    assert tv.max() < 2e-2, tv.max()


def test_tiny_shadow_queue_reports_overflow(torch_cuda):
    sd = S.load_xml(S.SCENES / "box.xml")
    cam = sd.camera
    cam.width = cam.height = 64
    cfg = S.render_cfg(shader=S.SHADER_DIRECT_MIS, spp=2, max_depth=1, n_light=10, n_brdf=60, seed=4)
    scene = S.RenderScene(sd)
    good = scene.render_host(cam, cfg)
    L = ckr.lib()
    L.ckr_internal_limit_shadow_queue.argtypes = [C.c_void_p, C.c_uint32]
    L.ckr_internal_limit_shadow_queue.restype = C.c_int
    assert L.ckr_internal_limit_shadow_queue(scene.handle, 64) == 0
    with pytest.raises(ckr.CkrError) as e:
        scene.render_host(cam, cfg)
    assert e.value.status == -5  # CKR_ERR_QUEUE_OVERFLOW
    again = scene.render_host(cam, cfg)
    assert np.allclose(again, good, rtol=1e-6, atol=1e-7)
