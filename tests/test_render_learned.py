"""Rendering with the learned light-selection proposal (ckr_render_learned): the
estimator stays unbiased while the network trains (it converges to the image of the
power-selection renderer), and a trained network lowers the error at equal samples
against that renderer, the method without it."""
from __future__ import annotations

import numpy as np
import pytest

from chakumrender_gb300 import scene as S
from scene_io import rel_mse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(torch_cuda):
    sd = S.manylight_scene(S.manylight_spec(subdiv=4, width=96, height=54, nemit=1024, nclusters=64))
    return torch_cuda, sd, S.RenderScene(sd)


def render(torch, scene, sd, spp, seed, prop=None):
    cam = sd.camera
    out = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device="cuda")
    cfg = S.render_cfg(shader=S.SHADER_PATH_NEE, spp=spp, max_depth=4, seed=seed)
    if prop is None:
        scene.render(cam, cfg, out.data_ptr())
    else:
        prop.render(cam, cfg, out.data_ptr())
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


def test_learned_render_is_unbiased(small):
    from chakumrender_gb300.proposal import Proposal

    torch, sd, scene = small
    prop = Proposal(scene, seed=5, minibatch=4096)
    a = render(torch, scene, sd, 2048, 1, prop)  # training from scratch while it renders
    b = render(torch, scene, sd, 2048, 2)
    st, steps, loss = prop.status()
    assert st == 0 and steps > 100
    diff = (a - b).ravel()
    z = diff.mean() / np.sqrt(diff.var() / diff.size)
    print(f"learned vs power selection: means {a.mean():.5f} {b.mean():.5f}, z {z:.2f}, steps {steps}, loss {loss:.3f}")
    assert np.all(np.isfinite(a)) and abs(z) < 4.0


def test_trained_network_lowers_error(small):
    from chakumrender_gb300.proposal import Proposal

    torch, sd, scene = small
    ref = render(torch, scene, sd, 16384, 100)
    prop = Proposal(scene, seed=6, minibatch=4096)
    for k in range(4):
        render(torch, scene, sd, 256, 10 + k, prop)
    prop.set_training(False)
    learned = np.mean([rel_mse(render(torch, scene, sd, 128, 20 + k, prop), ref) for k in range(4)])
    plain = np.mean([rel_mse(render(torch, scene, sd, 128, 20 + k), ref) for k in range(4)])
    print(f"relMSE at 128 spp: learned {learned:.4f}, power selection {plain:.4f}, ratio {plain / learned:.2f}")
    assert learned < 0.8 * plain
