"""Batched rendering (ckr_batch_*): jobs of uneven resolution, spp, depth and
materials packed into one pass (the persistent renderer: one launch whose lanes
run whole paths; or the wavefront renderer: waves of paths) and replayed from a
captured CUDA graph.  Each job's image equals the single render of that job (same
random streams), replays are repeatable, the per-job sequential mode agrees, and the
autotuner reports what it chose."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from chakumrender_gb300 import scene as S
from chakumrender_gb300.batch import BatchTuning, Job, box_jobs


def test_abi_struct_sizes():
    assert C.sizeof(Job) == 88 and C.sizeof(BatchTuning) == 20


def test_box_jobs_workload():
    sd = S.load_xml(S.SCENES / "box.xml")
    params, mats = box_jobs(sd, njobs=64, seed=4)
    assert len(params) == 64 and len(mats) == 64 * sd.nmat
    assert {p["cam"].width for p in params} <= {256, 512, 768, 1024}
    assert {p["spp"] for p in params} <= {4, 16, 64} and {p["max_depth"] for p in params} <= {3, 6}
    brdfs = {mats[j * sd.nmat + 10].brdf for j in range(64)}
    assert brdfs == {2, 3, 4}


def small_jobs(torch, sd, n=6):
    params, mats = box_jobs(sd, njobs=n, seed=9, sizes=(48, 64, 80), spps=(2, 4), depths=(3, 6))
    outs, jobs = [], []
    for p in params:
        out = torch.zeros((p["cam"].height, p["cam"].width, 3), dtype=torch.float32, device="cuda")
        outs.append(out)
        jobs.append(Job(p["cam"], p["spp"], p["max_depth"], p["seed"], p["material_set"], 0, out.data_ptr()))
    return params, mats, jobs, outs


@pytest.mark.gpu
@pytest.mark.parametrize("shader", [S.SHADER_PATH, S.SHADER_PATH_NEE])
@pytest.mark.parametrize("mode", ["autotune", "persistent", "wavefront"])
def test_batch_matches_single_renders(torch_cuda, shader, mode):
    from chakumrender_gb300.batch import Batch

    torch = torch_cuda
    sd = S.load_xml(S.SCENES / "box.xml")
    params, mats, jobs, outs = small_jobs(torch, sd)
    scene = S.RenderScene(sd)
    tuning = {"autotune": None, "persistent": BatchTuning(128, 128 * 152 * 4, 0.0, 0, 1),
              "wavefront": BatchTuning(128, 1 << 17, 0.0, 0, 0)}[mode]
    b = Batch(scene, jobs, materials=mats, shader=shader, tuning=tuning)
    t = b.tuning()
    assert t.block in (64, 128, 256) and t.wave >= 128 and t.mode in (0, 1)
    if mode == "autotune":
        assert t.candidates > 0 and t.ms > 0
    else:
        assert t.mode == tuning.mode
    paths, launches = b.stats()
    assert paths == sum(p["cam"].width * p["cam"].height * p["spp"] for p in params) and launches > 0
    if t.mode == 1:
        assert launches == 2  # the persistent launch and the resolve
    b.render()
    torch.cuda.synchronize()
    first = [o.cpu().numpy() for o in outs]
    b.render()  # a second replay of the graph
    torch.cuda.synchronize()
    for a, o in zip(first, outs):
        assert np.allclose(a, o.cpu().numpy(), rtol=1e-6, atol=1e-7)
    b.render_sequential()
    torch.cuda.synchronize()
    for a, o in zip(first, outs):
        assert np.allclose(a, o.cpu().numpy(), rtol=1e-6, atol=1e-7)
    # Against the single-render entry point on a scene with the job's materials.
    for j, p in enumerate(params):
        d = S.SceneData(sd.tri9, sd.tri_mat, sd.sph4, sd.sph_mat,
                        [S.Material.from_buffer_copy(mats[j * sd.nmat + k]) for k in range(sd.nmat)],
                        [sd.lights[k] for k in range(sd.nlights)])
        cfg = S.render_cfg(shader=shader, spp=p["spp"], max_depth=p["max_depth"], n_light=1, n_brdf=1,
                           rr_prob=0.3, seed=p["seed"])
        ref = S.RenderScene(d).render_host(p["cam"], cfg)
        assert np.all(np.isfinite(first[j])) and first[j].mean() > 0
        if t.mode == 0:
            assert np.allclose(first[j], ref, rtol=1e-6, atol=1e-7), j
        else:
            # The persistent kernel runs the same device functions compiled into
            # another kernel: a rare path may round differently in its last FP32 bit
            # and take another branch (measured: 1 pixel in 6,400, image relMSE 1e-15).
            close = np.abs(first[j] - ref).max(2) <= 1e-6 * np.maximum(1.0, np.abs(ref).max(2)) + 1e-7
            rel = float(np.mean((first[j].astype(np.float64) - ref) ** 2 / (ref.astype(np.float64) ** 2 + 1e-2)))
            assert close.mean() >= 0.999 and rel <= 1e-10, (j, close.mean(), rel)


@pytest.mark.gpu
def test_autotuner_under_scarce_memory(torch_cuda):
    """With device memory too scarce for the larger wave workspaces (simulated by a
    test cap on the workspace size) the autotuner keeps the best candidate that fits,
    and the batch still equals the single renders; with room for no candidate at all,
    creation fails with CKR_ERR_OUT_OF_MEMORY.  Eight light samples per vertex (n_light
    8) rule out the persistent renderer, so only wavefront candidates compete."""
    from chakumrender_gb300 import ckr
    from chakumrender_gb300.batch import Batch

    torch = torch_cuda
    L = ckr.lib()
    cap = L.ckr_internal_batch_workspace_cap
    cap.argtypes = [C.c_uint64]
    cap.restype = C.c_int
    sd = S.load_xml(S.SCENES / "box.xml")
    params, mats, jobs, outs = small_jobs(torch, sd)
    scene = S.RenderScene(sd)
    per_path = 8
    try:
        assert cap((72 + 52 * per_path) * (1 << 17) + 1) == 0  # room for 2^17-path waves only
        b = Batch(scene, jobs, materials=mats, shader=S.SHADER_PATH, n_light=per_path)
        t = b.tuning()
        assert t.mode == 0 and t.wave <= (1 << 17) and t.candidates > 0
        b.render()
        torch.cuda.synchronize()
        for j, p in enumerate(params):
            d = S.SceneData(sd.tri9, sd.tri_mat, sd.sph4, sd.sph_mat,
                            [S.Material.from_buffer_copy(mats[j * sd.nmat + k]) for k in range(sd.nmat)],
                            [sd.lights[k] for k in range(sd.nlights)])
            cfg = S.render_cfg(shader=S.SHADER_PATH, spp=p["spp"], max_depth=p["max_depth"], n_light=per_path,
                               n_brdf=1, rr_prob=0.3, seed=p["seed"])
            ref = S.RenderScene(d).render_host(p["cam"], cfg)
            assert np.allclose(outs[j].cpu().numpy(), ref, rtol=1e-6, atol=1e-7), j
        del b
        assert cap(1024) == 0  # no wave fits
        with pytest.raises(ckr.CkrError) as e:
            Batch(scene, jobs, materials=mats, shader=S.SHADER_PATH, n_light=per_path)
        assert e.value.status == -3  # CKR_ERR_OUT_OF_MEMORY
    finally:
        cap(0)
