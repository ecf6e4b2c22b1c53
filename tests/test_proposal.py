"""The learned light-selection proposal: its tensor-core network (BF16 operands, FP32
accumulation) against the FP64 oracle of orc_mlp.c -- forward probabilities, the
backward pass's gradients, Adam steps -- and rendering with it: unbiased (it converges
to the power-selection image) and, once trained, lower error at equal samples."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import scene as S

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round to BF16 (nearest even), returned as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def emulate(params, rec, centre, scale, C):
    """The kernel's arithmetic in numpy: BF16 features, weights, biases and
    activations, wide accumulation, softmax."""
    f = bf16(O.mlp_features(rec, centre, scale))
    p = np.asarray(params, np.float64)
    W1 = bf16(p[0:6144].reshape(64, 96))
    # Biases ride in the weight operands (BF16) against a constant-1 activation.
    W2, b2 = bf16(p[6144:10240].reshape(64, 64)), bf16(p[10240:10304])
    W3, b3 = bf16(p[10304:14400].reshape(64, 64)), bf16(p[14400:14464])
    W4, b4 = bf16(p[14464:18560].reshape(64, 64)), bf16(p[18560:18624])
    h = bf16(np.maximum(f @ W1.T, 0))
    h = bf16(np.maximum(h @ W2.T + b2, 0))
    h = bf16(np.maximum(h @ W3.T + b3, 0))
    z = h @ W4.T + b4
    z[:, C:] = -np.inf
    z -= z.max(1, keepdims=True)
    e = np.exp(z)
    return e / e.sum(1, keepdims=True)


def records(rng, n, lo, hi, C, weighted=True):
    rec = np.zeros((n, 12), np.float32)
    rec[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    rec[:, 3] = rng.uniform(0.1, 0.8, n)
    for a, b in ((4, 7), (8, 11)):
        v = rng.normal(size=(n, 3))
        rec[:, a:b] = v / np.linalg.norm(v, axis=1, keepdims=True)
    rec[:, 7] = (rng.exponential(size=n) * (rng.random(n) < 0.6)) if weighted else 1.0
    rec[:, 11] = rng.integers(0, C, n).astype(np.uint32).view(np.float32)
    return rec


@pytest.fixture(scope="module")
def setup(torch_cuda):
    from chakumrender_gb300.proposal import Proposal

    sd = S.manylight_scene(S.manylight_spec(subdiv=3, width=64, height=36, nemit=512, nclusters=64))
    scene = S.RenderScene(sd)
    prop = Proposal(scene, seed=7)
    return torch_cuda, sd, scene, prop


def to_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_infer_vs_oracle(setup):
    torch, sd, scene, prop = setup
    centre, scale, C = prop.encoding()
    assert C == 64
    rng = np.random.default_rng(1)
    lo, hi = sd.tri9.reshape(-1, 3).min(0), sd.tri9.reshape(-1, 3).max(0)
    # Random weights of a realistic scale, so that the distribution is far from uniform.
    params = (rng.normal(size=O.MLP_NPARAMS) * 0.15).astype(np.float32)
    prop.set_params(params)
    n = 1000  # not a multiple of the 128-row tile
    rec = records(rng, n, lo, hi, C)
    d_rec = to_dev(torch, rec)
    d_p = torch.zeros((n, 64), dtype=torch.float16, device="cuda")
    prop.infer(d_rec.data_ptr(), n, d_p.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = d_p.float().cpu().numpy().astype(np.float64)
    assert prop.status()[0] == 0
    emu = emulate(params, rec, centre, scale, C)
    ref = O.mlp_forward(params.astype(np.float64), rec, centre, scale, C)
    tv_emu = 0.5 * np.abs(got - emu).sum(1)
    tv_ref = 0.5 * np.abs(got - ref).sum(1)
    print(f"total variation vs BF16 emulation: max {tv_emu.max():.2e}; vs FP64 oracle: mean {tv_ref.mean():.2e} "
          f"max {tv_ref.max():.2e}")
    assert np.all(np.isfinite(got)) and np.allclose(got.sum(1), 1.0, atol=2e-2)
    assert tv_emu.max() < 1e-2
    assert tv_ref.mean() < 2e-2 and tv_ref.max() < 0.1


def test_gradients_vs_oracle(setup):
    torch, sd, scene, prop = setup
    centre, scale, C = prop.encoding()
    rng = np.random.default_rng(2)
    lo, hi = sd.tri9.reshape(-1, 3).min(0), sd.tri9.reshape(-1, 3).max(0)
    params = (rng.normal(size=O.MLP_NPARAMS) * 0.15).astype(np.float32)
    prop.set_params(params)
    n = 3000
    rec = records(rng, n, lo, hi, C)
    d_rec = to_dev(torch, rec)
    loss, g = prop.gradients(d_rec.data_ptr(), n)
    loss_ref, g_ref = O.mlp_loss_grad(params.astype(np.float64), rec, centre, scale, C)
    print(f"loss GPU {loss:.5f} oracle {loss_ref:.5f}")
    assert abs(loss - loss_ref) < 2e-2 * abs(loss_ref)
    blocks = {"W1": (0, 6144), "W2": (6144, 10240), "b2": (10240, 10304), "W3": (10304, 14400),
              "b3": (14400, 14464), "W4": (14464, 18560), "b4": (18560, 18624)}
    for name, (a, b) in blocks.items():
        x, y = g[a:b].astype(np.float64), g_ref[a:b]
        cos = x @ y / (np.linalg.norm(x) * np.linalg.norm(y) + 1e-30)
        ratio = np.linalg.norm(x) / (np.linalg.norm(y) + 1e-30)
        print(f"{name}: cosine {cos:.5f} norm ratio {ratio:.4f}")
        assert cos > 0.99 and abs(ratio - 1) < 0.05, name


def test_adam_steps_follow_oracle(setup):
    """Three steps on the same batch from the same start: parameter changes agree
    with the FP64 oracle's (Adam normalises the step, so compare directions)."""
    torch, sd, scene, prop = setup
    centre, scale, C = prop.encoding()
    rng = np.random.default_rng(3)
    lo, hi = sd.tri9.reshape(-1, 3).min(0), sd.tri9.reshape(-1, 3).max(0)
    params = (rng.normal(size=O.MLP_NPARAMS) * 0.15).astype(np.float32)
    prop.set_params(params)
    n = 4096
    rec = records(rng, n, lo, hi, C)
    d_rec = to_dev(torch, rec)
    p64, m, v = params.astype(np.float64), np.zeros(O.MLP_NPARAMS), np.zeros(O.MLP_NPARAMS)
    for step in range(1, 4):
        prop.train_step(d_rec.data_ptr(), n)
        _, gr = O.mlp_loss_grad(p64, rec, centre, scale, C)
        O.mlp_adam(p64, m, v, gr, step)
    st, steps, last = prop.status()
    assert st == 0 and steps == 3
    dg = prop.params().astype(np.float64) - params
    do = p64 - params
    big = np.abs(do) > 1e-4  # parameters whose gradient is not ~0
    agree = np.mean(np.sign(dg[big]) == np.sign(do[big]))
    cos = dg @ do / (np.linalg.norm(dg) * np.linalg.norm(do))
    print(f"Adam: sign agreement {agree:.4f}, cosine {cos:.4f}, last loss {last:.4f}")
    assert agree > 0.95 and cos > 0.95


def test_training_learns_a_selection(setup):
    """Records whose contribution comes only from the cluster nearest to the
    position: the trained network puts most of its mass there."""
    torch, sd, scene, prop = setup
    centre, scale, C = prop.encoding()
    rng = np.random.default_rng(4)
    from chakumrender_gb300.proposal import Proposal

    fresh = Proposal(scene, seed=11, lr=3e-3)
    lo, hi = sd.tri9.reshape(-1, 3).min(0), sd.tri9.reshape(-1, 3).max(0)
    cent = rng.uniform(lo, hi, (C, 3))
    n = 16384
    losses = []
    for it in range(300):
        rec = records(rng, n, lo, hi, C, weighted=False)
        best = np.argmin(((rec[:, None, 0:3] - cent[None]) ** 2).sum(-1), axis=1)
        rec[:, 11] = best.astype(np.uint32).view(np.float32)
        d_rec = to_dev(torch, rec)
        fresh.train_step(d_rec.data_ptr(), n)
        if it % 50 == 0 or it == 299:
            losses.append(fresh.status()[2])
    test = records(rng, 2048, lo, hi, C, weighted=False)
    best = np.argmin(((test[:, None, 0:3] - cent[None]) ** 2).sum(-1), axis=1)
    d_t = to_dev(torch, test)
    d_p = torch.zeros((2048, 64), dtype=torch.float16, device="cuda")
    fresh.infer(d_t.data_ptr(), 2048, d_p.data_ptr())
    torch.cuda.synchronize()
    pr = d_p.float().cpu().numpy()
    mass = pr[np.arange(2048), best].mean()
    print(f"loss trajectory {losses}, mean mass on the right cluster {mass:.3f} (uniform {1 / C:.3f})")
    assert losses[-1] < 0.6 * losses[0]
    assert mass > 0.3
