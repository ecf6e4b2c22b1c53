"""The Monte Carlo reference of the LTC integral (ckr_ltc_mc): the FP64 oracle's own
correctness on CPU, then the GPU kernel against the oracle on the same random streams,
and the LTC shading against the MC reference at the full 1024^2 G-buffer.

Known answer: with spec = 0 the material is Lambertian and the LTC diffuse term is the
exact polygon form factor, so LTC and MC must agree to within the MC's own noise."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr


def rel_mse(a, b, eps=1e-2):
    return float(np.mean((a - b) ** 2 / (b * b + eps)))


def materials(g, spec=None, fresnel=False):
    m = np.zeros(len(g), dtype=O.MATERIAL)
    m["brdf"] = 2
    m["alpha"] = g[:, 3]
    m["spec"] = g[:, 11] if spec is None else spec
    f0 = np.sqrt(g[:, 7].astype(np.float64))
    m["int_ior"] = (1 + f0) / (1 - f0) if fresnel else 1e5
    m["ext_ior"] = 1
    return m


def oracle_mc(g, lt, lc, spp, seed, spec=None, fresnel=False, pixel_index=None):
    return O.ltc_mc(materials(g, spec, fresnel), g[:, 0:3], g[:, 4:7], g[:, 8:11], lt, lc, spp, seed,
                    pixel_index=pixel_index)


def oracle_ltc(g, lt, lc, spec=None):
    return O.ltc_shade_batch(materials(g, spec), g[:, 0:3], g[:, 4:7], g[:, 8:11], lt, lc)


def test_oracle_mc_known_answer_lambertian():
    g = ckr.gbuffer(11, 1024)
    lt, lc = ckr.quad_lights(5)
    ltc = oracle_ltc(g, lt, lc, spec=0.0)
    mc, mc2 = oracle_mc(g, lt, lc, 4096, 1, spec=0.0), oracle_mc(g, lt, lc, 4096, 2, spec=0.0)
    noise = rel_mse(mc2, mc)  # twice one estimate's variance
    assert noise < 2e-3
    # The expected value of rel_mse(ltc, mc) is half of `noise` when LTC is exact.
    assert rel_mse(ltc, mc) < 0.8 * noise
    assert abs(mc.mean() - ltc.mean()) < 2e-3 * ltc.mean()


def test_oracle_mc_glossy_converges():
    """The glossy integrand: two independent estimates agree to their variance, and
    the LTC fit stays within a few percent of it (the fit's own error)."""
    g = ckr.gbuffer(12, 1024)
    lt, lc = ckr.quad_lights(6)
    mc, mc2 = oracle_mc(g, lt, lc, 4096, 1), oracle_mc(g, lt, lc, 4096, 2)
    assert rel_mse(mc2, mc) < 2e-3
    assert rel_mse(oracle_ltc(g, lt, lc), mc) < 2e-2
    assert abs(mc.mean() - mc2.mean()) < 5e-3 * mc.mean()


def gpu_mc(torch, g, lt, lc, spp, seed, fresnel=False):
    dg = torch.from_numpy(np.ascontiguousarray(g, np.float32)).cuda()
    dt = torch.from_numpy(np.ascontiguousarray(lt, np.float32)).cuda()
    dc = torch.from_numpy(np.ascontiguousarray(lc, np.float32)).cuda()
    out = torch.empty((len(g), 3), dtype=torch.float64, device="cuda")
    ckr.ltc_mc(dg.data_ptr(), len(g), dt.data_ptr(), dc.data_ptr(), len(lt), spp, seed, fresnel, out.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    return out.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("fresnel", [False, True])
def test_gpu_mc_vs_oracle(torch_cuda, fresnel):
    """Same streams: FP32 per-sample arithmetic against FP64.  A sample whose direction
    grazes an emitter edge may flip between hit and miss; each carries 1/spp of the
    pixel, so the bar is a small relMSE, not bit equality."""
    g = ckr.gbuffer(21, 4096)
    lt, lc = ckr.quad_lights(22)
    got = gpu_mc(torch_cuda, g, lt, lc, 1024, 9, fresnel)
    ref = oracle_mc(g, lt, lc, 1024, 9, fresnel=fresnel)
    e = rel_mse(got, ref)
    print(f"fresnel={fresnel}: relMSE GPU MC vs oracle MC {e:.3e}")
    assert np.all(np.isfinite(got)) and got.min() >= 0
    assert e <= 1e-5


@pytest.mark.gpu
def test_full_size_ltc_vs_mc(torch_cuda):
    """1024^2 G-buffer, 8 quads, 4096 spp: the LTC diffuse term equals the MC to within
    the MC's noise; the full LTC is reported against the MC (its fit error)."""
    from test_ltc_gpu import shade_gpu

    g = ckr.gbuffer(2, 1024 * 1024)
    lt, lc = ckr.quad_lights(3, 8)
    gd = g.copy()
    gd[:, 11] = 0.0  # spec = 0: Lambertian
    mc_a, mc_b = gpu_mc(torch_cuda, gd, lt, lc, 4096, 1), gpu_mc(torch_cuda, gd, lt, lc, 4096, 2)
    noise = rel_mse(mc_b, mc_a)
    ltc_d = shade_gpu(torch_cuda, gd, lt, lc).astype(np.float64)
    e = rel_mse(ltc_d, mc_a)
    print(f"Lambertian: relMSE LTC vs MC {e:.3e}, MC seed-to-seed {noise:.3e}")
    assert e < 0.8 * noise
    mc = gpu_mc(torch_cuda, g, lt, lc, 4096, 1)
    ltc = shade_gpu(torch_cuda, g, lt, lc).astype(np.float64)
    e_full = rel_mse(ltc, mc)
    print(f"GGX (F = 1): relMSE LTC vs MC {e_full:.3e}")
    assert np.all(np.isfinite(mc)) and e_full < 2e-2
