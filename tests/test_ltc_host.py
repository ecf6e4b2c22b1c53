"""CPU checks of the LTC shading path: the FP64 oracle against the reference (golden
fixture), and the FP32 per-pixel code of ckr_ltc_shade (host replay) against the oracle."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr

GOLD = Path(__file__).resolve().parent / "golden"


def materials_from_gbuffer(g):
    m = np.zeros(len(g), dtype=O.MATERIAL)
    m["brdf"] = 2  # GGX
    m["alpha"] = g[:, 3]
    m["spec"] = g[:, 11]
    f0 = g[:, 7].astype(np.float64)
    m["int_ior"] = (1 + np.sqrt(f0)) / (1 - np.sqrt(f0))
    m["ext_ior"] = 1.0
    return m


def oracle_ltc(g, lt, lc):
    return O.ltc_shade_batch(materials_from_gbuffer(g), g[:, 0:3], g[:, 4:7], g[:, 8:11], lt, lc)


def host_replay(g, lt, lc):
    f = ckr.lib().ckr_internal_ltc_shade_host
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    f.restype = C.c_int
    g = np.ascontiguousarray(g, np.float32)
    out = np.empty((len(g), 3), np.float32)
    assert f(g.ctypes.data, len(g), lt.ctypes.data, lc.ctypes.data, len(lt), out.ctypes.data) == 0
    return out


def ltc_errors(got, ref):
    """Per-pixel error relative to the pixel's own magnitude, floored at 1% of the image
    mean: pixels darker than that (emitters at grazing angles, where the polygon
    integral is a small difference of larger edge terms) are held to an absolute error
    of 1e-4 x 1% of the mean instead."""
    mag = np.maximum(np.abs(ref).max(axis=1), 1e-2 * np.abs(ref).mean())
    return np.abs(got - ref).max(axis=1) / mag


def test_oracle_matches_reference_golden():
    g = np.load(GOLD / "shading.npz")
    out = O.ltc_shade_batch(g["ltc_mat"], g["ltc_x"], g["ltc_n"], g["ltc_v"], g["ltc_tri"], g["ltc_rgb"])
    assert np.array_equal(out, g["ltc_out"])
    for k in range(len(g["mggx_in"])):
        th, al = g["mggx_in"][k]
        M, det, Mi, amp = O.m_ggx(float(th), float(al))
        assert np.array_equal(M, g["mggx_M"][k]) and det == g["mggx_det"][k]
        assert np.array_equal(Mi, g["mggx_Minv"][k]) and amp == g["mggx_amp"][k]
    b, p = O.brdf_batch(g["brdf_mat"], g["brdf_n"], g["brdf_wo_ref"], g["brdf_wo"], g["brdf_wi"])
    assert np.array_equal(b, g["brdf_out"]) and np.array_equal(p, g["brdf_pdf"])
    b, _ = O.brdf_batch(g["brdf_mat_ltc"], g["brdf_n"], g["brdf_wo_ref"], g["brdf_wo"], g["brdf_wi"], use_ltc=True)
    assert np.array_equal(b, g["brdf_out_ltc"])


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not built here")
def test_oracle_matches_live_reference():
    g = ckr.gbuffer(5, 3000)
    lt, lc = ckr.quad_lights(6, 8)
    m = materials_from_gbuffer(g)
    a = O.ltc_shade_batch(m, g[:, 0:3], g[:, 4:7], g[:, 8:11], lt, lc)
    b = O.ltc_shade_batch(m, g[:, 0:3], g[:, 4:7], g[:, 8:11], lt, lc, reference=True)
    assert np.array_equal(a, b)


@pytest.mark.slow
def test_fp32_ltc_replay_full_size():
    """All 1024^2 pixels of the benchmark G-buffer (about 8 s of CPU)."""
    g = ckr.gbuffer(2, 1024 * 1024)
    lt, lc = ckr.quad_lights(3, 8)
    err = ltc_errors(host_replay(g, lt, lc), oracle_ltc(g, lt, lc))
    assert err.max() <= 1e-4, np.sort(err)[-10:]


def test_fp32_ltc_replay_vs_oracle():
    g = ckr.gbuffer(11, 20000)
    lt, lc = ckr.quad_lights(12, 8)
    ref = oracle_ltc(g, lt, lc)
    got = host_replay(g, lt, lc)
    err = ltc_errors(got, ref)
    assert err.max() <= 1e-4, np.sort(err)[-10:]


def test_gbuffer_distributions():
    g = ckr.gbuffer(1, 50000)
    n, v = g[:, 4:7].astype(np.float64), g[:, 8:11].astype(np.float64)
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-6) and np.all(n[:, 2] >= 0)
    assert np.allclose(np.linalg.norm(v, axis=1), 1, atol=1e-6)
    c = np.sum(n * v, axis=1)
    assert np.all(c >= -1e-6)
    assert abs(np.mean(c) - 2 / 3) < 0.01  # E[cos] under a cosine lobe
    assert abs(n[:, 2].mean() - 0.5) < 0.01  # uniform hemisphere
    assert g[:, 3].min() >= 0.05 and g[:, 3].max() <= 1.0
    assert g[:, 7].min() >= 0.02 and g[:, 7].max() <= 0.9
    lt, lc = ckr.quad_lights(2, 8)
    assert lt.shape == (16, 9) and np.all(lc == 5)
    z = lt.reshape(-1, 3)[:, 2]
    assert z.min() >= 1 and z.max() <= 3


def test_theta_over_sin_polynomial():
    """The edge integral's theta / sin(theta), theta = acos(c), evaluated by the
    polynomial of theta_over_sin (host build of the device code) against FP64 on a
    dense grid of FP32 cosines, the ends and the sign change included: within 1e-6
    relative (the FP32 acos / sqrt / division it replaced were within about 3e-7)."""
    f = ckr.lib().ckr_internal_theta_over_sin_host
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
    f.restype = C.c_int
    c = np.concatenate([np.linspace(-1, 1, 400001), -1 + np.logspace(-7, -1, 2000), 1 - np.logspace(-7, -1, 2000),
                        np.logspace(-30, -1, 500), -np.logspace(-30, -1, 500), [0.0, 1.0]]).astype(np.float32)
    c = np.ascontiguousarray(c[(c > -1) & (c <= 1)])
    out = np.empty_like(c)
    assert f(c.ctypes.data, len(c), out.ctypes.data) == 0
    cd = c.astype(np.float64)
    s = np.sqrt(np.maximum((1 - cd) * (1 + cd), 0))
    exact = np.where(cd < 1, np.arccos(np.minimum(cd, 1)) / np.where(s > 0, s, 1), 1.0)
    rel = np.abs(out - exact) / exact
    assert np.all(np.isfinite(out)) and rel.max() < 1e-6, (rel.max(), c[np.argmax(rel)])
    assert out[c == 1][0] == np.float32(1.0) or abs(out[c == 1][0] - 1) < 1e-6
    assert abs(out[c == 0][0] - np.pi / 2) < 1e-6
