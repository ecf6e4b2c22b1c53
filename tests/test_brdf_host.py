"""CPU check of the renderer's FP32 BRDF and pdf (host replay of shading_device.cuh)
against the FP64 oracle, which is itself pinned to the reference (test_ltc_host golden).

Inputs are FP32 unit vectors; the oracle receives them renormalised in FP64, because
the reference's tan^2 = 1/cos^2 - 1 (src/materialTypes.cpp:180-239) is only accurate for
vectors normalised in FP64 (an FP32 length error of 1 ulp adds ~1e-7 to tan^2, more
than tan^2 itself near the mirror direction of a lobe with alpha ~ 5e-4)."""
from __future__ import annotations

import ctypes as C

import numpy as np

import oracle as O
from chakumrender_gb300 import ckr
from chakumrender_gb300 import scene as S


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def test_fp32_brdf_vs_oracle():
    rng = np.random.default_rng(5)
    n_ = 60000
    n, wo = unit(rng, n_), unit(rng, n_)
    wo[np.sum(wo * n, 1) < 0] *= -1
    wi = unit(rng, n_)
    wi[np.sum(wi * n, 1) < 0] *= -1
    wo_ref = 2 * np.sum(n * wo, 1, keepdims=True) * n - wo
    near = rng.random(n_) < 0.5  # half of the directions inside glossy lobes
    wi[near] = wo_ref[near] + unit(rng, n_)[near] * rng.uniform(0, 3e-3, (int(near.sum()), 1))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    keep = np.sum(wi * n, 1) > 1e-3
    n, wo, wi, wo_ref = n[keep], wo[keep], wi[keep], wo_ref[keep]
    m = len(n)
    mat = np.zeros(m, dtype=O.MATERIAL)
    mat["brdf"] = rng.integers(1, 5, m)
    mat["alpha"] = 10 ** rng.uniform(-3.3, 0, m)
    phong = mat["brdf"] == 4
    mat["alpha"][phong] = rng.uniform(1, 2000, int(phong.sum()))
    mat["phong_exp"] = rng.uniform(1, 2000, m)
    mat["spec"] = rng.uniform(0, 1, m)
    mat["int_ior"] = rng.uniform(1.1, 1e5, m)
    mat["ext_ior"] = 1
    for k in ("alpha", "phong_exp", "spec", "int_ior"):
        mat[k] = mat[k].astype(np.float32)
    f32 = [np.ascontiguousarray(a, np.float32) for a in (n, wo_ref, wo, wi)]
    renorm = [a.astype(np.float64) / np.linalg.norm(a.astype(np.float64), axis=1, keepdims=True) for a in f32]
    ob, op = O.brdf_batch(mat, *renorm)
    cm = (S.Material * m)()
    for i in range(m):
        cm[i].brdf, cm[i].alpha, cm[i].phong_exp = int(mat["brdf"][i]), mat["alpha"][i], mat["phong_exp"][i]
        cm[i].spec, cm[i].int_ior, cm[i].ext_ior = mat["spec"][i], mat["int_ior"][i], 1.0
    fn = ckr.lib().ckr_internal_brdf_host
    fn.argtypes = [C.c_void_p, C.c_uint32] + [C.c_void_p] * 6
    fn.restype = C.c_int
    gb, gp = np.empty(m, np.float32), np.empty(m, np.float32)
    assert fn(C.addressof(cm), m, *[a.ctypes.data for a in f32], gb.ctypes.data, gp.ctypes.data) == 0
    for g, o in ((gb, ob), (gp, op)):
        rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-6)
        assert np.quantile(rel, 0.999) <= 1e-3, np.quantile(rel, [0.99, 0.999, 1])
        assert rel.max() <= 3e-2
