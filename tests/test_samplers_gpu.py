"""Chi-square tests of the renderer's device samplers (the functions the shading
kernels call), one million draws each through ckr_internal_sample_probe:

- the one-sample BRDF mixture (specular lobe with probability specularCoef, else
  cosine; getBrdfDirectionSampleRandomized, src/materialTypes.cpp:136-153) for GGX,
  Beckmann, microfacet Phong and classic Phong, with the lobe samplers of
  src/domainSampler.cpp:193-314: the histogram of directions over the sphere against
  the density written here in FP64 from the distributions' definitions
      p(w) = s p_lobe(w) + (1 - s) max(w.n, 0) / pi,
      microfacet: p_lobe = D(h) (h.n) / (4 |h.wo|), h = +-normalize(w + wo), h.n > 0,
      classic Phong: p_lobe = (e + 1) / (2 pi) max(w.wo_ref, 0)^e,
  and the device's pdf_eval (src/materialTypes.cpp:89-116) against the same density
  above the horizon;
- cosine (src/domainSampler.cpp:154-189), uniform hemisphere (:89-100) and cone
  (:320-369) against cos / pi, 1 / 2 pi and 1 / (2 pi (1 - cos_max));
- uniform points on a triangle (:138-150) over 256 equal-area sub-triangles.

Expected counts come from 8 x 8-point Gauss-Legendre quadrature over each (theta, phi)
cell; cells expecting fewer than 5 draws are pooled.  The draws are seeded, so a
pass is reproducible; the bar is p > 1e-4."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from chakumrender_gb300 import ckr
from chakumrender_gb300 import scene as S

pytestmark = pytest.mark.gpu
N = 1 << 20
NT, NP, Q = 48, 48, 8
PI = np.pi

PROBE_BRDF, PROBE_COSINE, PROBE_HEMISPHERE, PROBE_CONE, PROBE_TRIANGLE = range(5)
GGX, BECKMANN, PHONG, CLASSIC_PHONG = 2, 3, 4, 1


def probe(torch, kind, mat=None, n=(0, 0, 1), wo=(0, 0, 1), tri=None, param=0.0, seed=11):
    L = ckr.lib()
    f = L.ckr_internal_sample_probe
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_uint64, C.c_uint32,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    out = torch.empty((N, 4), dtype=torch.float32, device="cuda")
    nn = np.ascontiguousarray(n, np.float32)
    ww = np.ascontiguousarray(wo, np.float32)
    tt = np.ascontiguousarray(tri, np.float32) if tri is not None else None
    st = f(kind, C.byref(mat) if mat is not None else None, nn.ctypes.data, ww.ctypes.data,
           tt.ctypes.data if tt is not None else None, param, seed, N, out.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


def frame(n):
    n = np.asarray(n, np.float64)
    n = n / np.linalg.norm(n)
    a = np.array([1.0, 0, 0]) if abs(n[0]) < 0.9 else np.array([0, 1.0, 0])
    x = np.cross(a, n)
    x /= np.linalg.norm(x)
    return x, np.cross(n, x), n


def chi2_sphere(dirs, density, axis, cap=None):
    """Histogram of unit directions over (theta, phi) cells about `axis` against the
    integral of `density` (FP64, a function of (N, 3) unit vectors) over each cell;
    for a density uniform on the cap cos(theta) >= `cap` the cell integrals are
    exact (quadrature does not resolve the cap's edge inside a cell)."""
    from scipy.stats import chi2

    X, Y, Z = frame(axis)
    d = dirs / np.linalg.norm(dirs, axis=1, keepdims=True)
    th = np.arccos(np.clip(d @ Z, -1, 1))
    ph = np.mod(np.arctan2(d @ Y, d @ X), 2 * PI)
    it = np.minimum((th / PI * NT).astype(int), NT - 1)
    ip = np.minimum((ph / (2 * PI) * NP).astype(int), NP - 1)
    obs = np.bincount(it * NP + ip, minlength=NT * NP).astype(np.float64)
    # Gauss-Legendre nodes in every cell.
    g, w = np.polynomial.legendre.leggauss(Q)
    tt = (np.arange(NT)[:, None] + (g[None] + 1) / 2) * (PI / NT)  # NT x Q
    pp = (np.arange(NP)[:, None] + (g[None] + 1) / 2) * (2 * PI / NP)
    T = tt[:, None, :, None]
    P = pp[None, :, None, :]
    st, ct = np.sin(T), np.cos(T)
    vec = (st * np.cos(P))[..., None] * X + (st * np.sin(P))[..., None] * Y + np.broadcast_to(ct, st.shape)[..., None] * Z
    vec = np.broadcast_to(vec, (NT, NP, Q, Q, 3))
    dens = density(vec.reshape(-1, 3)).reshape(NT, NP, Q, Q)
    wts = (w[:, None] * w[None, :]) * (PI / NT / 2) * (2 * PI / NP / 2)
    exp = (dens * np.broadcast_to(st, (NT, NP, Q, Q)) * wts).sum((2, 3)).ravel() * len(dirs)
    if cap is not None:
        c0 = np.cos(np.arange(NT) * PI / NT)
        c1 = np.cos((np.arange(NT) + 1) * PI / NT)
        band = np.maximum(c0 - np.maximum(c1, cap), 0.0) / (1.0 - cap) / NP  # share of the cap per cell
        exp = np.repeat(band, NP) * len(dirs)
    assert abs(exp.sum() / len(dirs) - 1) < 2e-3, exp.sum() / len(dirs)  # the density integrates to 1
    big = exp >= 5
    o = np.append(obs[big], obs[~big].sum())
    e = np.append(exp[big], exp[~big].sum())
    if e[-1] < 5:
        o, e = o[:-1], e[:-1]
    stat = float(((o - e) ** 2 / e).sum())
    return float(chi2.sf(stat, len(e) - 1)), stat, len(e)


def d_ggx(a, ct):
    ct2 = ct * ct
    t2 = (1 - ct2) / ct2
    return a * a / (PI * ct2 * ct2 * (a * a + t2) ** 2)


def d_beckmann(a, ct):
    ct2 = ct * ct
    t2 = (1 - ct2) / ct2
    return np.exp(-t2 / (a * a)) / (PI * a * a * ct2 * ct2)


def d_phong(e, ct):
    return (e + 2) / (2 * PI) * ct ** e


def brdf_density(brdf, alpha, exp_c, spec, n, wo):
    n = np.asarray(n, np.float64)
    wo = np.asarray(wo, np.float64)
    wref = 2 * (n @ wo) * n - wo

    def dens(w):
        diff = (1 - spec) * np.maximum(w @ n, 0) / PI
        if brdf == CLASSIC_PHONG:
            lobe = (exp_c + 1) / (2 * PI) * np.maximum(w @ wref, 0) ** exp_c
        else:
            h = w + wo
            hn = np.linalg.norm(h, axis=1, keepdims=True)
            h = h / np.where(hn > 0, hn, 1)
            h *= np.where(h @ n < 0, -1.0, 1.0)[:, None]
            ct = np.clip(h @ n, 1e-12, 1)
            D = {GGX: d_ggx, BECKMANN: d_beckmann, PHONG: d_phong}[brdf](alpha, ct)
            lobe = D * ct / (4 * np.maximum(np.abs(h @ wo), 1e-12))
        return spec * lobe + diff

    return dens


def material(brdf, alpha, phong_exp, spec):
    m = S.Material()
    m.brdf, m.alpha, m.phong_exp, m.spec, m.int_ior, m.ext_ior, m.reflectance = brdf, alpha, phong_exp, spec, 1.5, 1.0, 1
    return m


N0 = np.array([0.2, -0.3, 0.9])
N0 /= np.linalg.norm(N0)
X0, Y0, _ = frame(N0)
WO = np.cos(np.radians(40)) * N0 + np.sin(np.radians(40)) * X0  # 40 degrees off the normal


@pytest.mark.parametrize("brdf,alpha,exp_c,spec", [(GGX, 0.3, 0, 1.0), (GGX, 0.7, 0, 0.5), (BECKMANN, 0.25, 0, 1.0),
                                                   (BECKMANN, 0.6, 0, 0.5), (PHONG, 20.0, 0, 1.0),
                                                   (CLASSIC_PHONG, 0, 16.0, 1.0), (CLASSIC_PHONG, 0, 8.0, 0.5)])
def test_brdf_sampler_chi2(torch_cuda, brdf, alpha, exp_c, spec):
    out = probe(torch_cuda, PROBE_BRDF, material(brdf, alpha, exp_c, spec), N0, WO)
    dens = brdf_density(brdf, alpha, exp_c, spec, N0, WO)
    p, stat, dof = chi2_sphere(out[:, :3], dens, N0)
    assert p > 1e-4, (p, stat, dof)
    # pdf_eval on the device against the FP64 density, above the horizon.
    d = out[:, :3] / np.linalg.norm(out[:, :3], axis=1, keepdims=True)
    up = (d @ N0) > 1e-3
    ref = dens(d[up])
    ok = ref > 1e-6
    rel = np.abs(out[up, 3][ok] - ref[ok]) / ref[ok]
    assert np.quantile(rel, 0.999) < 2e-3 and np.median(rel) < 1e-4, (np.median(rel), rel.max())


@pytest.mark.parametrize("kind,param", [(PROBE_COSINE, 0.0), (PROBE_HEMISPHERE, 0.0), (PROBE_CONE, 0.8),
                                        (PROBE_CONE, 0.2)])
def test_direction_sampler_chi2(torch_cuda, kind, param):
    out = probe(torch_cuda, kind, None, N0, WO, param=param)
    if kind == PROBE_COSINE:
        dens = lambda w: np.maximum(w @ N0, 0) / PI  # noqa: E731
    elif kind == PROBE_HEMISPHERE:
        dens = lambda w: np.where(w @ N0 >= 0, 1 / (2 * PI), 0.0)  # noqa: E731
    else:
        dens = lambda w: np.where(w @ N0 >= param, 1 / (2 * PI * (1 - param)), 0.0)  # noqa: E731
    cap = None if kind == PROBE_COSINE else (0.0 if kind == PROBE_HEMISPHERE else param)
    p, stat, dof = chi2_sphere(out[:, :3], dens, N0, cap=cap)
    assert p > 1e-4, (p, stat, dof)
    d = out[:, :3] / np.linalg.norm(out[:, :3], axis=1, keepdims=True)
    inside = np.ones(len(d), bool) if cap is None else (d @ N0) > cap + 1e-5
    assert np.allclose(out[inside, 3], dens(d[inside]), rtol=1e-5, atol=1e-6)


def test_triangle_points_are_uniform(torch_cuda):
    from scipy.stats import chi2

    tri = np.array([0.3, -1.0, 2.0, 2.5, 0.1, 1.0, -0.7, 1.4, 0.6])
    out = probe(torch_cuda, PROBE_TRIANGLE, None, tri=tri)
    A, B, Cc = tri.reshape(3, 3)
    M = np.stack([B - A, Cc - A], 1)
    b12, *_ = np.linalg.lstsq(M, (out[:, :3] - A).T, rcond=None)
    b1, b2 = b12
    assert np.all(b1 > -1e-5) and np.all(b2 > -1e-5) and np.all(b1 + b2 < 1 + 1e-5)
    K = 16  # 256 congruent sub-triangles of equal area
    i = np.clip((K * b1).astype(int), 0, K - 1)
    j = np.clip((K * b2).astype(int), 0, K - 1)
    upper = (K * b1 - i) + (K * b2 - j) > 1
    cell = (i * K + j) * 2 + upper
    valid = np.zeros(K * K * 2, bool)
    for a in range(K):
        for b in range(K):
            valid[(a * K + b) * 2] = a + b <= K - 1
            valid[(a * K + b) * 2 + 1] = a + b <= K - 2
    obs = np.bincount(cell, minlength=K * K * 2)
    assert obs[~valid].sum() <= 4  # points a rounding away from the diagonal
    o = obs[valid].astype(float)
    e = np.full(len(o), N / len(o))
    stat = float(((o - e) ** 2 / e).sum())
    p = float(chi2.sf(stat, len(o) - 1))
    assert len(o) == 256 and p > 1e-4, (p, stat)
